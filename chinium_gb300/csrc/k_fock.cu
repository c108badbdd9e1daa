// FP64 V_xc assembly (plain path).  For grid block b and spin s, with
// L = [phi, d_x phi, d_y phi, d_z phi] and R = [A, B_x, B_y, B_z],
//   A(g, nu)   = c0(g) phi(g, nu) + sum_r c1_r(g) d_r phi(g, nu)
//   B_r(g, nu) = c2(g) d_r phi(g, nu)
//   V(mu, nu) += sum_c sum_g L_c(g, mu) R_c(g, nu) + R_c(g, mu) L_c(g, nu)
// which is GridFock.cpp:11-49 (F0, F1, F2 einsums, F + F^T, scatter through
// BasisList) written as one symmetric rank-2k update per block.  Only tile
// pairs I <= J are formed; each result is scattered to (I, J) and (J, I)
// with FP64 atomics.  One CTA per (block, tile pair, spin).
#include "common.h"
#include "kernels.h"

namespace cgb {
namespace {

constexpr int kThreads = 256;
constexpr int kT = 32;   // output tile
constexpr int kKG = 32;  // points per inner chunk

template <int NC>
__global__ void __launch_bounds__(kThreads) fock_fp64_kernel(const BlockDesc* __restrict__ blocks,
                                                             const int* __restrict__ lists, int n, int type,
                                                             const double* __restrict__ ao, long Gp,
                                                             const double* __restrict__ fcoef,
                                                             double* __restrict__ V) {
    __shared__ double LI[kKG][kT + 1], RI[kKG][kT + 1], LJ[kKG][kT + 1], RJ[kKG][kT + 1];
    const BlockDesc bd = blocks[blockIdx.x];
    const int nb = bd.nb, ng = bd.ng;
    const int ntile = (nb + kT - 1) / kT;
    int p = blockIdx.y, I = 0;
    while (I < ntile && p >= ntile - I) {
        p -= ntile - I;
        I++;
    }
    if (I >= ntile) return;
    const int J = I + p;
    const int spin = blockIdx.z;
    const int* list = lists + bd.bas_off;
    const double* A0 = ao + bd.ao_off;
    const long cs = (long)nb * ng;
    const double* fc = fcoef + (long)spin * 5 * Gp + bd.pt_off;
    const int tid = threadIdx.x;
    const int tx = tid & 31, ty = tid >> 5;  // mu = I*32 + tx, nu = J*32 + ty*4 + j
    double acc[4] = {0, 0, 0, 0};

    for (int c = 0; c < NC; c++) {
        for (int g0 = 0; g0 < ng; g0 += kKG) {
            for (int idx = tid; idx < kKG * kT; idx += kThreads) {
                const int k = idx / kT, m = idx % kT;
                const int g = g0 + k;
                const int mi = I * kT + m, mj = J * kT + m;
                double li = 0, ri = 0, lj = 0, rj = 0;
                if (g < ng) {
                    const double c0 = fc[g];
                    if (c == 0) {
                        const double c1x = type >= 1 ? fc[Gp + g] : 0.0, c1y = type >= 1 ? fc[2 * Gp + g] : 0.0,
                                     c1z = type >= 1 ? fc[3 * Gp + g] : 0.0;
                        if (mi < nb) {
                            const long o = (long)mi * ng + g;
                            li = A0[o];
                            ri = c0 * li;
                            if (type >= 1) ri += c1x * A0[cs + o] + c1y * A0[2 * cs + o] + c1z * A0[3 * cs + o];
                        }
                        if (mj < nb) {
                            const long o = (long)mj * ng + g;
                            lj = A0[o];
                            rj = c0 * lj;
                            if (type >= 1) rj += c1x * A0[cs + o] + c1y * A0[2 * cs + o] + c1z * A0[3 * cs + o];
                        }
                    } else {
                        const double c2 = fc[4 * Gp + g];
                        if (mi < nb) {
                            li = A0[c * cs + (long)mi * ng + g];
                            ri = c2 * li;
                        }
                        if (mj < nb) {
                            lj = A0[c * cs + (long)mj * ng + g];
                            rj = c2 * lj;
                        }
                    }
                }
                LI[k][m] = li;
                RI[k][m] = ri;
                LJ[k][m] = lj;
                RJ[k][m] = rj;
            }
            __syncthreads();
#pragma unroll 8
            for (int k = 0; k < kKG; k++) {
                const double li = LI[k][tx], ri = RI[k][tx];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    acc[j] = fma(li, RJ[k][ty * 4 + j], acc[j]);
                    acc[j] = fma(ri, LJ[k][ty * 4 + j], acc[j]);
                }
            }
            __syncthreads();
        }
    }
    const int mu = I * kT + tx;
    if (mu >= nb) return;
    double* Vs = V + (long)spin * n * n;
    const int gmu = list[mu];
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int nu = J * kT + ty * 4 + j;
        if (nu >= nb) continue;
        const int gnu = list[nu];
        atomicAdd(&Vs[(long)gnu * n + gmu], acc[j]);
        if (I != J) atomicAdd(&Vs[(long)gmu * n + gnu], acc[j]);
    }
}

}  // namespace

void launch_fock_fp64(int nblocks, const BlockDesc* d_blocks, const int* d_lists, int max_nb, int nbasis, int nspin,
                      int type, const double* ao, long Gp, const double* fcoef, double* V, cudaStream_t s) {
    if (nblocks == 0 || max_nb == 0) return;
    const int nt = (max_nb + kT - 1) / kT;
    dim3 grid(nblocks, nt * (nt + 1) / 2, nspin);
    if (type >= 2)
        fock_fp64_kernel<4><<<grid, kThreads, 0, s>>>(d_blocks, d_lists, nbasis, type, ao, Gp, fcoef, V);
    else
        fock_fp64_kernel<1><<<grid, kThreads, 0, s>>>(d_blocks, d_lists, nbasis, type, ao, Gp, fcoef, V);
    CGB_CUDA(cudaGetLastError());
}

}  // namespace cgb
