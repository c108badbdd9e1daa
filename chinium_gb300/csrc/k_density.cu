// FP64 density kernel (plain path): per grid block b,
//   T_c(g, nu) = sum_mu phi_c(g, mu) D(list mu, list nu)      (c = 0, and 1..3 for meta-GGA)
//   rho(g)     = sum_nu T_0(g, nu) phi(g, nu)
//   rho1_r(g)  = 2 sum_nu T_0(g, nu) d_r phi(g, nu)
//   tau(g)     = 1/2 sum_r sum_nu T_r(g, nu) d_r phi(g, nu)
// which is GridDensity.cpp:12-41 with the D*phi product formed once per
// block and reused for rho and grad rho.  One CTA per (block, spin); the
// product is tiled 128 points x 32 functions x 16 inner, staged in shared
// memory, so the FP64 pipe (not memory) bounds it.
#include "common.h"
#include "kernels.h"

namespace cgb {
namespace {

constexpr int kThreads = 256;
constexpr int kNV = 32;  // nu tile

template <int NC, int kKC>  // kKC: inner (mu) chunk, sized to fit 48 KB static smem
__global__ void __launch_bounds__(kThreads) density_fp64_kernel(const BlockDesc* __restrict__ blocks,
                                                                const int* __restrict__ lists, int n, int type,
                                                                const double* __restrict__ D,
                                                                const double* __restrict__ ao, long Gp,
                                                                double* __restrict__ rho, double* __restrict__ rho1,
                                                                double* __restrict__ tau) {
    __shared__ double Ps[NC][kKC][kMaxBlockPts];
    __shared__ double Ds[kKC][kNV];
    __shared__ double red[8][kMaxBlockPts];

    const BlockDesc bd = blocks[blockIdx.x];
    const int spin = blockIdx.y;
    const int ng = bd.ng, nb = bd.nb;
    const int* list = lists + bd.bas_off;
    const double* A0 = ao + bd.ao_off;
    const long cs = (long)nb * ng;
    const double* Dsp = D + (long)spin * n * n;
    const int tid = threadIdx.x;
    const int tg = tid & 31, tv = tid >> 5;

    double prho[4] = {0, 0, 0, 0};
    double pgr[3][4] = {};
    double ptau[4] = {0, 0, 0, 0};

    for (int nu0 = 0; nu0 < nb; nu0 += kNV) {
        double acc[NC][4][4];
#pragma unroll
        for (int c = 0; c < NC; c++)
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[c][i][j] = 0;
        for (int mu0 = 0; mu0 < nb; mu0 += kKC) {
            for (int idx = tid; idx < NC * kKC * kMaxBlockPts; idx += kThreads) {
                const int c = idx / (kKC * kMaxBlockPts);
                const int rem = idx % (kKC * kMaxBlockPts);
                const int k = rem / kMaxBlockPts, g = rem % kMaxBlockPts;
                const int mu = mu0 + k;
                Ps[c][k][g] = (mu < nb && g < ng) ? A0[c * cs + (long)mu * ng + g] : 0.0;
            }
            for (int idx = tid; idx < kKC * kNV; idx += kThreads) {
                const int k = idx / kNV, j = idx % kNV;
                const int mu = mu0 + k, nu = nu0 + j;
                Ds[k][j] = (mu < nb && nu < nb) ? Dsp[(long)list[nu] * n + list[mu]] : 0.0;
            }
            __syncthreads();
#pragma unroll 4
            for (int k = 0; k < kKC; k++) {
                double dv[4];
#pragma unroll
                for (int j = 0; j < 4; j++) dv[j] = Ds[k][tv * 4 + j];
#pragma unroll
                for (int c = 0; c < NC; c++) {
#pragma unroll
                    for (int i = 0; i < 4; i++) {
                        const double pv = Ps[c][k][tg + 32 * i];
#pragma unroll
                        for (int j = 0; j < 4; j++) acc[c][i][j] = fma(pv, dv[j], acc[c][i][j]);
                    }
                }
            }
            __syncthreads();
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int nu = nu0 + tv * 4 + j;
            if (nu >= nb) continue;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int g = tg + 32 * i;
                if (g >= ng) continue;
                const long o = (long)nu * ng + g;
                prho[i] = fma(acc[0][i][j], A0[o], prho[i]);
                if (type >= 1) {
#pragma unroll
                    for (int r = 0; r < 3; r++) pgr[r][i] = fma(2.0 * acc[0][i][j], A0[(1 + r) * cs + o], pgr[r][i]);
                }
                if (NC == 4) {
                    double t = 0;
#pragma unroll
                    for (int r = 0; r < 3; r++) t = fma(acc[NC == 4 ? 1 + r : 0][i][j], A0[(1 + r) * cs + o], t);
                    ptau[i] = fma(0.5, t, ptau[i]);
                }
            }
        }
    }
    // reduce the 8 nu-groups: rho, rho1 x3, tau
    const int nq = (NC == 4) ? 5 : (type >= 1 ? 4 : 1);
    for (int q = 0; q < nq; q++) {
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const double v = q == 0 ? prho[i] : (q < 4 ? pgr[q - 1][i] : ptau[i]);
            red[tv][tg + 32 * i] = v;
        }
        __syncthreads();
        if (tid < kMaxBlockPts && tid < ng) {
            double s = 0;
#pragma unroll
            for (int t = 0; t < 8; t++) s += red[t][tid];
            const long gi = bd.pt_off + tid;
            if (q == 0) rho[(long)spin * Gp + gi] = s;
            else if (q < 4) rho1[((long)spin * 3 + (q - 1)) * Gp + gi] = s;
            else tau[(long)spin * Gp + gi] = s;
        }
        __syncthreads();
    }
}

}  // namespace

void launch_density_fp64(int nblocks, const BlockDesc* d_blocks, const int* d_lists, int nbasis, int nspin, int type,
                         const double* D, const double* ao, long Gp, double* rho, double* rho1, double* tau,
                         cudaStream_t s) {
    if (nblocks == 0) return;
    dim3 grid(nblocks, nspin);
    if (type >= 2)
        density_fp64_kernel<4, 8><<<grid, kThreads, 0, s>>>(d_blocks, d_lists, nbasis, type, D, ao, Gp, rho, rho1, tau);
    else
        density_fp64_kernel<1, 16><<<grid, kThreads, 0, s>>>(d_blocks, d_lists, nbasis, type, D, ao, Gp, rho, rho1, tau);
    CGB_CUDA(cudaGetLastError());
}

}  // namespace cgb
