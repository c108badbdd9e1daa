// Hessian skeleton terms of V_xc, FP64, LDA and GGA, with the grid held
// fixed: the skeleton density derivatives of SubGrid::getDensitySkeleton
// (GridDensity.cpp:79-130) and the skeleton Fock derivatives of
// SubGrid::getFockSkeleton (GridFock.cpp:52-95), for every atom A and
// direction t (matrix m = 3 A + t; q = s nmat + m over spins).  getFockU<s_t>
// then runs the response coefficient and V kernels on these densities.
//
//   T_c(g, nu)            = sum_mu phi_c(g, mu) D(mu, nu)          (c = 0: phi; 1..3: d_r phi)
//   RhoGrad(g, t, A)      = -2 sum_{nu on A} d_t phi_nu T_0(g, nu)
//   Rho1Grad(g, r, t, A)  = -2 sum_{nu on A} [d_r d_t phi_nu T_0(g, nu) + d_t phi_nu T_r(g, nu)]
//   X_t(mu, nu)           = sum_g [d_t phi_mu (2 c0 phi_nu + c1 . grad phi_nu) + (sum_r c1_r d_r d_t phi_mu) phi_nu]
//   F_skel[A, t]          = -(X_t restricted to rows mu on A) - its transpose
// with c0 = 1/2 w v_rho and c1 the gradient coefficients of V_xc (fcoef).  AO
// store components: 0 phi, 1-3 d_x, d_y, d_z phi, 4-9 xx, xy, xz, yy, yz, zz.
#include "common.h"
#include "kernels.h"

namespace cgb {
namespace {

constexpr int kThreads = 256;
constexpr int kNV = 32;
__constant__ int c_hess[3][3] = {{4, 5, 6}, {5, 7, 8}, {6, 8, 9}};

// One CTA per (block, spin): the products T_c tiled as in the FP64 density
// kernel (128 points x 32 functions), then per point the sums over each
// atom's functions, flushed with FP64 atomics when the atom changes.
template <int FAM, int NC, int kKC>
__global__ void __launch_bounds__(kThreads) skel_density_kernel(const BlockDesc* __restrict__ blocks,
                                                                const int* __restrict__ lists,
                                                                const int* __restrict__ atom_list, int n, int nmat,
                                                                const double* __restrict__ D,
                                                                const double* __restrict__ ao, long Gp,
                                                                double* __restrict__ rhog,
                                                                double* __restrict__ rho1g) {
    __shared__ double Ps[NC][kKC][kMaxBlockPts];
    __shared__ double Ds[kKC][kNV];
    const BlockDesc bd = blocks[blockIdx.x];
    const int spin = blockIdx.y;
    const int ng = bd.ng, nb = bd.nb;
    const int* list = lists + bd.bas_off;
    const int* atoms = atom_list + bd.bas_off;
    const double* A0 = ao + bd.ao_off;
    const long cs = (long)nb * ng;
    const double* Dsp = D + (long)spin * n * n;
    const int tid = threadIdx.x;
    const int tg = tid & 31, tv = tid >> 5;
    const long q0 = (long)spin * nmat;

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
                for (int c = 0; c < NC; c++)
#pragma unroll
                    for (int i = 0; i < 4; i++) {
                        const double pv = Ps[c][k][tg + 32 * i];
#pragma unroll
                        for (int j = 0; j < 4; j++) acc[c][i][j] = fma(pv, dv[j], acc[c][i][j]);
                    }
            }
            __syncthreads();
        }
        // per point: the thread's four functions, grouped by atom
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int g = tg + 32 * i;
            if (g >= ng) continue;
            const long gp = bd.pt_off + g;
            double r0[3] = {0, 0, 0}, r1[3][3] = {};
            int cur = -1;
            auto flush = [&]() {
                if (cur < 0) return;
#pragma unroll
                for (int t = 0; t < 3; t++) {
                    const long q = q0 + 3 * cur + t;
                    atomicAdd(&rhog[q * Gp + gp], -2.0 * r0[t]);
                    r0[t] = 0;
                    if (FAM >= 1) {
#pragma unroll
                        for (int r = 0; r < 3; r++) {
                            atomicAdd(&rho1g[(q * 3 + r) * Gp + gp], -2.0 * r1[t][r]);
                            r1[t][r] = 0;
                        }
                    }
                }
            };
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int nu = nu0 + tv * 4 + j;
                if (nu >= nb) break;
                const int a = atoms[nu];
                if (a != cur) {
                    flush();
                    cur = a;
                }
                const long o = (long)nu * ng + g;
                const double T0 = acc[0][i][j];
#pragma unroll
                for (int t = 0; t < 3; t++) {
                    const double dt = A0[(1 + t) * cs + o];
                    r0[t] = fma(dt, T0, r0[t]);
                    if (FAM >= 1) {
#pragma unroll
                        for (int r = 0; r < 3; r++)
                            r1[t][r] += A0[c_hess[r][t] * cs + o] * T0 + dt * acc[NC == 4 ? 1 + r : 0][i][j];
                    }
                }
            }
            flush();
        }
    }
}

constexpr int kT = 32;   // output tile
constexpr int kKG = 32;  // points per chunk

// One CTA per (block, tile pair I x J, spin and direction): X_t(mu in I, nu in J),
// scattered with FP64 atomics to F[s, 3 A(mu) + t] at (mu, nu) and (nu, mu) with a minus sign.
template <int FAM>
__global__ void __launch_bounds__(kThreads) fock_skel_kernel(const BlockDesc* __restrict__ blocks,
                                                             const int* __restrict__ lists,
                                                             const int* __restrict__ atom_list, int n, int nmat,
                                                             const double* __restrict__ ao, long Gp,
                                                             const double* __restrict__ fcoef,
                                                             double* __restrict__ F) {
    __shared__ double L1[kKG][kT + 1], L2[kKG][kT + 1], R1[kKG][kT + 1], R2[kKG][kT + 1];
    const BlockDesc bd = blocks[blockIdx.x];
    const int nb = bd.nb, ng = bd.ng;
    if (nb == 0) return;
    const int ntile = (nb + kT - 1) / kT;
    const int I = blockIdx.y / ntile, J = blockIdx.y % ntile;
    if (I >= ntile) return;
    const int spin = blockIdx.z / 3, t = blockIdx.z % 3;
    const int* list = lists + bd.bas_off;
    const int* atoms = atom_list + bd.bas_off;
    const double* A0 = ao + bd.ao_off;
    const long cs = (long)nb * ng;
    const double* fc = fcoef + (long)spin * 5 * Gp + bd.pt_off;
    const int tid = threadIdx.x;
    const int tx = tid & 31, ty = tid >> 5;  // mu = I*32 + tx, nu = J*32 + ty*4 + j
    double acc[4] = {0, 0, 0, 0};
    for (int g0 = 0; g0 < ng; g0 += kKG) {
        for (int idx = tid; idx < kKG * kT; idx += kThreads) {
            const int k = idx / kT, m = idx % kT;
            const int g = g0 + k;
            const int mi = I * kT + m, mj = J * kT + m;
            double l1 = 0, l2 = 0, r1 = 0, r2 = 0;
            if (g < ng) {
                const double c0 = fc[g];
                const double c1x = FAM >= 1 ? fc[Gp + g] : 0.0, c1y = FAM >= 1 ? fc[2 * Gp + g] : 0.0,
                             c1z = FAM >= 1 ? fc[3 * Gp + g] : 0.0;
                if (mi < nb) {
                    const long o = (long)mi * ng + g;
                    l1 = A0[(1 + t) * cs + o];
                    if (FAM >= 1)
                        l2 = c1x * A0[c_hess[0][t] * cs + o] + c1y * A0[c_hess[1][t] * cs + o] +
                             c1z * A0[c_hess[2][t] * cs + o];
                }
                if (mj < nb) {
                    const long o = (long)mj * ng + g;
                    r2 = A0[o];
                    r1 = 2.0 * c0 * r2;
                    if (FAM >= 1) r1 += c1x * A0[cs + o] + c1y * A0[2 * cs + o] + c1z * A0[3 * cs + o];
                }
            }
            L1[k][m] = l1;
            L2[k][m] = l2;
            R1[k][m] = r1;
            R2[k][m] = r2;
        }
        __syncthreads();
#pragma unroll 8
        for (int k = 0; k < kKG; k++) {
            const double a1 = L1[k][tx], a2 = L2[k][tx];
#pragma unroll
            for (int j = 0; j < 4; j++) acc[j] = fma(a1, R1[k][ty * 4 + j], fma(a2, R2[k][ty * 4 + j], acc[j]));
        }
        __syncthreads();
    }
    const int mu = I * kT + tx;
    if (mu >= nb) return;
    const int gmu = list[mu];
    double* Fq = F + ((long)spin * nmat + 3 * atoms[mu] + t) * n * n;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int nu = J * kT + ty * 4 + j;
        if (nu >= nb) continue;
        const int gnu = list[nu];
        atomicAdd(&Fq[(long)gnu * n + gmu], -acc[j]);
        atomicAdd(&Fq[(long)gmu * n + gnu], -acc[j]);
    }
}

}  // namespace

void launch_skel_density(int nblocks, const BlockDesc* d_blocks, const int* d_lists, const int* d_atom_list,
                         int nbasis, int nspin, int nmat, int family, const double* D, const double* ao, long Gp,
                         double* rhog, double* rho1g, cudaStream_t s) {
    if (nblocks == 0) return;
    CGB_CHECK(family <= 1, XC_ERR_UNSUPPORTED, "skeleton terms cover LDA and GGA (as the reference's Hessian)");
    CGB_CHECK((long)nspin <= 65535, XC_ERR_ARG, "too many spins");
    dim3 grid(nblocks, nspin);
    if (family == 0)
        skel_density_kernel<0, 1, 16><<<grid, kThreads, 0, s>>>(d_blocks, d_lists, d_atom_list, nbasis, nmat, D, ao,
                                                                Gp, rhog, rho1g);
    else
        skel_density_kernel<1, 4, 8><<<grid, kThreads, 0, s>>>(d_blocks, d_lists, d_atom_list, nbasis, nmat, D, ao,
                                                               Gp, rhog, rho1g);
    CGB_CUDA(cudaGetLastError());
}

void launch_fock_skel(int nblocks, const BlockDesc* d_blocks, const int* d_lists, const int* d_atom_list,
                      int max_nb, int nbasis, int nspin, int nmat, int family, const double* ao, long Gp,
                      const double* fcoef, double* F, cudaStream_t s) {
    if (nblocks == 0 || max_nb == 0) return;
    CGB_CHECK(family <= 1, XC_ERR_UNSUPPORTED, "skeleton terms cover LDA and GGA (as the reference's Hessian)");
    const int nt = (max_nb + kT - 1) / kT;
    CGB_CHECK((long)nt * nt <= 65535 && 3L * nspin <= 65535, XC_ERR_ARG, "block too large for the tile grid");
    dim3 grid(nblocks, nt * nt, 3 * nspin);
    if (family == 0)
        fock_skel_kernel<0><<<grid, kThreads, 0, s>>>(d_blocks, d_lists, d_atom_list, nbasis, nmat, ao, Gp, fcoef, F);
    else
        fock_skel_kernel<1><<<grid, kThreads, 0, s>>>(d_blocks, d_lists, d_atom_list, nbasis, nmat, ao, Gp, fcoef, F);
    CGB_CUDA(cudaGetLastError());
}

}  // namespace cgb
