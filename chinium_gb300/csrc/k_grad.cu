// FP64 XC nuclear gradient with the grid held fixed (the reference's
// SubGrid::getDensitySkeleton + SubGrid::getEnergyGrad, GridDensity.cpp:79-130
// and GridEnergy.cpp:15-30: LDA and GGA).  With fcoef(s, 0) = 1/2 w v_rho and
// fcoef(s, 1:4) = f_r (the gradient coefficients of V_xc), per spin and grid
// block
//   T(g, nu)  = sum_mu D(nu, mu) phi(g, mu)
//   U(g, nu)  = sum_mu D(nu, mu) [2 fcoef0(g) phi(g, mu) + sum_r f_r(g) d_r phi(g, mu)]
//   dE/dR_{A,t} += -2 sum_{nu on A} sum_g [d_t phi(g, nu) U(g, nu) + sum_r d_t d_r phi(g, nu) f_r(g) T(g, nu)]
// which is dE = sum_g w (v_rho d rho + v_sigma d sigma) with d rho and d grad rho
// the derivatives of the functions centred on A.  T and U are tiled like the
// FP64 density kernel (128 points x 32 functions x 16 inner); each warp owns
// four functions of the tile and reduces its point sums with shuffles; the
// per-(block, function) partials are summed by atom on the host in a fixed
// order.
#include "common.h"
#include "kernels.h"

namespace cgb {
namespace {

constexpr int kThreads = 256;
constexpr int kNV = 32;  // nu tile
constexpr int kKC = 16;  // inner (mu) chunk

template <int FAM>
__global__ void __launch_bounds__(kThreads) grad_fp64_kernel(const BlockDesc* __restrict__ blocks,
                                                             const int* __restrict__ lists, int n,
                                                             const double* __restrict__ D,
                                                             const double* __restrict__ ao, long Gp,
                                                             const double* __restrict__ fcoef, long nlist,
                                                             double* __restrict__ part) {
    __shared__ double Ps[2][kKC][kMaxBlockPts];  // phi and the Z-like combination of the mu chunk
    __shared__ double Ds[kKC][kNV];
    __shared__ double fs[4][kMaxBlockPts];       // 2 fcoef0, f_x, f_y, f_z of the block's points

    const BlockDesc bd = blocks[blockIdx.x];
    const int spin = blockIdx.y;
    const int ng = bd.ng, nb = bd.nb;
    const int* list = lists + bd.bas_off;
    const double* A0 = ao + bd.ao_off;
    const long cs = (long)nb * ng;
    const double* Dsp = D + (long)spin * n * n;
    const double* fc = fcoef + (long)spin * 5 * Gp + bd.pt_off;
    const int tid = threadIdx.x;
    const int tg = tid & 31, tv = tid >> 5;
    for (int g = tid; g < kMaxBlockPts; g += kThreads) {
        const bool in = g < ng;
        fs[0][g] = in ? 2.0 * fc[g] : 0.0;
        fs[1][g] = (in && FAM >= 1) ? fc[Gp + g] : 0.0;
        fs[2][g] = (in && FAM >= 1) ? fc[2 * Gp + g] : 0.0;
        fs[3][g] = (in && FAM >= 1) ? fc[3 * Gp + g] : 0.0;
    }
    __syncthreads();

    for (int nu0 = 0; nu0 < nb; nu0 += kNV) {
        double accT[4][4], accU[4][4];
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int j = 0; j < 4; j++) accT[i][j] = accU[i][j] = 0;
        for (int mu0 = 0; mu0 < nb; mu0 += kKC) {
            for (int idx = tid; idx < kKC * kMaxBlockPts; idx += kThreads) {
                const int k = idx / kMaxBlockPts, g = idx % kMaxBlockPts;
                const int mu = mu0 + k;
                double p = 0, z = 0;
                if (mu < nb && g < ng) {
                    const long o = (long)mu * ng + g;
                    p = A0[o];
                    z = fs[0][g] * p;
                    if (FAM >= 1) z += fs[1][g] * A0[cs + o] + fs[2][g] * A0[2 * cs + o] + fs[3][g] * A0[3 * cs + o];
                }
                Ps[0][k][g] = p;
                Ps[1][k][g] = z;
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
                for (int i = 0; i < 4; i++) {
                    const double pv = Ps[0][k][tg + 32 * i], zv = Ps[1][k][tg + 32 * i];
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        accT[i][j] = fma(pv, dv[j], accT[i][j]);
                        accU[i][j] = fma(zv, dv[j], accU[i][j]);
                    }
                }
            }
            __syncthreads();
        }
        // per function of the tile: sum over this thread's points, then over the warp
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int nu = nu0 + tv * 4 + j;
            double gx = 0, gy = 0, gz = 0;
            if (nu < nb) {
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const int g = tg + 32 * i;
                    if (g >= ng) continue;
                    const long o = (long)nu * ng + g;
                    const double U = accU[i][j], T = accT[i][j];
                    gx = fma(A0[cs + o], U, gx);
                    gy = fma(A0[2 * cs + o], U, gy);
                    gz = fma(A0[3 * cs + o], U, gz);
                    if (FAM >= 1) {
                        const double fx = fs[1][g] * T, fy = fs[2][g] * T, fz = fs[3][g] * T;
                        const double hxx = A0[4 * cs + o], hxy = A0[5 * cs + o], hxz = A0[6 * cs + o];
                        const double hyy = A0[7 * cs + o], hyz = A0[8 * cs + o], hzz = A0[9 * cs + o];
                        gx += hxx * fx + hxy * fy + hxz * fz;
                        gy += hxy * fx + hyy * fy + hyz * fz;
                        gz += hxz * fx + hyz * fy + hzz * fz;
                    }
                }
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                gx += __shfl_xor_sync(0xffffffffu, gx, off);
                gy += __shfl_xor_sync(0xffffffffu, gy, off);
                gz += __shfl_xor_sync(0xffffffffu, gz, off);
            }
            if (tg == 0 && nu < nb) {  // part[spin][list entry][t]
                double* o = part + ((long)spin * nlist + bd.bas_off + nu) * 3;
                o[0] = -2.0 * gx;
                o[1] = -2.0 * gy;
                o[2] = -2.0 * gz;
            }
        }
    }
}

}  // namespace

void launch_xc_grad(int nblocks, const BlockDesc* d_blocks, const int* d_lists, long nlist, int nbasis, int nspin,
                    int family, const double* D, const double* ao, long Gp, const double* fcoef, double* part,
                    cudaStream_t s) {
    if (nblocks == 0) return;
    CGB_CHECK(family <= 1, XC_ERR_UNSUPPORTED, "XC gradients cover LDA and GGA (as the reference's getEnergyGrad)");
    dim3 grid(nblocks, nspin);
    if (family == 0)
        grad_fp64_kernel<0><<<grid, kThreads, 0, s>>>(d_blocks, d_lists, nbasis, D, ao, Gp, fcoef, nlist, part);
    else
        grad_fp64_kernel<1><<<grid, kThreads, 0, s>>>(d_blocks, d_lists, nbasis, D, ao, Gp, fcoef, nlist, part);
    CGB_CUDA(cudaGetLastError());
}

}  // namespace cgb
