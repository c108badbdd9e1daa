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
// FP64 density kernel (128 points x 32 functions x 16 inner); the
// per-(block, function) partials are summed by atom on the host in a fixed
// order.
//
// The two products run on the FP64 tensor path: mma.sync m8n8k4 (A 8 x 4
// row-major, B 4 x 8 column-major, one element of each per lane; C 8 x 8, two
// per lane: row lane / 4, columns 2 (lane % 4) + {0, 1}).  Warp w owns the
// 8-function column tile w % 4 of the 32-function tile and the 64 points of
// half w / 4: eight 8-point row tiles, for T and U.  The contraction with the
// AO gradients and Hessians then sums its points in registers, across the
// lanes of a column group by shuffles, and across the two point halves in
// shared memory.
#include "common.h"
#include "kernels.h"

namespace cgb {
namespace {

constexpr int kThreads = 256;
constexpr int kNV = 32;                // nu tile
constexpr int kKC = 16;                // inner (mu) chunk
constexpr int kPS = kMaxBlockPts + 4;  // padded point stride of the staged chunk (bank spread)

// d += a b, FP64 8 x 8 x 4 (fragments as above)
__device__ __forceinline__ void dmma(double (&d)[2], double a, double b) {
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};\n"
                 : "+d"(d[0]), "+d"(d[1])
                 : "d"(a), "d"(b));
}

template <int FAM>
__global__ void __launch_bounds__(kThreads) grad_fp64_kernel(const BlockDesc* __restrict__ blocks,
                                                             const int* __restrict__ lists, int n,
                                                             const double* __restrict__ D,
                                                             const double* __restrict__ ao, long Gp,
                                                             const double* __restrict__ fcoef, long nlist,
                                                             double* __restrict__ part) {
    __shared__ double Ps[2][kKC][kPS];      // phi and the Z-like combination of the mu chunk
    __shared__ double Ds[kKC][kNV + 1];
    __shared__ double fs[4][kMaxBlockPts];  // 2 fcoef0, f_x, f_y, f_z of the block's points
    __shared__ double red[2][kNV][3];       // per point half: the column tile's sums

    const BlockDesc bd = blocks[blockIdx.x];
    const int spin = blockIdx.y;
    const int ng = bd.ng, nb = bd.nb;
    const int* list = lists + bd.bas_off;
    const double* A0 = ao + bd.ao_off;
    const long cs = (long)nb * ng;
    const double* Dsp = D + (long)spin * n * n;
    const double* fc = fcoef + (long)spin * 5 * Gp + bd.pt_off;
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int nt = warp & 3, ph = warp >> 2;  // column tile, point half
    const int gr = lane >> 2, kq = lane & 3;  // fragment row / column group, k index / column pair
    for (int g = tid; g < kMaxBlockPts; g += kThreads) {
        const bool in = g < ng;
        fs[0][g] = in ? 2.0 * fc[g] : 0.0;
        fs[1][g] = (in && FAM >= 1) ? fc[Gp + g] : 0.0;
        fs[2][g] = (in && FAM >= 1) ? fc[2 * Gp + g] : 0.0;
        fs[3][g] = (in && FAM >= 1) ? fc[3 * Gp + g] : 0.0;
    }
    __syncthreads();

    for (int nu0 = 0; nu0 < nb; nu0 += kNV) {
        double accT[8][2], accU[8][2];
#pragma unroll
        for (int i = 0; i < 8; i++) accT[i][0] = accT[i][1] = accU[i][0] = accU[i][1] = 0.0;
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
#pragma unroll
            for (int ks = 0; ks < kKC / 4; ks++) {
                const int k = 4 * ks + kq;
                const double b = Ds[k][8 * nt + gr];  // B(mu = k, nu = 8 nt + gr)
#pragma unroll
                for (int mt = 0; mt < 8; mt++) {
                    const int g = 64 * ph + 8 * mt + gr;  // A(point g, mu = k)
                    dmma(accT[mt], Ps[0][k][g], b);
                    dmma(accU[mt], Ps[1][k][g], b);
                }
            }
            __syncthreads();
        }
        // contraction: this lane holds points 64 ph + 8 mt + gr and functions nu0 + 8 nt + 2 kq + i
        double sx[2] = {0, 0}, sy[2] = {0, 0}, sz[2] = {0, 0};
#pragma unroll
        for (int i = 0; i < 2; i++) {
            const int nu = nu0 + 8 * nt + 2 * kq + i;
            if (nu >= nb) continue;
#pragma unroll
            for (int mt = 0; mt < 8; mt++) {
                const int g = 64 * ph + 8 * mt + gr;
                if (g >= ng) continue;
                const long o = (long)nu * ng + g;
                const double U = accU[mt][i], T = accT[mt][i];
                double gx = A0[cs + o] * U, gy = A0[2 * cs + o] * U, gz = A0[3 * cs + o] * U;
                if (FAM >= 1) {
                    const double fx = fs[1][g] * T, fy = fs[2][g] * T, fz = fs[3][g] * T;
                    const double hxx = A0[4 * cs + o], hxy = A0[5 * cs + o], hxz = A0[6 * cs + o];
                    const double hyy = A0[7 * cs + o], hyz = A0[8 * cs + o], hzz = A0[9 * cs + o];
                    gx += hxx * fx + hxy * fy + hxz * fz;
                    gy += hxy * fx + hyy * fy + hyz * fz;
                    gz += hxz * fx + hyz * fy + hzz * fz;
                }
                sx[i] += gx;
                sy[i] += gy;
                sz[i] += gz;
            }
        }
        // sum over the eight row groups (the lanes with equal kq)
#pragma unroll
        for (int i = 0; i < 2; i++)
#pragma unroll
            for (int off = 4; off < 32; off <<= 1) {
                sx[i] += __shfl_xor_sync(0xffffffffu, sx[i], off);
                sy[i] += __shfl_xor_sync(0xffffffffu, sy[i], off);
                sz[i] += __shfl_xor_sync(0xffffffffu, sz[i], off);
            }
        if (gr == 0) {
#pragma unroll
            for (int i = 0; i < 2; i++) {
                const int j = 8 * nt + 2 * kq + i;
                red[ph][j][0] = sx[i];
                red[ph][j][1] = sy[i];
                red[ph][j][2] = sz[i];
            }
        }
        __syncthreads();
        if (tid < kNV * 3) {  // part[spin][list entry][t] for the tile's functions
            const int j = tid / 3, t = tid % 3;
            const int nu = nu0 + j;
            if (nu < nb) part[((long)spin * nlist + bd.bas_off + nu) * 3 + t] = -2.0 * (red[0][j][t] + red[1][j][t]);
        }
        __syncthreads();
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
