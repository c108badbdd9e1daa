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

// Float-float arithmetic (value = hi + lo, two FP32s, 48-bit significand):
// FP64-level products and sums on the FP32 pipe, which GB300 runs at 64x its
// FP64 rate.  ff_split is exact to 2^-48 relative; ff_fma adds the exact
// product error (FMA) and the exact sum error (TwoSum, Knuth) to lo.
__device__ __forceinline__ float2 ff_split(double v) {
    const float hi = (float)v;
    return make_float2(hi, (float)(v - (double)hi));
}
__device__ __forceinline__ void ff_fma(float2 a, float2 b, float2& acc) {
    const float p = __fmul_rn(a.x, b.x);
    const float e = __fmaf_rn(a.x, b.x, -p);
    const float t = __fadd_rn(acc.x, p);
    const float z = __fsub_rn(t, acc.x);
    const float err = __fadd_rn(__fsub_rn(acc.x, __fsub_rn(t, z)), __fsub_rn(p, z));
    acc.x = t;
    acc.y = __fadd_rn(acc.y, __fadd_rn(__fadd_rn(err, e), __fmaf_rn(a.x, b.y, __fmul_rn(a.y, b.x))));
}
__device__ __forceinline__ double ff_value(float2 a) { return (double)a.x + (double)a.y; }

__global__ void split_ff_kernel(long n, const double* __restrict__ src, float2* __restrict__ dst) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        dst[i] = ff_split(src[i]);
}

// density_fp64_kernel in float-float: the same tiles and block layout, with
// the AO store and D already split into float pairs (split_ff_kernel), so
// the product and the contraction run on the FP32 pipe; the FP64 pipe only
// sums the eight nu-groups of each point.  ~1e-14 relative: the density of
// the incremental build's references.
template <int NC, int kKC>
__global__ void __launch_bounds__(kThreads) density_ff_kernel(const BlockDesc* __restrict__ blocks,
                                                              const int* __restrict__ lists, int n, int type,
                                                              const float2* __restrict__ D,
                                                              const float2* __restrict__ ao, long Gp,
                                                              double* __restrict__ rho, double* __restrict__ rho1,
                                                              double* __restrict__ tau) {
    __shared__ float2 Ps[NC][kKC][kMaxBlockPts];
    __shared__ float2 Ds[kKC][kNV];
    __shared__ double red[8][kMaxBlockPts];

    const BlockDesc bd = blocks[blockIdx.x];
    const int spin = blockIdx.y;
    const int ng = bd.ng, nb = bd.nb;
    const int* list = lists + bd.bas_off;
    const float2* A0 = ao + bd.ao_off;
    const long cs = (long)nb * ng;
    const float2* Dsp = D + (long)spin * n * n;
    const int tid = threadIdx.x;
    const int tg = tid & 31, tv = tid >> 5;
    const float2 zero = make_float2(0.f, 0.f);

    float2 prho[4], pgr[3][4], ptau[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        prho[i] = ptau[i] = zero;
#pragma unroll
        for (int r = 0; r < 3; r++) pgr[r][i] = zero;
    }

    for (int nu0 = 0; nu0 < nb; nu0 += kNV) {
        float2 acc[NC][4][4];
#pragma unroll
        for (int c = 0; c < NC; c++)
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[c][i][j] = zero;
        for (int mu0 = 0; mu0 < nb; mu0 += kKC) {
            for (int idx = tid; idx < NC * kKC * kMaxBlockPts; idx += kThreads) {
                const int c = idx / (kKC * kMaxBlockPts);
                const int rem = idx % (kKC * kMaxBlockPts);
                const int k = rem / kMaxBlockPts, g = rem % kMaxBlockPts;
                const int mu = mu0 + k;
                Ps[c][k][g] = (mu < nb && g < ng) ? A0[c * cs + (long)mu * ng + g] : zero;
            }
            for (int idx = tid; idx < kKC * kNV; idx += kThreads) {
                const int k = idx / kNV, j = idx % kNV;
                const int mu = mu0 + k, nu = nu0 + j;
                Ds[k][j] = (mu < nb && nu < nb) ? Dsp[(long)list[nu] * n + list[mu]] : zero;
            }
            __syncthreads();
#pragma unroll 2
            for (int k = 0; k < kKC; k++) {
                float2 dv[4];
#pragma unroll
                for (int j = 0; j < 4; j++) dv[j] = Ds[k][tv * 4 + j];
#pragma unroll
                for (int c = 0; c < NC; c++) {
#pragma unroll
                    for (int i = 0; i < 4; i++) {
                        const float2 pv = Ps[c][k][tg + 32 * i];
#pragma unroll
                        for (int j = 0; j < 4; j++) ff_fma(pv, dv[j], acc[c][i][j]);
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
                const float2 t0 = acc[0][i][j];
                ff_fma(t0, A0[o], prho[i]);
                if (type >= 1) {
                    const float2 t2 = make_float2(2.f * t0.x, 2.f * t0.y);  // exact
#pragma unroll
                    for (int r = 0; r < 3; r++) ff_fma(t2, A0[(1 + r) * cs + o], pgr[r][i]);
                }
                if (NC == 4) {
#pragma unroll
                    for (int r = 0; r < 3; r++) {
                        const float2 a = acc[NC == 4 ? 1 + r : 0][i][j];
                        ff_fma(make_float2(0.5f * a.x, 0.5f * a.y), A0[(1 + r) * cs + o], ptau[i]);
                    }
                }
            }
        }
    }
    const int nq = (NC == 4) ? 5 : (type >= 1 ? 4 : 1);
    for (int q = 0; q < nq; q++) {
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const float2 v = q == 0 ? prho[i] : (q < 4 ? pgr[q - 1][i] : ptau[i]);
            red[tv][tg + 32 * i] = ff_value(v);
        }
        __syncthreads();
        if (tid < kMaxBlockPts && tid < ng) {
            double sum = 0;
#pragma unroll
            for (int t = 0; t < 8; t++) sum += red[t][tid];
            const long gi = bd.pt_off + tid;
            if (q == 0) rho[(long)spin * Gp + gi] = sum;
            else if (q < 4) rho1[((long)spin * 3 + (q - 1)) * Gp + gi] = sum;
            else tau[(long)spin * Gp + gi] = sum;
        }
        __syncthreads();
    }
}

}  // namespace

void launch_split_ff(long n, const double* src, float2* dst, cudaStream_t s) {
    if (n <= 0) return;
    const long want = (n + 255) / 256;
    split_ff_kernel<<<(unsigned)(want < 152 * 16 ? want : 152 * 16), 256, 0, s>>>(n, src, dst);
    CGB_CUDA(cudaGetLastError());
}

void launch_density_ff(int nblocks, const BlockDesc* d_blocks, const int* d_lists, int nbasis, int nspin, int type,
                       const float2* D, const float2* ao, long Gp, double* rho, double* rho1, double* tau,
                       cudaStream_t s) {
    if (nblocks == 0) return;
    dim3 grid(nblocks, nspin);
    if (type >= 2)
        density_ff_kernel<4, 8><<<grid, kThreads, 0, s>>>(d_blocks, d_lists, nbasis, type, D, ao, Gp, rho, rho1, tau);
    else
        density_ff_kernel<1, 16><<<grid, kThreads, 0, s>>>(d_blocks, d_lists, nbasis, type, D, ao, Gp, rho, rho1, tau);
    CGB_CUDA(cudaGetLastError());
}

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
