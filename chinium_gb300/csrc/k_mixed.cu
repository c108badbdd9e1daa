// Mixed-precision XC contractions on the 5th-generation tensor cores.
//
// Points are re-tiled into tiles of 128 consecutive points (generation order,
// spatially compact); each tile keeps the 64-function chunks of the basis
// that its screening test marks significant, packed into "slots".  Operands
// are three-term BF16 splits (x = h + m + l); a product sums the six
// cross terms of order <= 2 (hh, hm, mh, hl, mm, lh) in FP32 on the tensor
// core, ~FP32 accuracy.  The leading hh term and the five corrections go to
// separate TMEM accumulators, and every accumulation unit (one K-chunk of the
// density product, one point tile of the V_xc product) starts a fresh
// accumulator that the epilogue warps drain into round-to-nearest FP32
// registers: tensor-core accumulation chains stay a few instructions long.
// Cross-unit sums of the final quantities are FP64.
//
// HBM layouts (bf16, all rows 16-byte aligned, TMA 128-byte swizzle):
//   PF  (point-major): row (c*3+p)*Gt + t*128 + g, col slot*64 + f      [c: phi, d/dx, d/dy, d/dz]
//   FP  (function-major): row (c*3+p)*T*K + t*K + slot*64 + f, col g     (+64 zero rows)
//   R   (function-major, per build): row (c*3+p)*T*K + t*K + slot*64 + f, col g (+64 zero rows)
//   Dp  (density planes): row (s*3+p)*npad + nu, col mu
//
// CTA roles (192 threads): warp 0 issues TMA loads into a 2-stage ring,
// warp 1 issues tcgen05.mma into one of two TMEM buffers (256 columns each:
// hh | corrections), warps 2-5 drain TMEM (lane quadrant = warp % 4) and
// run the epilogue.  Every wait is bounded (2 s of %globaltimer) and a
// timeout sets XC_ERR_TIMEOUT in a global flag instead of hanging.
#include <cstdio>

#include "common.h"
#include "kernels.h"
#include "mixed.h"
#include "tc.cuh"

namespace cgb {
namespace {

using bf16 = __nv_bfloat16;

constexpr int kThreads = 192;
constexpr int kStages = 2;
constexpr uint32_t kPlaneA = 128 * 64 * 2;     // bytes of one 128x64 bf16 operand plane
constexpr uint32_t kStageBytes = 6 * kPlaneA;  // A (3 planes) + B (3 planes)
constexpr uint32_t kIdesc = tc::idesc_bf16(128, 128);
constexpr uint32_t kTmemCols = 512;            // 2 buffers x (hh 128 | corrections 128)
// cross terms (i, j) of the three-term splits with i + j <= 2; term 0 is hh
__constant__ int c_prod_a[6] = {0, 0, 1, 0, 1, 2};
__constant__ int c_prod_b[6] = {0, 1, 0, 2, 1, 0};

struct Smem {
    uint64_t full[kStages];
    uint64_t empty[kStages];
    uint64_t tfull[2];
    uint64_t tempty[2];
    uint32_t tmem;
    int abort;
};

__device__ __forceinline__ uint8_t* stage_base(uint8_t* aligned, int s) { return aligned + (size_t)s * kStageBytes; }

__device__ __forceinline__ void flag_timeout(int* err, Smem* sm) {
    atomicExch(err, XC_ERR_TIMEOUT);
    atomicExch(&sm->abort, 1);
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_u32(bar)) : "memory");
}

__device__ void init_cta(Smem& sm) {
    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; s++) {
            tc::mbar_init(&sm.full[s], 1);
            tc::mbar_init(&sm.empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            tc::mbar_init(&sm.tfull[b], 1);
            tc::mbar_init(&sm.tempty[b], 128);
        }
        sm.abort = 0;
        tc::fence_mbar_init();
    }
    if ((threadIdx.x >> 5) == 0) tc::tmem_alloc(&sm.tmem, kTmemCols);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
}

// The six split products of one stage into TMEM buffer `buf`: term hh into
// the hh accumulator, the five corrections into the correction accumulator.
// `first` starts both accumulators (unit boundary).
__device__ __forceinline__ void mma_stage(uint32_t tmem, int buf, uint8_t* st, bool first) {
    const uint32_t a0 = tc::smem_u32(st), b0 = a0 + 3 * kPlaneA;
    const uint32_t d_hh = tmem + buf * 256, d_corr = tmem + buf * 256 + 128;
#pragma unroll
    for (int q = 0; q < 6; q++) {
        const uint64_t ad = tc::smem_desc_sw128(a0 + c_prod_a[q] * kPlaneA);
        const uint64_t bd = tc::smem_desc_sw128(b0 + c_prod_b[q] * kPlaneA);
        const uint32_t d = q == 0 ? d_hh : d_corr;
#pragma unroll
        for (int k = 0; k < 4; k++) {  // K = 16 per instruction: +32 bytes in the swizzled row
            const bool start = first && k == 0 && (q == 0 || q == 1);
            tc::mma_bf16(d, ad + 2 * k, bd + 2 * k, kIdesc, start ? 0u : 1u);
        }
    }
}

// Drain TMEM buffer `buf` (hh + corrections) into acc[128] (this thread's lane).
__device__ __forceinline__ void drain(uint32_t tmem, int buf, int quad, float* acc) {
    const uint32_t base = tmem + ((uint32_t)(quad * 32) << 16) + buf * 256;
#pragma unroll
    for (int c16 = 0; c16 < 8; c16++) {
        float a[16], b[16];
        tc::tmem_ld16(base + c16 * 16, a);
        tc::tmem_ld16(base + 128 + c16 * 16, b);
#pragma unroll
        for (int j = 0; j < 16; j++) acc[c16 * 16 + j] += a[j] + b[j];
    }
}

// ------------------------------------------------------------ density
// T = Phi D for one tile, unit = (nu block vb of two slots, mu chunk kc).
// EPI 0: rho; 1: rho + grad rho; 2: tau contribution of A component acomp.
template <int EPI>
__global__ void __launch_bounds__(kThreads, 1) density_tc_kernel(const __grid_constant__ CUtensorMap tm_pf,
                                                                 const __grid_constant__ CUtensorMap tm_d,
                                                                 MixedDev md, int acomp, int spin,
                                                                 double* __restrict__ rho, double* __restrict__ rho1,
                                                                 double* __restrict__ tau, long Gp, int* err) {
    extern __shared__ uint8_t smem_raw[];
    __shared__ Smem sm;
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const int t = blockIdx.x;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nkept = md.tile_nkept[t];
    const int* chunks = md.tile_chunks + (size_t)t * md.nchunk;
    const int nvb = (nkept + 1) / 2;
    const int nunits = nvb * nkept;
    init_cta(sm);
    const uint32_t tmem = sm.tmem;

    if (warp == 0) {
        if (lane == 0) {
            for (int u = 0; u < nunits; u++) {
                const int vb = u / nkept, kc = u % nkept;
                const int s = u % kStages;
                const uint32_t ph = (u / kStages) & 1;
                if (sm.abort || !tc::mbar_wait(&sm.empty[s], ph ^ 1)) {
                    flag_timeout(err, &sm);
                    break;
                }
                uint8_t* st = stage_base(smem, s);
                tc::mbar_arrive_expect_tx(&sm.full[s], kStageBytes);
                for (int p = 0; p < 3; p++)
                    tc::tma_load_2d(st + p * kPlaneA, &tm_pf, kc * 64, (int)((acomp * 3 + p) * md.Gt + (long)t * 128),
                                    &sm.full[s]);
                const int gmu = chunks[kc];
                for (int p = 0; p < 3; p++)
                    for (int h = 0; h < 2; h++) {
                        const int vs = 2 * vb + h < nkept ? 2 * vb + h : nkept - 1;
                        tc::tma_load_2d(st + (3 + p) * kPlaneA + h * (kPlaneA / 2), &tm_d, gmu * 64,
                                        (spin * 3 + p) * md.npad + chunks[vs] * 64, &sm.full[s]);
                    }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            for (int u = 0; u < nunits; u++) {
                const int s = u % kStages, b = u & 1;
                const uint32_t ph = (u / kStages) & 1, bph = (u >> 1) & 1;
                if (sm.abort || !tc::mbar_wait(&sm.tempty[b], bph ^ 1) || !tc::mbar_wait(&sm.full[s], ph)) {
                    flag_timeout(err, &sm);
                    tc::mma_commit(&sm.tfull[b]);  // release the epilogue
                    break;
                }
                tc::fence_after_sync();
                mma_stage(tmem, b, stage_base(smem, s), true);
                tc::mma_commit(&sm.empty[s]);
                tc::mma_commit(&sm.tfull[b]);
            }
        }
    } else {
        // epilogue warps: row g of the tile
        const int quad = warp & 3;
        const int g = quad * 32 + lane;
        const long pt = (long)t * 128 + g;
        const bool live = pt < Gp;
        const size_t cs = (size_t)md.ntiles * md.kmax * 128;  // component stride of the FP32 store
        double acc_r = 0, acc_g0 = 0, acc_g1 = 0, acc_g2 = 0, acc_t = 0;
        float T[128];
#pragma unroll
        for (int j = 0; j < 128; j++) T[j] = 0.f;
        for (int u = 0; u < nunits; u++) {
            const int vb = u / nkept, kc = u % nkept, b = u & 1;
            const uint32_t bph = (u >> 1) & 1;
            if (sm.abort) break;
            if (!tc::mbar_wait(&sm.tfull[b], bph)) {
                flag_timeout(err, &sm);
                break;
            }
            tc::fence_after_sync();
            drain(tmem, b, quad, T);
            tc::fence_before_sync();
            mbar_arrive(&sm.tempty[b]);
            if (kc != nkept - 1) continue;
            // nu block complete: contract T with this row's AO values, read
            // from the function-major FP32 store (a warp reads 32 consecutive
            // points of one function: one 128-byte line per load)
            if (live && !sm.abort) {
                float pr = 0, pg0 = 0, pg1 = 0, pg2 = 0, pt_ = 0;
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int slot = 2 * vb + h;
                    if (slot >= nkept) break;
                    const float* e0 = md.e32 + ((size_t)t * md.kmax + slot * 64) * 128 + g;
#pragma unroll
                    for (int j = 0; j < 64; j++) {
                        const float tv = T[h * 64 + j];
                        const size_t o = (size_t)j * 128;
                        if (EPI <= 1) pr = fmaf(tv, __ldg(e0 + o), pr);
                        if (EPI == 1) {
                            pg0 = fmaf(tv, __ldg(e0 + cs + o), pg0);
                            pg1 = fmaf(tv, __ldg(e0 + 2 * cs + o), pg1);
                            pg2 = fmaf(tv, __ldg(e0 + 3 * cs + o), pg2);
                        }
                        if (EPI == 2) pt_ = fmaf(tv, __ldg(e0 + (size_t)acomp * cs + o), pt_);
                    }
                }
                acc_r += pr;
                acc_g0 += 2.0 * pg0;
                acc_g1 += 2.0 * pg1;
                acc_g2 += 2.0 * pg2;
                acc_t += 0.5 * pt_;
            }
#pragma unroll
            for (int j = 0; j < 128; j++) T[j] = 0.f;
        }
        if (live) {
            if (EPI <= 1) rho[(long)spin * Gp + pt] = acc_r;
            if (EPI == 1) {
                rho1[((long)spin * 3 + 0) * Gp + pt] = acc_g0;
                rho1[((long)spin * 3 + 1) * Gp + pt] = acc_g1;
                rho1[((long)spin * 3 + 2) * Gp + pt] = acc_g2;
            }
            if (EPI == 2) tau[(long)spin * Gp + pt] += acc_t;
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, kTmemCols);
}

// ------------------------------------------------------------- V_xc
// One CTA per (128 x 128 block (I, J) of W, split of tiles):
//   W_IJ = sum_t sum_c L_c,t[I]^T R_c,t[J]   (unit = one point tile, K = 128 points per component)
__global__ void __launch_bounds__(kThreads, 1) fock_tc_kernel(const __grid_constant__ CUtensorMap tm_fp,
                                                              const __grid_constant__ CUtensorMap tm_r, MixedDev md,
                                                              int ncomp, int r_rows, int nblk, int nsplit,
                                                              double* __restrict__ wpart, int* err) {
    extern __shared__ uint8_t smem_raw[];
    __shared__ Smem sm;
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const int I = blockIdx.x / nblk, J = blockIdx.x % nblk;
    const int split = blockIdx.y;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int t0 = (int)((long)md.ntiles * split / nsplit), t1 = (int)((long)md.ntiles * (split + 1) / nsplit);
    const long TK = (long)md.ntiles * md.kmax;
    const int zero_row = (int)(12 * TK);  // 64 zero rows after the FP planes
    const int zero_row_r = r_rows;        // 64 zero rows after the R planes
    init_cta(sm);
    const uint32_t tmem = sm.tmem;

    auto slot_of = [&](int t, int chunk) -> int {
        return chunk < md.nchunk ? md.tile_slot[(size_t)t * md.nchunk + chunk] : -1;
    };
    auto wanted = [&](int t) {
        return (slot_of(t, 2 * I) >= 0 || slot_of(t, 2 * I + 1) >= 0) &&
               (slot_of(t, 2 * J) >= 0 || slot_of(t, 2 * J + 1) >= 0);
    };

    if (warp == 0) {
        if (lane == 0) {
            uint32_t i2 = 0;
            for (int t = t0; t < t1 && !sm.abort; t++) {
                if (!wanted(t)) continue;
                const int sa0 = slot_of(t, 2 * I), sa1 = slot_of(t, 2 * I + 1);
                const int sb0 = slot_of(t, 2 * J), sb1 = slot_of(t, 2 * J + 1);
                for (int c = 0; c < ncomp && !sm.abort; c++)
                    for (int kh = 0; kh < 2; kh++, i2++) {
                        const int s = i2 % kStages;
                        const uint32_t ph = (i2 / kStages) & 1;
                        if (sm.abort || !tc::mbar_wait(&sm.empty[s], ph ^ 1)) {
                            flag_timeout(err, &sm);
                            break;
                        }
                        uint8_t* st = stage_base(smem, s);
                        tc::mbar_arrive_expect_tx(&sm.full[s], kStageBytes);
                        for (int p = 0; p < 3; p++)
                            for (int h = 0; h < 2; h++) {
                                const int sa = h ? sa1 : sa0, sb = h ? sb1 : sb0;
                                const long rbase = (long)(c * 3 + p) * TK + (long)t * md.kmax;
                                const int ra = sa >= 0 ? (int)(rbase + sa * 64) : zero_row;
                                const int rb = sb >= 0 ? (int)(rbase + sb * 64) : zero_row_r;
                                tc::tma_load_2d(st + p * kPlaneA + h * (kPlaneA / 2), &tm_fp, kh * 64, ra, &sm.full[s]);
                                tc::tma_load_2d(st + (3 + p) * kPlaneA + h * (kPlaneA / 2), &tm_r, kh * 64, rb,
                                                &sm.full[s]);
                            }
                    }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            uint32_t i2 = 0, u = 0;
            for (int t = t0; t < t1 && !sm.abort; t++) {
                if (!wanted(t)) continue;
                const int b = u & 1;
                const uint32_t bph = (u >> 1) & 1;
                if (!tc::mbar_wait(&sm.tempty[b], bph ^ 1)) {
                    flag_timeout(err, &sm);
                    tc::mma_commit(&sm.tfull[b]);
                    break;
                }
                bool first = true;
                for (int c = 0; c < ncomp; c++)
                    for (int kh = 0; kh < 2; kh++, i2++) {
                        const int s = i2 % kStages;
                        const uint32_t ph = (i2 / kStages) & 1;
                        if (sm.abort || !tc::mbar_wait(&sm.full[s], ph)) {
                            flag_timeout(err, &sm);
                            break;
                        }
                        tc::fence_after_sync();
                        mma_stage(tmem, b, stage_base(smem, s), first);
                        first = false;
                        tc::mma_commit(&sm.empty[s]);
                    }
                tc::mma_commit(&sm.tfull[b]);
                u++;
            }
        }
    } else {
        const int quad = warp & 3;
        const int g = quad * 32 + lane;  // row of the W block
        float W[128];
#pragma unroll
        for (int j = 0; j < 128; j++) W[j] = 0.f;
        uint32_t u = 0;
        bool any = false;
        for (int t = t0; t < t1; t++) {
            if (!wanted(t)) continue;
            const int b = u & 1;
            const uint32_t bph = (u >> 1) & 1;
            if (sm.abort) break;
            if (!tc::mbar_wait(&sm.tfull[b], bph)) {
                flag_timeout(err, &sm);
                break;
            }
            if (sm.abort) break;
            tc::fence_after_sync();
            drain(tmem, b, quad, W);
            tc::fence_before_sync();
            mbar_arrive(&sm.tempty[b]);
            any = true;
            u++;
        }
        const int npadw = nblk * 128;
        double* out = wpart + (size_t)split * npadw * npadw + (size_t)(I * 128 + g) * npadw + J * 128;
#pragma unroll
        for (int j = 0; j < 128; j++) out[j] = (any && !sm.abort) ? (double)W[j] : 0.0;
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, kTmemCols);
}

// out = a * x + b * y (FP64, n elements).
__global__ void axpby_kernel(long n, double a, const double* __restrict__ x, double b, const double* __restrict__ y,
                             double* __restrict__ out) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = a * x[i] + b * y[i];
}

// V(mu, nu) = sum_s W_s(mu, nu) + W_s(nu, mu), column-major n x n (FP64).
__global__ void wsum_kernel(const double* __restrict__ wpart, int nsplit, int npadw, int n, double* __restrict__ V) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)n * n) return;
    const int mu = (int)(idx % n), nu = (int)(idx / n);
    double acc = 0;
    for (int s = 0; s < nsplit; s++) {
        const double* w = wpart + (size_t)s * npadw * npadw;
        acc += w[(size_t)mu * npadw + nu] + w[(size_t)nu * npadw + mu];
    }
    V[(long)nu * n + mu] = acc;
}

// D (s, n, n) column-major FP64 -> three BF16 planes per spin, row nu, col mu.
__global__ void split_d_kernel(const double* __restrict__ D, int n, int npad, int nspin, bf16* __restrict__ Dp) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long total = (long)nspin * npad * npad;
    if (idx >= total) return;
    const int mu = (int)(idx % npad);
    const int nu = (int)((idx / npad) % npad);
    const int s = (int)(idx / ((long)npad * npad));
    const double v = (mu < n && nu < n) ? D[(long)s * n * n + (long)nu * n + mu] : 0.0;
    bf16 h, m, l;
    tc::split3(v, h, m, l);
    const size_t plane = (size_t)npad * npad;
    Dp[(size_t)(s * 3 + 0) * plane + (size_t)nu * npad + mu] = h;
    Dp[(size_t)(s * 3 + 1) * plane + (size_t)nu * npad + mu] = m;
    Dp[(size_t)(s * 3 + 2) * plane + (size_t)nu * npad + mu] = l;
}

// R operand: comp 0 = c0 phi + c1 . grad phi, comps 1..3 = c2 d_r phi (meta-GGA).
__global__ void prep_r_kernel(MixedDev md, int ncomp, int type, const double* __restrict__ fcoef, long Gp,
                              bf16* __restrict__ R) {
    const long TK = (long)md.ntiles * md.kmax;
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;  // over TK * 128
    if (idx >= TK * 128) return;
    const int g = (int)(idx & 127);
    const long row = idx >> 7;  // t * kmax + slot*64 + f
    const int t = (int)(row / md.kmax);
    const int colslot = (int)(row % md.kmax);
    const long pt = (long)t * 128 + g;
    if (colslot >= md.tile_nkept[t] * 64 || pt >= Gp) {
        for (int c = 0; c < ncomp; c++)
            for (int p = 0; p < 3; p++) R[((size_t)(c * 3 + p) * TK + row) * 128 + g] = __float2bfloat16(0.f);
        return;
    }
    // FP32 arithmetic: R carries ~2^-24 relative precision in its three planes
    auto fpv = [&](int c) { return __ldg(md.e32 + ((size_t)c * TK + row) * 128 + g); };
    const float phi = fpv(0);
    float a = (float)fcoef[pt] * phi;
    float d[3] = {0, 0, 0};
    if (type >= 1) {
        for (int r = 0; r < 3; r++) d[r] = fpv(1 + r);
        a = fmaf((float)fcoef[Gp + pt], d[0], a);
        a = fmaf((float)fcoef[2 * Gp + pt], d[1], a);
        a = fmaf((float)fcoef[3 * Gp + pt], d[2], a);
    }
    bf16 h, m, l;
    tc::split3f(a, h, m, l);
    const size_t ps = (size_t)TK * 128;
    R[row * 128 + g] = h;
    R[ps + row * 128 + g] = m;
    R[2 * ps + row * 128 + g] = l;
    if (ncomp == 4) {
        const float c2 = (float)fcoef[4 * Gp + pt];
        for (int r = 0; r < 3; r++) {
            tc::split3f(c2 * d[r], h, m, l);
            R[((size_t)((1 + r) * 3 + 0) * TK + row) * 128 + g] = h;
            R[((size_t)((1 + r) * 3 + 1) * TK + row) * 128 + g] = m;
            R[((size_t)((1 + r) * 3 + 2) * TK + row) * 128 + g] = l;
        }
    }
}

// AO values and gradients of every mixed tile in both layouts, FP64 then
// split.  One CTA per tile, thread = point; loops over the tile's shells.
constexpr int kNcart = (kMaxL + 1) * (kMaxL + 2) / 2;

__global__ void __launch_bounds__(128) ao_mixed_kernel(MixedDev md, DevShells sh, const int* __restrict__ tile_shells,
                                                       const int* __restrict__ tile_shell_off,
                                                       const double* __restrict__ px, const double* __restrict__ py,
                                                       const double* __restrict__ pz, long Gp,
                                                       const double* __restrict__ shtab, bf16* __restrict__ pf,
                                                       bf16* __restrict__ fp, float* __restrict__ e32) {
    const int t = blockIdx.x, g = threadIdx.x;
    const long pt = (long)t * 128 + g;
    const long src = pt < Gp ? pt : 0;  // tail points: copies of point 0 (their weight is zero)
    const double X = px[src], Y = py[src], Z = pz[src];
    const long TK = (long)md.ntiles * md.kmax;
    const int* slots = md.tile_slot + (size_t)t * md.nchunk;
    for (int k = tile_shell_off[t]; k < tile_shell_off[t + 1]; k++) {
        const int s = tile_shells[k];
        const int l = sh.l[s], type = sh.type[s], np = sh.nprim[s], po = sh.prim_off[s], first = sh.first[s];
        const double x = X - sh.xyz[3 * s], y = Y - sh.xyz[3 * s + 1], z = Z - sh.xyz[3 * s + 2];
        const double r2 = x * x + y * y + z * z;
        double t0 = 0, t1 = 0;
        for (int p = 0; p < np; p++) {
            const double e = sh.exps[po + p];
            const double v = sh.coefs[po + p] * exp(-e * r2);
            t0 += v;
            t1 += v * e;
        }
        const double A = t0, Ax = -2 * x * t1, Ay = -2 * y * t1, Az = -2 * z * t1;
        double xp[kMaxL + 1], yp[kMaxL + 1], zp[kMaxL + 1];
        xp[0] = yp[0] = zp[0] = 1;
        for (int i = 1; i <= l; i++) {
            xp[i] = xp[i - 1] * x;
            yp[i] = yp[i - 1] * y;
            zp[i] = zp[i - 1] * z;
        }
        for (int f = 0; f < 2 * l + 1; f++) {
            const int mu = first + f;
            const int slot = slots[mu >> 6];
            if (slot < 0) continue;
            const int row = (type == 1) ? (f == 0 ? 2 : f - 1) : f;
            double Q = 0, Qx = 0, Qy = 0, Qz = 0;
            int kk = 0;
            for (int a = l; a >= 0; a--)
                for (int b = l - a; b >= 0; b--, kk++) {
                    const double c = shtab[(l * (2 * kMaxL + 1) + row) * kNcart + kk];
                    if (c == 0) continue;
                    const int cc = l - a - b;
                    Q += c * xp[a] * yp[b] * zp[cc];
                    if (a) Qx += c * a * xp[a - 1] * yp[b] * zp[cc];
                    if (b) Qy += c * b * xp[a] * yp[b - 1] * zp[cc];
                    if (cc) Qz += c * cc * xp[a] * yp[b] * zp[cc - 1];
                }
            const double vals[4] = {A * Q, Ax * Q + A * Qx, Ay * Q + A * Qy, Az * Q + A * Qz};
            const int col = slot * 64 + (mu & 63);
            for (int c = 0; c < 4; c++) {
                bf16 h[3];
                tc::split3(vals[c], h[0], h[1], h[2]);
                for (int p = 0; p < 3; p++) {
                    pf[((size_t)(c * 3 + p) * md.Gt + pt) * md.kmax + col] = h[p];
                    fp[((size_t)(c * 3 + p) * TK + (size_t)t * md.kmax + col) * 128 + g] = h[p];
                }
                e32[((size_t)c * TK + (size_t)t * md.kmax + col) * 128 + g] = (float)vals[c];
            }
        }
    }
}

}  // namespace

void launch_ao_mixed(const MixedDev& md, DevShells sh, const int* tile_shells, const int* tile_shell_off, const double* x,
                     const double* y, const double* z, long Gp, const double* shtab, bf16* pf, bf16* fp, float* e32,
                     cudaStream_t s) {
    ao_mixed_kernel<<<md.ntiles, 128, 0, s>>>(md, sh, tile_shells, tile_shell_off, x, y, z, Gp, shtab, pf, fp, e32);
    CGB_CUDA(cudaGetLastError());
}

void launch_split_d(const double* D, int n, int npad, int nspin, bf16* Dp, cudaStream_t s) {
    const long total = (long)nspin * npad * npad;
    split_d_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(D, n, npad, nspin, Dp);
    CGB_CUDA(cudaGetLastError());
}

size_t mixed_smem_bytes() { return (size_t)kStages * kStageBytes + 1024; }

void launch_density_tc(const CUtensorMap& tm_pf, const CUtensorMap& tm_d, const MixedDev& md, int epi, int acomp,
                       int spin, double* rho, double* rho1, double* tau, long Gp, int* err, cudaStream_t s) {
    const size_t smem = mixed_smem_bytes();
    if (epi == 0) {
        CGB_CUDA(cudaFuncSetAttribute(density_tc_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        density_tc_kernel<0><<<md.ntiles, kThreads, smem, s>>>(tm_pf, tm_d, md, acomp, spin, rho, rho1, tau, Gp, err);
    } else if (epi == 1) {
        CGB_CUDA(cudaFuncSetAttribute(density_tc_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        density_tc_kernel<1><<<md.ntiles, kThreads, smem, s>>>(tm_pf, tm_d, md, acomp, spin, rho, rho1, tau, Gp, err);
    } else {
        CGB_CUDA(cudaFuncSetAttribute(density_tc_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        density_tc_kernel<2><<<md.ntiles, kThreads, smem, s>>>(tm_pf, tm_d, md, acomp, spin, rho, rho1, tau, Gp, err);
    }
    CGB_CUDA(cudaGetLastError());
}

void launch_prep_r(const MixedDev& md, int ncomp, int type, const double* fcoef, long Gp, bf16* R, cudaStream_t s) {
    const long total = (long)md.ntiles * md.kmax * 128;
    prep_r_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(md, ncomp, type, fcoef, Gp, R);
    CGB_CUDA(cudaGetLastError());
}

void launch_fock_tc(const CUtensorMap& tm_fp, const CUtensorMap& tm_r, const MixedDev& md, int ncomp, int r_rows,
                    int nblk, int nsplit, double* wpart, int* err, cudaStream_t s) {
    const size_t smem = mixed_smem_bytes();
    CGB_CUDA(cudaFuncSetAttribute(fock_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid(nblk * nblk, nsplit);
    fock_tc_kernel<<<grid, kThreads, smem, s>>>(tm_fp, tm_r, md, ncomp, r_rows, nblk, nsplit, wpart, err);
    CGB_CUDA(cudaGetLastError());
}

void launch_axpby(long n, double a, const double* x, double b, const double* y, double* out, cudaStream_t s) {
    if (n <= 0) return;
    axpby_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, a, x, b, y, out);
    CGB_CUDA(cudaGetLastError());
}

void launch_wsum(const double* wpart, int nsplit, int npadw, int n, double* V, cudaStream_t s) {
    const long total = (long)n * n;
    wsum_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(wpart, nsplit, npadw, n, V);
    CGB_CUDA(cudaGetLastError());
}

}  // namespace cgb
