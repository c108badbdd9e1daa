// Mixed-precision XC contractions on the 5th-generation tensor cores.
//
// Points are grouped into tiles of 128 (spatially compact, one molecule per
// tile); each tile keeps the 64-function chunks of its molecule that the
// screening test marks significant, packed into "slots".  The AO values and
// gradients are stored once, in FP32, function-major (one 512-byte row of
// 128 points per kept function).  Operands reach tcgen05.mma as three-term
// BF16 planes (x = h + m + l, exact for an FP32 x) in the 128-byte-swizzled
// layout, in one of two forms:
//   pre-split (density16_kernel, fock16_kernel): the planes are split once in
//     HBM (split_store_kernel for the AO store, prep16_kernel per build for
//     the V kernel's R operand) and TMA loads them straight into the stages;
//   in-kernel split (density_tc_kernel, fock_tc_kernel): TMA stages FP32
//     tiles in shared memory and converter warps split them (transposing on
//     the way for the density product) — 1.5x less HBM, used when the planes
//     do not fit.
// A product sums the six cross terms of order <= 2 (hh, hm, mh, hl, mm, lh)
// in FP32; hh and the five corrections go to separate TMEM accumulators, and
// every accumulation unit starts fresh and is drained by the epilogue warps
// into round-to-nearest FP32 registers.  Cross-unit sums of the final
// quantities are FP64.
//
// HBM layouts:
//   e32 (FP32): component c (phi, d/dx, d/dy, d/dz), row c*rows + tile_row[t] + slot*64 + f, col g (128 points)
//   e16 (BF16): row (c*3 + p)*rows + (the e32 row within component c), p = h, m, l
//   R16 (BF16, per build): row (c*3 + p)*rows + ..., c = 0: Z, c = 1..3: c2 d_c phi (meta-GGA)
//   Z   (FP32, per build, in-kernel split): c0 phi + c1 . grad phi, same rows as e32 component 0
//   Dp  (BF16 density planes): row (s*3+p)*drows + f0(mol) + nu, col mu
//
// The tensor-core kernels are persistent: one CTA per SM walks a host-made
// list of work items (tiles, or (I, J, tile range) blocks of V) balanced by
// cost.  Roles: warp 0 issues every TMA load and owns TMEM, warp 1 issues
// tcgen05.mma into one of two TMEM buffers (256 columns each: hh |
// corrections), warps 4-11 drain TMEM (lane quadrant = warp % 4; warps 4-7
// columns 0-63, warps 8-11 columns 64-127) and run the epilogue; the
// in-kernel-split kernels (512 threads) add converter warps (2-3 and 12-15,
// and for V also 4-11), the pre-split ones run 384 threads.  Shared memory:
// pre-split = two 96 KB operand stages; in-kernel split (224 KB): density =
// two operand stages + one raw FP32 tile, V_xc = one operand stage + a ring
// of raw FP32 half-stages.  Every wait is bounded (2 s of %globaltimer); a
// timeout sets XC_ERR_TIMEOUT in a global flag and the CTA unwinds instead
// of hanging.
#include <cstdio>

#include "common.h"
#include "kernels.h"
#include "mixed.h"
#include "tc.cuh"

namespace cgb {
namespace {

using bf16 = __nv_bfloat16;

constexpr int kThreads = 512;
constexpr int kF16Threads = 384;               // kernels on pre-split operands: no converter warps
constexpr int kEpiWarp0 = 4;                   // epilogue warps 4-11 (two per TMEM lane quadrant)
constexpr int kEpiThreads = 256;
constexpr int kConvWarps = 6;                  // warps 2-3 and 12-15
constexpr uint32_t kPlaneA = 128 * 64 * 2;     // bytes of one 128x64 bf16 operand plane
constexpr uint32_t kStageBytes = 6 * kPlaneA;  // A (3 planes) + B (3 planes)
constexpr uint32_t kRawD = 64 * 128 * 4;       // density raw tile: 64 functions x 128 points FP32
constexpr uint32_t kRawBox = 64 * 32 * 4;      // V_xc raw box: 64 functions x 32 points FP32
constexpr uint32_t kRawF = 4 * kRawBox;        // V_xc raw half-stage: L (2 boxes) + R (2 boxes)
constexpr int kRawSlots = 4;                   // V_xc raw ring
constexpr uint32_t kSmemBytes = 2 * kStageBytes + kRawD;  // = kStageBytes + kRawSlots * kRawF
static_assert(2 * kStageBytes + kRawD == kStageBytes + kRawSlots * kRawF, "shared-memory plans differ");
constexpr uint32_t kIdesc = tc::idesc_bf16(128, 128);
constexpr uint32_t kTmemCols = 512;            // 2 buffers x (hh 128 | corrections 128)
// cross terms (i, j) of the three-term splits with i + j <= 2; term 0 is hh
__constant__ int c_prod_a[6] = {0, 0, 1, 0, 1, 2};
__constant__ int c_prod_b[6] = {0, 1, 0, 2, 1, 0};

struct Smem {
    uint64_t full[2];
    uint64_t empty[2];
    uint64_t rfull[4];
    uint64_t rempty[4];
    uint64_t tfull[2];
    uint64_t tempty[2];
    uint32_t tmem;
    int abort;
};

__device__ __forceinline__ int conv_index() {
    const int w = threadIdx.x >> 5;
    return w < kEpiWarp0 ? w - 2 : w - 10;  // warps 2, 3 -> 0, 1; warps 12..15 -> 2..5
}

__device__ __forceinline__ void flag_timeout(int* err, Smem* sm) {
    atomicExch(err, XC_ERR_TIMEOUT);
    atomicExch(&sm->abort, 1);
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_u32(bar)) : "memory");
}

__device__ void init_cta(Smem& sm, uint32_t full_count, uint32_t rempty_count) {
    if (threadIdx.x == 0) {
        for (int s = 0; s < 2; s++) {
            tc::mbar_init(&sm.full[s], full_count);
            tc::mbar_init(&sm.empty[s], 1);
            tc::mbar_init(&sm.tfull[s], 1);
            tc::mbar_init(&sm.tempty[s], kEpiThreads);
        }
        for (int s = 0; s < 4; s++) {
            tc::mbar_init(&sm.rfull[s], 1);
            tc::mbar_init(&sm.rempty[s], rempty_count);
        }
        sm.abort = 0;
        tc::fence_mbar_init();
    }
    if ((threadIdx.x >> 5) == 0) tc::tmem_alloc(&sm.tmem, kTmemCols);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
}

// A converter warp waits (lane 0, bounded) for a barrier phase; all lanes
// learn the outcome.
__device__ __forceinline__ bool warp_wait(Smem& sm, uint64_t* bar, uint32_t parity, int* err) {
    int ok = 1;
    if ((threadIdx.x & 31) == 0) {
        ok = !sm.abort && tc::mbar_wait(bar, parity);
        if (!ok) flag_timeout(err, &sm);
    }
    return __shfl_sync(0xffffffffu, ok, 0) != 0;
}

// One arrival per warp once every lane is done.
__device__ __forceinline__ void warp_arrive(uint64_t* bar) {
    __syncwarp();
    if ((threadIdx.x & 31) == 0) mbar_arrive(bar);
}

// The converted planes of this warp are complete: make them visible to the
// tensor core (async proxy) and arrive once per warp on the stage.
__device__ __forceinline__ void conv_publish(uint64_t* full) {
    tc::fence_proxy_async();
    warp_arrive(full);
}

// Three-term split of 8 consecutive K-elements into one 16-byte chunk per plane
// (round to nearest at each term; the residuals in packed FP32x2 arithmetic).
__device__ __forceinline__ void split8(const float* v, uint4& h, uint4& m, uint4& l) {
    uint32_t hh[4], mm[4], ll[4];
    const float2 neg1 = make_float2(-1.f, -1.f);
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const float2 a = make_float2(v[2 * k], v[2 * k + 1]);
        const __nv_bfloat162 H = __floats2bfloat162_rn(a.x, a.y);
        const float2 r = __ffma2_rn(__bfloat1622float2(H), neg1, a);  // a - H, exact
        const __nv_bfloat162 Mv = __floats2bfloat162_rn(r.x, r.y);
        const float2 r2 = __ffma2_rn(__bfloat1622float2(Mv), neg1, r);
        const __nv_bfloat162 Lv = __floats2bfloat162_rn(r2.x, r2.y);
        hh[k] = *reinterpret_cast<const uint32_t*>(&H);
        mm[k] = *reinterpret_cast<const uint32_t*>(&Mv);
        ll[k] = *reinterpret_cast<const uint32_t*>(&Lv);
    }
    h = make_uint4(hh[0], hh[1], hh[2], hh[3]);
    m = make_uint4(mm[0], mm[1], mm[2], mm[3]);
    l = make_uint4(ll[0], ll[1], ll[2], ll[3]);
}

// Store chunk j (8 K-elements) of row r of an operand (three planes from
// `planes`) in the 128-byte-swizzled K-major layout.
__device__ __forceinline__ void store_chunk(uint32_t planes, int r, int j, const float* v) {
    uint4 h, m, l;
    split8(v, h, m, l);
    const uint32_t off = (uint32_t)r * 128u + ((uint32_t)(j ^ (r & 7)) << 4);
    tc::sts128(planes + off, h);
    tc::sts128(planes + kPlaneA + off, m);
    tc::sts128(planes + 2 * kPlaneA + off, l);
}

// The same for a K range that shares one fixed-point exponent e
// (tc::split3_fixed_f).
__device__ __forceinline__ void store_chunk_fixed(uint32_t planes, int r, int j, const float* v, int e) {
    uint32_t hh[4], mm[4], ll[4];
#pragma unroll
    for (int k = 0; k < 4; k++) tc::split3_fixed_f2(make_float2(v[2 * k], v[2 * k + 1]), e, hh[k], mm[k], ll[k]);
    const uint32_t off = (uint32_t)r * 128u + ((uint32_t)(j ^ (r & 7)) << 4);
    tc::sts128(planes + off, make_uint4(hh[0], hh[1], hh[2], hh[3]));
    tc::sts128(planes + kPlaneA + off, make_uint4(mm[0], mm[1], mm[2], mm[3]));
    tc::sts128(planes + 2 * kPlaneA + off, make_uint4(ll[0], ll[1], ll[2], ll[3]));
}

// The six split products of one stage into TMEM buffer `buf`: term hh into
// the hh accumulator, the five corrections into the correction accumulator.
// `first` starts both accumulators (unit boundary).
// `halve` (V kernel, items with c2 doubled): the first product into each
// accumulator halves it (D = A B + D / 2); the drain doubles the unit.
// A_MN: the A planes are MN-major (two 64-row TMA boxes of a [K][M] array,
// 8 KB apart), as the pre-split density kernel stages them.
template <bool A_MN = false>
__device__ __forceinline__ void mma_stage(uint32_t tmem, int buf, uint8_t* st, bool first, bool halve = false) {
    const uint32_t a0 = tc::smem_u32(st), b0 = a0 + 3 * kPlaneA;
    const uint32_t d_hh = tmem + buf * 256, d_corr = tmem + buf * 256 + 128;
    constexpr uint32_t idesc = A_MN ? tc::idesc_bf16_amn(128, 128) : kIdesc;
#pragma unroll
    for (int q = 0; q < 6; q++) {
        const uint32_t pa = a0 + c_prod_a[q] * kPlaneA;
        const uint64_t bd = tc::smem_desc_sw128(b0 + c_prod_b[q] * kPlaneA);
        const uint32_t d = q == 0 ? d_hh : d_corr;
#pragma unroll
        for (int k = 0; k < 4; k++) {  // K = 16 per instruction: +32 bytes in a K-major row, +2048 MN-major
            const uint64_t ad = A_MN ? tc::smem_desc_sw128_mn(pa + k * 2048, kPlaneA / 2) : tc::smem_desc_sw128(pa) + 2 * k;
            const bool lead = k == 0 && (q == 0 || q == 1);
            if (halve && lead)
                tc::mma_bf16_halve_d(d, ad, bd + 2 * k, idesc);
            else
                tc::mma_bf16(d, ad, bd + 2 * k, idesc, (first && lead) ? 0u : 1u);
        }
    }
}

// Drain columns half*64 .. half*64 + 63 of TMEM buffer `buf` (hh +
// corrections) into acc[64] (this thread's lane).
__device__ __forceinline__ void drain(uint32_t tmem, int buf, int quad, int half, float* acc, float w = 1.f) {
    const uint32_t base = tmem + ((uint32_t)(quad * 32) << 16) + buf * 256 + half * 64;
#pragma unroll
    for (int c16 = 0; c16 < 4; c16++) {
        float a[16], b[16];
        tc::tmem_ld16x2_nomem(base + c16 * 16, base + 128 + c16 * 16, a, b);
#pragma unroll
        for (int j = 0; j < 16; j++) acc[c16 * 16 + j] += w * (a[j] + b[j]);
    }
}

// ------------------------------------------------------------ density
// T = Phi D for one tile, unit = (nu block vb of two slots, mu chunk kc).
// Every unit starts fresh TMEM accumulators (hh | corrections); the
// epilogue warps drain each unit into round-to-nearest FP32 registers (T,
// 64 columns per thread) and, at the end of a nu block, contract T with the
// AO values of their slot.  The two column halves of a row write separate
// partial outputs (rho / rho_b ...), summed by combine_kernel.
// EPI 0: rho; 1: rho + grad rho; 2: tau contribution of A component acomp.
// rho and tau are symmetric in (mu, nu): their nu block vb only takes mu
// chunks from its own first slot on, and units of later chunks count twice
// (the mirrored pairs of later nu blocks are skipped).  grad rho is not.

// Position in the density unit sequence of one CTA (host-made job list).
struct DensCursor {
    int j, end, vb, kc;
    bool sym;
    DensJob job;
    __device__ void load(const DensJob* jobs) {
        const int4 r = __ldg(reinterpret_cast<const int4*>(jobs) + j);
        job.t = r.x;
        job.nk = r.y;
        job.trow = r.z;
        job.c0 = r.w;
    }
    __device__ DensCursor(const int* off, const DensJob* jobs, bool symmetric) {
        j = off[blockIdx.x];
        end = off[blockIdx.x + 1];
        vb = kc = 0;
        sym = symmetric;
        job = DensJob{0, 1, 0, 0};
        if (j < end) load(jobs);
    }
    __device__ bool valid() const { return j < end; }
    __device__ int nvb() const { return (job.nk + 1) / 2; }
    // weight of the current unit in T (exact in FP32)
    __device__ float weight() const { return (sym && kc >= 2 * vb + 2) ? 2.f : 1.f; }
    __device__ void advance(const DensJob* jobs) {
        if (++kc < job.nk) return;
        if (++vb < nvb()) {
            kc = sym ? 2 * vb : 0;
            return;
        }
        vb = kc = 0;
        if (++j < end) load(jobs);
    }
};

constexpr int kMaxChunks = 256;                                       // chunks of one molecule (n <= 16384)

struct DensOut {
    double *rho, *rho1, *tau;  // column half 0
    double *rho_b, *rho1_b, *tau_b;  // column half 1
};

// Epilogue warps 4-11 of both density kernels: row g of the tile, columns
// of slot 2 vb + half.
template <int EPI>
__device__ __forceinline__ void density_epilogue(Smem& sm, uint32_t tmem, const MixedDev& md, const int* job_off,
                                                 const DensJob* jobs, int acomp, int spin, const DensOut& out, int* err,
                                                 int warp, int lane) {
    const long Gt = md.Gt;
    const int quad = warp & 3, half = (warp - kEpiWarp0) >> 2;
    const int g = quad * 32 + lane;
    const size_t cs = (size_t)md.rows * 128;  // component stride of the FP32 store
    double* rho = half ? out.rho_b : out.rho;
    double* rho1 = half ? out.rho1_b : out.rho1;
    double* tau = half ? out.tau_b : out.tau;
    float T[64];
#pragma unroll
    for (int j = 0; j < 64; j++) T[j] = 0.f;
    double acc_r = 0, acc_g0 = 0, acc_g1 = 0, acc_g2 = 0, acc_t = 0;
    uint32_t uu = 0;
    for (DensCursor c(job_off, jobs, EPI != 1); c.valid(); c.advance(jobs), uu++) {
        const int b = uu & 1;
        if (sm.abort) break;
        if (!tc::mbar_wait(&sm.tfull[b], (uu >> 1) & 1)) {
            flag_timeout(err, &sm);
            break;
        }
        tc::fence_after_sync();
        drain(tmem, b, quad, half, T, c.weight());
        tc::fence_before_sync();
        mbar_arrive(&sm.tempty[b]);
        if (c.kc != c.job.nk - 1) continue;
        // nu block complete: contract T with this row's AO values of the
        // slot (a warp reads 32 consecutive points of one function: one
        // 128-byte line per load)
        const int slot = 2 * c.vb + half;
        if (slot < c.job.nk && !sm.abort) {
            float pr = 0, pg0 = 0, pg1 = 0, pg2 = 0, pt_ = 0;
            const float* e0 = md.e32 + ((size_t)c.job.trow + slot * 64) * 128 + g;
#pragma unroll
            for (int j = 0; j < 64; j++) {
                const float tv = T[j];
                const size_t o = (size_t)j * 128;
                // streaming loads (evict-first): each value is read once per build,
                // and the L2 keeps the operand planes that are re-read
                if (EPI <= 1) pr = fmaf(tv, __ldcs(e0 + o), pr);
                if (EPI == 1) {
                    pg0 = fmaf(tv, __ldcs(e0 + cs + o), pg0);
                    pg1 = fmaf(tv, __ldcs(e0 + 2 * cs + o), pg1);
                    pg2 = fmaf(tv, __ldcs(e0 + 3 * cs + o), pg2);
                }
                if (EPI == 2) pt_ = fmaf(tv, __ldcs(e0 + (size_t)acomp * cs + o), pt_);
            }
            acc_r += pr;
            acc_g0 += 2.0 * pg0;
            acc_g1 += 2.0 * pg1;
            acc_g2 += 2.0 * pg2;
            acc_t += 0.5 * pt_;
        }
#pragma unroll
        for (int j = 0; j < 64; j++) T[j] = 0.f;
        if (c.vb == c.nvb() - 1) {  // tile complete
            const long pt = (long)c.job.t * 128 + g;
            if (EPI <= 1) rho[(long)spin * Gt + pt] = acc_r;
            if (EPI == 1) {
                rho1[((long)spin * 3 + 0) * Gt + pt] = acc_g0;
                rho1[((long)spin * 3 + 1) * Gt + pt] = acc_g1;
                rho1[((long)spin * 3 + 2) * Gt + pt] = acc_g2;
            }
            if (EPI == 2) tau[(long)spin * Gt + pt] += acc_t;
            acc_r = acc_g0 = acc_g1 = acc_g2 = acc_t = 0;
        }
    }
}

template <int EPI>
__global__ void __launch_bounds__(kThreads, 1) density_tc_kernel(const __grid_constant__ CUtensorMap tm_d,
                                                                 const __grid_constant__ CUtensorMap tm_raw, MixedDev md,
                                                                 const int* __restrict__ job_off,
                                                                 const DensJob* __restrict__ jobs, int acomp, int spin,
                                                                 DensOut out, int* err) {
    extern __shared__ uint8_t smem_raw[];
    __shared__ Smem sm;
    __shared__ int s_chunks[kMaxChunks];
    uint8_t* smem = smem_raw + (((tc::smem_u32(smem_raw) + 1023u) & ~1023u) - tc::smem_u32(smem_raw));
    const uint32_t ssm = tc::smem_u32(smem);
    uint8_t* raw = smem + 2 * kStageBytes;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    init_cta(sm, 1 + kConvWarps, kConvWarps);
    const uint32_t tmem = sm.tmem;

    if (warp == 0) {
        if (lane == 0) {
            uint32_t uu = 0;
            for (DensCursor c(job_off, jobs, EPI != 1); c.valid(); c.advance(jobs), uu++) {
                if (c.vb == 0 && c.kc == 0) {  // new tile: its kept chunk ids
                    const int* src = md.tile_chunks + (size_t)c.job.t * md.nchunk;
                    for (int k = 0; k < c.job.nk; k++) s_chunks[k] = __ldg(src + k);
                }
                // raw Phi tile (one buffer)
                if (sm.abort || !tc::mbar_wait(&sm.rempty[0], (uu & 1) ^ 1)) {
                    flag_timeout(err, &sm);
                    break;
                }
                tc::mbar_arrive_expect_tx(&sm.rfull[0], kRawD);
                tc::tma_load_2d(raw, &tm_raw, 0, (int)((long)acomp * md.rows + c.job.trow + (long)c.kc * 64),
                                &sm.rfull[0]);
                // density planes into the stage
                const int s = uu & 1;
                if (sm.abort || !tc::mbar_wait(&sm.empty[s], ((uu >> 1) & 1) ^ 1)) {
                    flag_timeout(err, &sm);
                    break;
                }
                uint8_t* st = smem + (size_t)s * kStageBytes;
                tc::mbar_arrive_expect_tx(&sm.full[s], 3 * kPlaneA);
                const int gmu = s_chunks[c.kc];
                for (int p = 0; p < 3; p++)
                    for (int h = 0; h < 2; h++) {
                        const int vs = 2 * c.vb + h < c.job.nk ? 2 * c.vb + h : c.job.nk - 1;
                        tc::tma_load_2d(st + (3 + p) * kPlaneA + h * (kPlaneA / 2), &tm_d, gmu * 64,
                                        (int)((spin * 3 + p) * md.drows + (long)(c.job.c0 + s_chunks[vs]) * 64),
                                        &sm.full[s]);
                    }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            uint32_t uu = 0;
            for (DensCursor c(job_off, jobs, EPI != 1); c.valid(); c.advance(jobs), uu++) {
                const int s = uu & 1, b = uu & 1;
                const uint32_t ph = (uu >> 1) & 1;
                if (sm.abort || !tc::mbar_wait(&sm.tempty[b], ph ^ 1) || !tc::mbar_wait(&sm.full[s], ph)) {
                    flag_timeout(err, &sm);
                    tc::mma_commit(&sm.tfull[b]);  // release the epilogue
                    break;
                }
                tc::fence_after_sync();
                mma_stage(tmem, b, smem + (size_t)s * kStageBytes, true);
                tc::mma_commit(&sm.empty[s]);
                tc::mma_commit(&sm.tfull[b]);
            }
        }
    } else if (warp >= kEpiWarp0 && warp < kEpiWarp0 + 8) {
        density_epilogue<EPI>(sm, tmem, md, job_off, jobs, acomp, spin, out, err, warp, lane);
    } else if (warp >= 2) {
        // converter warps: the raw Phi tile [64 functions][128 points] is read
        // into registers (releasing the buffer for the next TMA load), split
        // on the fixed-point grid of each point (one exponent over the 64
        // functions, as split_store_fixed_kernel does for the pre-split
        // planes: the same slices) and stored transposed (point-major) as the
        // stage's A planes.  Thread ct < 128 takes point ct; the other
        // converter threads only take part in the barrier arrivals.
        const int ct = conv_index() * 32 + lane;
        uint32_t uu = 0;
        for (DensCursor c(job_off, jobs, EPI != 1); c.valid(); c.advance(jobs), uu++) {
            if (!warp_wait(sm, &sm.rfull[0], uu & 1, err)) break;
            float v[64];
            int e = tc::kFixedZero;
            const uint32_t rf = ssm + 2 * kStageBytes;
            if (ct < 128) {
                float mx = 0.f;
#pragma unroll
                for (int f = 0; f < 64; f++) {
                    v[f] = tc::lds32f(rf + (f * 128 + ct) * 4);
                    mx = fmaxf(mx, fabsf(v[f]));
                }
                e = tc::fixed_exponent_f(mx);
            }
            warp_arrive(&sm.rempty[0]);
            const int s = uu & 1;
            if (!warp_wait(sm, &sm.empty[s], ((uu >> 1) & 1) ^ 1, err)) break;
            const uint32_t st = ssm + s * kStageBytes;
            if (ct < 128) {
#pragma unroll
                for (int jj = 0; jj < 8; jj++) store_chunk_fixed(st, ct, jj, v + 8 * jj, e);
            }
            conv_publish(&sm.full[s]);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, kTmemCols);
}

// The density kernel on the pre-split AO planes: the A operand (Phi of the
// mu chunk, points x functions) is TMA-loaded MN-major from the BF16 store
// (two 64-point boxes per plane), so no warp converts; 384 threads (warp 0
// TMA, warp 1 MMA, warps 4-11 epilogue).
template <int EPI>
__global__ void __launch_bounds__(kF16Threads, 1) density16_kernel(const __grid_constant__ CUtensorMap tm_d,
                                                                   const __grid_constant__ CUtensorMap tm_e16,
                                                                   MixedDev md, const int* __restrict__ job_off,
                                                                   const DensJob* __restrict__ jobs, int acomp,
                                                                   int spin, DensOut out, int* err) {
    extern __shared__ uint8_t smem_raw[];
    __shared__ Smem sm;
    __shared__ int s_chunks[kMaxChunks];
    uint8_t* smem = smem_raw + (((tc::smem_u32(smem_raw) + 1023u) & ~1023u) - tc::smem_u32(smem_raw));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    init_cta(sm, 1, 1);
    const uint32_t tmem = sm.tmem;

    if (warp == 0) {
        if (lane == 0) {
            uint32_t uu = 0;
            for (DensCursor c(job_off, jobs, EPI != 1); c.valid(); c.advance(jobs), uu++) {
                if (c.vb == 0 && c.kc == 0) {  // new tile: its kept chunk ids
                    const int* src = md.tile_chunks + (size_t)c.job.t * md.nchunk;
                    for (int k = 0; k < c.job.nk; k++) s_chunks[k] = __ldg(src + k);
                }
                const int s = uu & 1;
                if (sm.abort || !tc::mbar_wait(&sm.empty[s], ((uu >> 1) & 1) ^ 1)) {
                    flag_timeout(err, &sm);
                    break;
                }
                uint8_t* st = smem + (size_t)s * kStageBytes;
                tc::mbar_arrive_expect_tx(&sm.full[s], 6 * kPlaneA);
                const int gmu = s_chunks[c.kc];
                const long arow = (long)c.job.trow + (long)c.kc * 64;
                for (int p = 0; p < 3; p++) {
                    const int ya = (int)((long)(acomp * 3 + p) * md.rows + arow);
                    tc::tma_load_2d(st + p * kPlaneA, &tm_e16, 0, ya, &sm.full[s]);
                    tc::tma_load_2d(st + p * kPlaneA + kPlaneA / 2, &tm_e16, 64, ya, &sm.full[s]);
                    for (int h = 0; h < 2; h++) {
                        const int vs = 2 * c.vb + h < c.job.nk ? 2 * c.vb + h : c.job.nk - 1;
                        tc::tma_load_2d(st + (3 + p) * kPlaneA + h * (kPlaneA / 2), &tm_d, gmu * 64,
                                        (int)((spin * 3 + p) * md.drows + (long)(c.job.c0 + s_chunks[vs]) * 64),
                                        &sm.full[s]);
                    }
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            uint32_t uu = 0;
            for (DensCursor c(job_off, jobs, EPI != 1); c.valid(); c.advance(jobs), uu++) {
                const int s = uu & 1, b = uu & 1;
                const uint32_t ph = (uu >> 1) & 1;
                if (sm.abort || !tc::mbar_wait(&sm.tempty[b], ph ^ 1) || !tc::mbar_wait(&sm.full[s], ph)) {
                    flag_timeout(err, &sm);
                    tc::mma_commit(&sm.tfull[b]);  // release the epilogue
                    break;
                }
                tc::fence_after_sync();
                mma_stage<true>(tmem, b, smem + (size_t)s * kStageBytes, true);
                tc::mma_commit(&sm.empty[s]);
                tc::mma_commit(&sm.tfull[b]);
            }
        }
    } else if (warp >= kEpiWarp0 && warp < kEpiWarp0 + 8) {
        density_epilogue<EPI>(sm, tmem, md, job_off, jobs, acomp, spin, out, err, warp, lane);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, kTmemCols);
}

// ------------------------------------------------------------- V_xc
// Job (tile t of item I, J):  W_IJ += sum_c L_c,t[I]^T R_c,t[J]
// with L = Phi component c and R = Z (c = 0) or c2 d_c Phi (c = 1..3).
// The operand stage is split along K into two halves (32 points each) that
// act as a two-slot ring: the tensor core runs on one half while the
// converters fill the other (the swizzled rows keep the halves' 16-byte
// chunks disjoint).  A half-stage is (component c, point half kh, K-half
// hk); a tile is one accumulation unit; an item's last tile writes W_IJ.
// Warps 2-15 convert; warps 4-11 also drain the accumulator of each tile.
//
// The meta-GGA part sum_r d_r phi^T c2 d_r phi of W is symmetric, so only
// items with I <= J carry components 1..3, with c2 doubled when I < J
// (job flags kTauItem, kTauDouble); V = W + W^T then receives it once.
constexpr int kTauItem = 4, kTauDouble = 8;

// Position in the half-stage sequence of one CTA (host-made job list).
struct FockCursor {
    int j, end, c, kh, hk, ncomp, nc_all;
    FockJob job;
    __device__ void load(const FockJob* jobs) {
        const int4* p = reinterpret_cast<const int4*>(jobs + j);
        const int4 a = __ldg(p), b = __ldg(p + 1);
        job.t = a.x;
        job.trow = a.y;
        job.sa0 = a.z;
        job.sa1 = a.w;
        job.sb0 = b.x;
        job.sb1 = b.y;
        job.item = b.z;
        job.flags = b.w;
        ncomp = (job.flags & kTauItem) ? nc_all : 1;
    }
    __device__ FockCursor(const int* off, const FockJob* jobs, int nc) {
        j = off[blockIdx.x];
        end = off[blockIdx.x + 1];
        nc_all = nc;
        ncomp = 1;
        c = kh = hk = 0;
        if (j < end) load(jobs);
    }
    __device__ bool valid() const { return j < end; }
    __device__ bool first_of_tile() const { return c == 0 && kh == 0 && hk == 0; }
    __device__ bool last_of_tile() const { return c == ncomp - 1 && kh == 1 && hk == 1; }
    __device__ void advance(const FockJob* jobs) {
        if (++hk < 2) return;
        hk = 0;
        if (++kh < 2) return;
        kh = 0;
        if (++c < ncomp) return;
        c = 0;
        if (++j < end) load(jobs);
    }
    __device__ int slot(int box) const {
        return box == 0 ? job.sa0 : box == 1 ? job.sa1 : box == 2 ? job.sb0 : job.sb1;
    }
};

constexpr int kFockConvWarps = 14;                     // warps 2-15
constexpr int kFockConvThreads = kFockConvWarps * 32;
constexpr int kFockItems = (1024 + kFockConvThreads - 1) / kFockConvThreads;  // (row, 8-point chunk) items

// The six split products of K-half hk (k-steps 2 hk, 2 hk + 1) of the stage.
__device__ __forceinline__ void mma_half(uint32_t tmem, int buf, uint8_t* st, int hk, bool first) {
    const uint32_t a0 = tc::smem_u32(st), b0 = a0 + 3 * kPlaneA;
    const uint32_t d_hh = tmem + buf * 256, d_corr = tmem + buf * 256 + 128;
#pragma unroll
    for (int q = 0; q < 6; q++) {
        const uint64_t ad = tc::smem_desc_sw128(a0 + c_prod_a[q] * kPlaneA);
        const uint64_t bd = tc::smem_desc_sw128(b0 + c_prod_b[q] * kPlaneA);
        const uint32_t d = q == 0 ? d_hh : d_corr;
#pragma unroll
        for (int kk = 0; kk < 2; kk++) {
            const int k = 2 * hk + kk;
            const bool start = first && kk == 0 && (q == 0 || q == 1);
            tc::mma_bf16(d, ad + 2 * k, bd + 2 * k, kIdesc, start ? 0u : 1u);
        }
    }
}

__global__ void __launch_bounds__(kThreads, 1) fock_tc_kernel(const __grid_constant__ CUtensorMap tm_e32,
                                                              const __grid_constant__ CUtensorMap tm_z, long rows,
                                                              const int* __restrict__ job_off,
                                                              const FockJob* __restrict__ jobs,
                                                              const float* __restrict__ c2, int ncomp,
                                                              double* __restrict__ wpart, int* err) {
    extern __shared__ uint8_t smem_raw[];
    __shared__ Smem sm;
    uint8_t* smem = smem_raw + (((tc::smem_u32(smem_raw) + 1023u) & ~1023u) - tc::smem_u32(smem_raw));
    const uint32_t ssm = tc::smem_u32(smem);
    uint8_t* raws = smem + kStageBytes;  // kRawSlots raw half-stages of kRawF bytes
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    init_cta(sm, kFockConvWarps, kFockConvWarps);
    const uint32_t tmem = sm.tmem;

    if (warp == 0) {
        if (lane == 0) {
            uint32_t hs = 0;
            for (FockCursor c(job_off, jobs, ncomp); c.valid(); c.advance(jobs), hs++) {
                const int r = hs % kRawSlots;
                if (sm.abort || !tc::mbar_wait(&sm.rempty[r], ((hs / kRawSlots) & 1) ^ 1)) {
                    flag_timeout(err, &sm);
                    break;
                }
                uint32_t bytes = 0;
                for (int k = 0; k < 4; k++) bytes += c.slot(k) >= 0 ? kRawBox : 0;
                tc::mbar_arrive_expect_tx(&sm.rfull[r], bytes);
                uint8_t* rb = raws + (size_t)r * kRawF;
                const int x = c.kh * 64 + c.hk * 32;
                for (int k = 0; k < 4; k++) {
                    const int sl = c.slot(k);
                    if (sl < 0) continue;
                    const long row = (long)c.job.trow + (long)sl * 64;
                    if (k >= 2 && c.c == 0)
                        tc::tma_load_2d(rb + k * kRawBox, &tm_z, x, (int)row, &sm.rfull[r]);
                    else
                        tc::tma_load_2d(rb + k * kRawBox, &tm_e32, x, (int)((long)c.c * rows + row), &sm.rfull[r]);
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            uint32_t hs = 0, ut = 0;
            for (FockCursor c(job_off, jobs, ncomp); c.valid(); c.advance(jobs), hs++) {
                const int b = ut & 1, h = c.hk;
                if (c.first_of_tile() && (sm.abort || !tc::mbar_wait(&sm.tempty[b], ((ut >> 1) & 1) ^ 1))) {
                    flag_timeout(err, &sm);
                    tc::mma_commit(&sm.tfull[b]);
                    break;
                }
                if (sm.abort || !tc::mbar_wait(&sm.full[h], (hs >> 1) & 1)) {
                    flag_timeout(err, &sm);
                    tc::mma_commit(&sm.tfull[b]);
                    break;
                }
                tc::fence_after_sync();
                mma_half(tmem, b, smem, h, c.first_of_tile());
                tc::mma_commit(&sm.empty[h]);
                if (c.last_of_tile()) {
                    tc::mma_commit(&sm.tfull[b]);
                    ut++;
                }
            }
        }
    } else {
        // warps 2-15: convert every half-stage (the raw L and R boxes into
        // the K-half of the operand planes; R = c2 d_c Phi for c > 0);
        // warps 4-11 drain tile u - 1 after converting tile u
        const int ct = (warp - 2) * 32 + lane;
        const bool drainer = warp >= kEpiWarp0 && warp < kEpiWarp0 + 8;
        const int quad = warp & 3, half = (warp - kEpiWarp0) >> 2;
        const int g = quad * 32 + lane;
        float W[64];
#pragma unroll
        for (int jw = 0; jw < 64; jw++) W[jw] = 0.f;
        uint32_t hs = 0, ut = 0;
        int prev_flags = 0, prev_item = 0;
        bool pending = false, ok = true;
        auto drain_prev = [&]() -> bool {
            const int b = ut & 1;
            if (sm.abort || !tc::mbar_wait(&sm.tfull[b], (ut >> 1) & 1)) {
                flag_timeout(err, &sm);
                return false;
            }
            tc::fence_after_sync();
            drain(tmem, b, quad, half, W);
            tc::fence_before_sync();
            mbar_arrive(&sm.tempty[b]);
            ut++;
            if (prev_flags & 2) {
                double* o = wpart + (size_t)prev_item * 16384 + (size_t)g * 128 + half * 64;
#pragma unroll
                for (int jw = 0; jw < 64; jw += 2) {
                    *reinterpret_cast<double2*>(o + jw) = make_double2((double)W[jw], (double)W[jw + 1]);
                    W[jw] = W[jw + 1] = 0.f;
                }
            }
            return true;
        };
        for (FockCursor c(job_off, jobs, ncomp); c.valid(); c.advance(jobs), hs++) {
            const int r = hs % kRawSlots, h = c.hk;
            if (!warp_wait(sm, &sm.rfull[r], (hs / kRawSlots) & 1, err)) {
                ok = false;
                break;
            }
            if (!warp_wait(sm, &sm.empty[h], ((hs >> 1) & 1) ^ 1, err)) {
                ok = false;
                break;
            }
            const uint32_t rb = ssm + kStageBytes + r * kRawF;
#pragma unroll
            for (int k = 0; k < kFockItems; k++) {
                const int q = ct + kFockConvThreads * k;
                if (q >= 1024) break;
                // a quarter-warp covers rows r and r + 4 (4 chunks each): its 16-byte
                // stores land in 8 distinct swizzle slots, and lanes of the second row
                // read the other 16-byte half first, so both reads are conflict-free
                const int op = q >> 9, jj = q & 3, odd = (q >> 2) & 1;
                const int rr = ((q & 511) >> 5) * 8 + odd * 4 + ((q >> 3) & 3);
                const int box = op * 2 + (rr >> 6);
                float v[8];
                if (c.slot(box) < 0) {
#pragma unroll
                    for (int i = 0; i < 8; i++) v[i] = 0.f;
                } else {
                    const uint32_t src = rb + box * kRawBox + (rr & 63) * 128 + jj * 32;
                    const float4 x0 = tc::lds128f(src + odd * 16), x1 = tc::lds128f(src + (odd ^ 1) * 16);
                    const float4 a = odd ? x1 : x0, b4 = odd ? x0 : x1;
                    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
                    v[4] = b4.x; v[5] = b4.y; v[6] = b4.z; v[7] = b4.w;
                    if (op == 1 && c.c > 0) {
                        const float* cp = c2 + (size_t)c.job.t * 128 + c.kh * 64 + h * 32 + 8 * jj;
                        const float4 ca = __ldg(reinterpret_cast<const float4*>(cp));
                        const float4 cb = __ldg(reinterpret_cast<const float4*>(cp + 4));
                        const float f = (c.job.flags & kTauDouble) ? 2.f : 1.f;  // exact scaling
                        v[0] *= f * ca.x; v[1] *= f * ca.y; v[2] *= f * ca.z; v[3] *= f * ca.w;
                        v[4] *= f * cb.x; v[5] *= f * cb.y; v[6] *= f * cb.z; v[7] *= f * cb.w;
                    }
                }
                store_chunk(ssm + (op ? 3 * kPlaneA : 0), rr, 4 * h + jj, v);
            }
            warp_arrive(&sm.rempty[r]);
            conv_publish(&sm.full[h]);
            if (drainer && c.last_of_tile()) {
                if (pending && !drain_prev()) {
                    ok = false;
                    break;
                }
                pending = true;
                prev_flags = c.job.flags;
                prev_item = c.job.item;
            }
        }
        if (drainer && ok && pending) drain_prev();
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, kTmemCols);
}

// ------------------------------------------------------------ V_xc, pre-split operands
// The jobs of fock_tc_kernel with both operands read as BF16 planes from HBM
// (L: the AO store split once per grid; R: Z and c2 d_c phi split once per
// build), so TMA feeds the tensor core with no conversion in the kernel.  A
// stage is (component c, 64-point half kh of the tile): three A planes and
// three B planes (96 KB), two stages in flight.  A dropped 64-function box
// is loaded from row -64: entirely out of bounds, so TMA fills it with zeros.
// Items with c2 doubled (I < J) halve the accumulators at their first
// meta-GGA product and are drained with weight 2 (both exact).
// CTA roles (384 threads): warp 0 TMA, warp 1 MMA, warps 4-11 drain.

struct Fock16Cursor {
    int j, end, c, kh, ncomp, nc_all;
    FockJob job;
    __device__ void load(const FockJob* jobs) {
        const int4* p = reinterpret_cast<const int4*>(jobs + j);
        const int4 a = __ldg(p), b = __ldg(p + 1);
        job = FockJob{a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
        ncomp = (job.flags & kTauItem) ? nc_all : 1;
    }
    __device__ Fock16Cursor(const int* off, const FockJob* jobs, int nc) {
        j = off[blockIdx.x];
        end = off[blockIdx.x + 1];
        nc_all = nc;
        ncomp = 1;
        c = kh = 0;
        if (j < end) load(jobs);
    }
    __device__ bool valid() const { return j < end; }
    __device__ bool first_of_tile() const { return c == 0 && kh == 0; }
    __device__ bool last_of_tile() const { return c == ncomp - 1 && kh == 1; }
    __device__ void advance(const FockJob* jobs) {
        if (++kh < 2) return;
        kh = 0;
        if (++c < ncomp) return;
        c = 0;
        if (++j < end) load(jobs);
    }
    __device__ int slot(int box) const {
        return box == 0 ? job.sa0 : box == 1 ? job.sa1 : box == 2 ? job.sb0 : job.sb1;
    }
};

__global__ void __launch_bounds__(kF16Threads, 1) fock16_kernel(const __grid_constant__ CUtensorMap tm_l,
                                                                const __grid_constant__ CUtensorMap tm_r, long rows,
                                                                const int* __restrict__ job_off,
                                                                const FockJob* __restrict__ jobs, int ncomp,
                                                                double* __restrict__ wpart, int* err) {
    extern __shared__ uint8_t smem_raw[];
    __shared__ Smem sm;
    uint8_t* smem = smem_raw + (((tc::smem_u32(smem_raw) + 1023u) & ~1023u) - tc::smem_u32(smem_raw));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    init_cta(sm, 1, 1);
    const uint32_t tmem = sm.tmem;

    if (warp == 0) {
        if (lane == 0) {
            uint32_t st = 0;
            for (Fock16Cursor c(job_off, jobs, ncomp); c.valid(); c.advance(jobs), st++) {
                const int s = st & 1;
                if (sm.abort || !tc::mbar_wait(&sm.empty[s], ((st >> 1) & 1) ^ 1)) {
                    flag_timeout(err, &sm);
                    break;
                }
                uint8_t* sb = smem + (size_t)s * kStageBytes;
                tc::mbar_arrive_expect_tx(&sm.full[s], 12 * (kPlaneA / 2));
                for (int k = 0; k < 4; k++) {
                    const int sl = c.slot(k);
                    const CUtensorMap* map = k < 2 ? &tm_l : &tm_r;
                    for (int p = 0; p < 3; p++) {
                        const int y = sl >= 0 ? (int)((long)(c.c * 3 + p) * rows + c.job.trow + (long)sl * 64) : -64;
                        tc::tma_load_2d(sb + ((k >> 1) * 3 + p) * kPlaneA + (k & 1) * (kPlaneA / 2), map, c.kh * 64,
                                        y, &sm.full[s]);
                    }
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            uint32_t st = 0, ut = 0;
            for (Fock16Cursor c(job_off, jobs, ncomp); c.valid(); c.advance(jobs), st++) {
                const int s = st & 1, b = ut & 1;
                if (c.first_of_tile() && (sm.abort || !tc::mbar_wait(&sm.tempty[b], ((ut >> 1) & 1) ^ 1))) {
                    flag_timeout(err, &sm);
                    tc::mma_commit(&sm.tfull[b]);
                    break;
                }
                if (sm.abort || !tc::mbar_wait(&sm.full[s], (st >> 1) & 1)) {
                    flag_timeout(err, &sm);
                    tc::mma_commit(&sm.tfull[b]);
                    break;
                }
                tc::fence_after_sync();
                const bool halve = (c.job.flags & kTauDouble) && c.c == 1 && c.kh == 0;
                mma_stage(tmem, b, smem + (size_t)s * kStageBytes, c.first_of_tile(), halve);
                tc::mma_commit(&sm.empty[s]);
                if (c.last_of_tile()) {
                    tc::mma_commit(&sm.tfull[b]);
                    ut++;
                }
            }
        }
    } else if (warp >= kEpiWarp0 && warp < kEpiWarp0 + 8) {
        // drain every tile into W (this thread's row g, 64 columns); flush W
        // at the item's last tile
        const int quad = warp & 3, half = (warp - kEpiWarp0) >> 2;
        const int g = quad * 32 + lane;
        float W[64];
#pragma unroll
        for (int jw = 0; jw < 64; jw++) W[jw] = 0.f;
        uint32_t ut = 0;
        for (int j = job_off[blockIdx.x]; j < job_off[blockIdx.x + 1]; j++, ut++) {
            const int4 jb = __ldg(reinterpret_cast<const int4*>(jobs + j) + 1);  // sb0, sb1, item, flags
            const int item = jb.z, flags = jb.w;
            const int b = ut & 1;
            if (sm.abort || !tc::mbar_wait(&sm.tfull[b], (ut >> 1) & 1)) {
                flag_timeout(err, &sm);
                break;
            }
            tc::fence_after_sync();
            const bool dbl = (flags & kTauDouble) && ncomp > 1;
            drain(tmem, b, quad, half, W, dbl ? 2.f : 1.f);
            tc::fence_before_sync();
            mbar_arrive(&sm.tempty[b]);
            if (flags & 2) {
                double* o = wpart + (size_t)item * 16384 + (size_t)g * 128 + half * 64;
#pragma unroll
                for (int jw = 0; jw < 64; jw += 2) {
                    *reinterpret_cast<double2*>(o + jw) = make_double2((double)W[jw], (double)W[jw + 1]);
                    W[jw] = W[jw + 1] = 0.f;
                }
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, kTmemCols);
}

// Sums the two column-half partials of the density outputs (deterministic).
__global__ void combine_kernel(long n1, long n3, double* __restrict__ rho, const double* __restrict__ rho_b,
                               double* __restrict__ rho1, const double* __restrict__ rho1_b, double* __restrict__ tau,
                               const double* __restrict__ tau_b, int type) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n1) {
        rho[i] += rho_b[i];
        if (type >= 2) tau[i] += tau_b[i];
    }
    if (type >= 1 && i < n3) rho1[i] += rho1_b[i];
}

// out = a * x + b * y (FP64, n elements).
__global__ void axpby_kernel(long n, double a, const double* __restrict__ x, double b, const double* __restrict__ y,
                             double* __restrict__ out) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = a * x[i] + b * y[i];
}

// Tile-order copy of FP64-order point arrays (ncomp planes).
__global__ void gather_kernel(const long* __restrict__ perm, long Gt, long Gp, int ncomp, const double* __restrict__ src,
                              double* __restrict__ dst, bool zero_pads) {
    const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= Gt) return;
    const long q = perm[p];
    const bool pad = q < 0;
    const long i = pad ? -q - 1 : q;
    for (int c = 0; c < ncomp; c++) dst[(long)c * Gt + p] = (pad && zero_pads) ? 0.0 : src[(long)c * Gp + i];
}

// V_m(mu, nu) = sum over splits of W(mu, nu) + W(nu, mu).  A block of 32 x 32
// threads owns a 32 x 32 tile of V (grid z = molecule): the W(nu, mu) partials
// are read along mu (coalesced, as V is written), the W(mu, nu) partials along
// nu and turned through shared memory.  Four splits per step keep eight loads
// in flight per thread.
__global__ void __launch_bounds__(1024) wsum_kernel(const double* __restrict__ wpart, const int* __restrict__ live,
                                                    const MolRange* __restrict__ mols, int spin,
                                                    double* __restrict__ V) {
    __shared__ double ta[32][33];
    const MolRange m = mols[blockIdx.z];
    const int mu0 = blockIdx.x * 32, nu0 = blockIdx.y * 32;
    if (mu0 >= m.n || nu0 >= m.n) return;  // uniform over the block
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int I = mu0 >> 7, J = nu0 >> 7;
    const long ia = m.item0 + ((long)I * m.nblk + J) * m.nsplit, ib = m.item0 + ((long)J * m.nblk + I) * m.nsplit;
    const double* wa = wpart + (size_t)ia * 16384 + (size_t)((mu0 & 127) + ty) * 128 + (nu0 & 127) + tx;
    const double* wb = wpart + (size_t)ib * 16384 + (size_t)((nu0 & 127) + ty) * 128 + (mu0 & 127) + tx;
    double acc_a = 0, acc_b = 0;  // (mu0 + ty, nu0 + tx) and (mu0 + tx, nu0 + ty)
    int s = 0;
    for (; s + 4 <= m.nsplit; s += 4) {
        double va[4], vb[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            va[k] = live[ia + s + k] ? wa[(size_t)(s + k) * 16384] : 0.0;
            vb[k] = live[ib + s + k] ? wb[(size_t)(s + k) * 16384] : 0.0;
        }
#pragma unroll
        for (int k = 0; k < 4; k++) {
            acc_a += va[k];
            acc_b += vb[k];
        }
    }
    for (; s < m.nsplit; s++) {
        if (live[ia + s]) acc_a += wa[(size_t)s * 16384];
        if (live[ib + s]) acc_b += wb[(size_t)s * 16384];
    }
    ta[ty][tx] = acc_a;
    __syncthreads();
    const int mu = mu0 + tx, nu = nu0 + ty;
    if (mu < m.n && nu < m.n) V[m.voff + (long)spin * m.n * m.n + (long)nu * m.n + mu] = ta[tx][ty] + acc_b;
}

// Packed D_m (s, n, n) column-major FP64 -> three BF16 planes per spin of the
// strip: row f0(m) + nu, col mu, of (D + D^T) / 2 (zero outside the
// molecule's n x n block).  One warp per (spin, row, 64-column chunk): the
// chunk's values share one fixed-point exponent (tc::split3_fixed), the K
// range of one accumulation unit of the density kernel, whose A operand
// (e16d) shares one exponent per point over the same 64 functions -- so the
// hh products of a unit accumulate exactly on the tensor core.
__global__ void split_d_kernel(const double* __restrict__ D, const MolRange* __restrict__ mols, int nmol, int nspin,
                               long drows, int dcols, bf16* __restrict__ Dp) {
    const long wid = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int nch = dcols / 64;
    const long total = (long)nspin * drows * nch;
    if (wid >= total) return;  // whole warps leave together (blockDim is a multiple of 32)
    const int ch = (int)(wid % nch);
    const long row = (wid / nch) % drows;
    const int s = (int)(wid / ((long)nch * drows));
    int lo = 0, hi = nmol - 1;  // molecule owning the row (f0 ascending)
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (mols[mid].f0 <= row) lo = mid;
        else hi = mid - 1;
    }
    const MolRange& m = mols[lo];
    const long nu = row - m.f0;
    // symmetric part (the tensor-core density uses one triangle of D for rho and tau)
    const double* Ds = D + m.voff + (long)s * m.n * m.n;
    double v[2];
#pragma unroll
    for (int k = 0; k < 2; k++) {
        const int mu = ch * 64 + k * 32 + lane;
        v[k] = (mu < m.n && nu < m.n) ? 0.5 * (Ds[nu * m.n + mu] + Ds[(long)mu * m.n + nu]) : 0.0;
    }
    double mx = fmax(fabs(v[0]), fabs(v[1]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    const int e = tc::fixed_exponent(mx);
    const size_t plane = (size_t)drows * dcols;
#pragma unroll
    for (int k = 0; k < 2; k++) {
        bf16 h, md_, l;
        tc::split3_fixed(v[k], e, h, md_, l);
        const size_t o = (size_t)row * dcols + ch * 64 + k * 32 + lane;
        Dp[(size_t)(s * 3 + 0) * plane + o] = h;
        Dp[(size_t)(s * 3 + 1) * plane + o] = md_;
        Dp[(size_t)(s * 3 + 2) * plane + o] = l;
    }
}

// Z = c0 phi + c1 . grad phi per kept row (FP32); c2 per point (meta-GGA).
// One CTA per tile, thread = point.
__global__ void __launch_bounds__(128) prep_z_kernel(MixedDev md, int type, const double* __restrict__ fcoef,
                                                     float* __restrict__ Z, float* __restrict__ c2) {
    const int t = blockIdx.x, g = threadIdx.x;
    const long pt = (long)t * 128 + g;
    const long Gt = md.Gt;
    const float a0 = (float)fcoef[pt];
    float a1 = 0, a2 = 0, a3 = 0;
    if (type >= 1) {
        a1 = (float)fcoef[Gt + pt];
        a2 = (float)fcoef[2 * Gt + pt];
        a3 = (float)fcoef[3 * Gt + pt];
    }
    if (type >= 2) c2[pt] = (float)fcoef[4 * Gt + pt];
    const long r0 = md.tile_row[t], nr = (long)md.tile_nkept[t] * 64;
    const size_t cs = (size_t)md.rows * 128;
    for (long r = 0; r < nr; r++) {
        const size_t o = (size_t)(r0 + r) * 128 + g;
        float z = a0 * __ldg(md.e32 + o);
        if (type >= 1) {
            z = fmaf(a1, __ldg(md.e32 + cs + o), z);
            z = fmaf(a2, __ldg(md.e32 + 2 * cs + o), z);
            z = fmaf(a3, __ldg(md.e32 + 3 * cs + o), z);
        }
        Z[o] = z;
    }
}

// x = h + m + l in BF16 (the arithmetic of split8, one element).
__device__ __forceinline__ void split1(float x, bf16& h, bf16& m, bf16& l) {
    h = __float2bfloat16_rn(x);
    const float r = x - __bfloat162float(h);
    m = __float2bfloat16_rn(r);
    l = __float2bfloat16_rn(r - __bfloat162float(m));
}

// The FP32 AO store as BF16 planes: e16[(c * 3 + p) * n + i] (n = rows * 128).
__global__ void split_store_kernel(const float* __restrict__ e32, long n, int ncomp, bf16* __restrict__ e16) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * ncomp) return;
    const int c = (int)(i / n);
    const long o = i - (long)c * n;
    bf16 h, m, l;
    split1(e32[i], h, m, l);
    e16[(size_t)(c * 3 + 0) * n + o] = h;
    e16[(size_t)(c * 3 + 1) * n + o] = m;
    e16[(size_t)(c * 3 + 2) * n + o] = l;
}

// The density kernel's A operand planes: components 0..ncomp-1 of the FP32
// store split on the fixed-point grid of each (point, 64-function slot): the
// 64 values of one point in one slot (the K range of a density unit) share
// one exponent (tc::split3_fixed).  Layout as e16: e16d[(c * 3 + p) * n +
// row * 128 + g].  One CTA per (component, 64-row slot), thread = point.
__global__ void __launch_bounds__(128) split_store_fixed_kernel(const float* __restrict__ e32, long rows, int ncomp,
                                                                bf16* __restrict__ e16d) {
    const long nslot = rows / 64;
    const int c = (int)(blockIdx.x / nslot);
    const long sl = blockIdx.x - (long)c * nslot;
    const int g = threadIdx.x;
    if (c >= ncomp) return;
    const size_t n = (size_t)rows * 128;
    const float* src = e32 + (size_t)c * n + (size_t)sl * 64 * 128 + g;
    float mx = 0.f;
    for (int f = 0; f < 64; f++) mx = fmaxf(mx, fabsf(src[(size_t)f * 128]));
    const int e = tc::fixed_exponent_f(mx);
    bf16* dst = e16d + (size_t)(c * 3) * n + (size_t)sl * 64 * 128 + g;
    for (int f = 0; f < 64; f++) {
        bf16 h, m, l;
        tc::split3_fixed_f(src[(size_t)f * 128], e, h, m, l);
        const size_t o = (size_t)f * 128;
        dst[o] = h;
        dst[n + o] = m;
        dst[2 * n + o] = l;
    }
}

// Two consecutive points of one row into the three planes (one 4-byte
// store per plane).
__device__ __forceinline__ void store3x2(bf16* __restrict__ R, size_t n, size_t o, float x0, float x1) {
    bf16 h0, m0, l0, h1, m1, l1;
    split1(x0, h0, m0, l0);
    split1(x1, h1, m1, l1);
    *reinterpret_cast<__nv_bfloat162*>(R + o) = __halves2bfloat162(h0, h1);
    *reinterpret_cast<__nv_bfloat162*>(R + n + o) = __halves2bfloat162(m0, m1);
    *reinterpret_cast<__nv_bfloat162*>(R + 2 * n + o) = __halves2bfloat162(l0, l1);
}

// R operands of the pre-split V kernel as BF16 planes, per kept row:
// component 0: Z = c0 phi + c1 . grad phi (the FP32 arithmetic of
// prep_z_kernel); components 1-3 (meta-GGA): c2 d_c phi.  One CTA per tile,
// 256 threads: thread = (point pair, row phase); rows phase + 4k, U at a
// time (U = 4 for LDA / GGA, 2 for meta-GGA with its twelve output planes).
template <int U>
__global__ void __launch_bounds__(256) prep16_kernel(MixedDev md, int type, const double* __restrict__ fcoef,
                                                     bf16* __restrict__ R16) {
    const int t = blockIdx.x, pp = threadIdx.x & 63, ph = threadIdx.x >> 6;
    const long pt = (long)t * 128 + 2 * pp;
    const long Gt = md.Gt;
    float a0[2], a1[2] = {0, 0}, a2[2] = {0, 0}, a3[2] = {0, 0}, c2[2] = {0, 0};
#pragma unroll
    for (int q = 0; q < 2; q++) {
        a0[q] = (float)fcoef[pt + q];
        if (type >= 1) {
            a1[q] = (float)fcoef[Gt + pt + q];
            a2[q] = (float)fcoef[2 * Gt + pt + q];
            a3[q] = (float)fcoef[3 * Gt + pt + q];
        }
        if (type >= 2) c2[q] = (float)fcoef[4 * Gt + pt + q];
    }
    const long r0 = md.tile_row[t], nr = (long)md.tile_nkept[t] * 64;  // a multiple of 4 U
    const size_t n = (size_t)md.rows * 128;
    const float* e = md.e32 + (size_t)r0 * 128 + 2 * pp;
    bf16* R = R16 + (size_t)r0 * 128 + 2 * pp;
    for (long r = ph; r < nr; r += 4 * U) {
        float2 v[U][4];
#pragma unroll
        for (int i = 0; i < U; i++) {
            const size_t o = (size_t)(r + 4 * i) * 128;
            v[i][0] = __ldg(reinterpret_cast<const float2*>(e + o));
            if (type >= 1) {
                v[i][1] = __ldg(reinterpret_cast<const float2*>(e + n + o));
                v[i][2] = __ldg(reinterpret_cast<const float2*>(e + 2 * n + o));
                v[i][3] = __ldg(reinterpret_cast<const float2*>(e + 3 * n + o));
            }
        }
#pragma unroll
        for (int i = 0; i < U; i++) {
            const size_t o = (size_t)(r + 4 * i) * 128;
            float z0 = a0[0] * v[i][0].x, z1 = a0[1] * v[i][0].y;
            if (type >= 1) {
                z0 = fmaf(a1[0], v[i][1].x, z0);
                z1 = fmaf(a1[1], v[i][1].y, z1);
                z0 = fmaf(a2[0], v[i][2].x, z0);
                z1 = fmaf(a2[1], v[i][2].y, z1);
                z0 = fmaf(a3[0], v[i][3].x, z0);
                z1 = fmaf(a3[1], v[i][3].y, z1);
            }
            store3x2(R, n, o, z0, z1);
            if (type >= 2) {
                store3x2(R + 3 * n, n, o, v[i][1].x * c2[0], v[i][1].y * c2[1]);
                store3x2(R + 6 * n, n, o, v[i][2].x * c2[0], v[i][2].y * c2[1]);
                store3x2(R + 9 * n, n, o, v[i][3].x * c2[0], v[i][3].y * c2[1]);
            }
        }
    }
}

// E_m = sum of the per-tile partials of molecule m (fixed order).
__global__ void energy_mols_kernel(const double* __restrict__ partial, const MolRange* __restrict__ mols,
                                   double* __restrict__ E) {
    const MolRange m = mols[blockIdx.x];
    __shared__ double red[256];
    double v = 0;
    for (int t = m.t0 + threadIdx.x; t < m.t1; t += blockDim.x) v += partial[t];
    red[threadIdx.x] = v;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) E[blockIdx.x] = red[0];
}

// AO values and gradients of every tile into the FP32 store, evaluated in
// FP64.  One CTA per tile, thread = point; loops over the tile's shells.
constexpr int kNcart = (kMaxL + 1) * (kMaxL + 2) / 2;

__global__ void __launch_bounds__(128) ao_mixed_kernel(MixedDev md, DevShells sh, const int* __restrict__ tile_shells,
                                                       const int* __restrict__ tile_shell_off,
                                                       const double* __restrict__ px, const double* __restrict__ py,
                                                       const double* __restrict__ pz, const double* __restrict__ shtab,
                                                       int ao_comp, float* __restrict__ e32) {
    const int t = blockIdx.x, g = threadIdx.x;
    const long pt = (long)t * 128 + g;
    const double X = px[pt], Y = py[pt], Z = pz[pt];
    const int* slots = md.tile_slot + (size_t)t * md.nchunk;
    const int c0 = md.tile_c0[t];
    const long trow = md.tile_row[t];
    const size_t cs = (size_t)md.rows * 128;
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
            const int slot = slots[(mu >> 6) - c0];
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
            const size_t o = (size_t)(trow + slot * 64 + (mu & 63)) * 128 + g;
            e32[o] = (float)(A * Q);
            if (ao_comp == 4) {
                e32[cs + o] = (float)(Ax * Q + A * Qx);
                e32[2 * cs + o] = (float)(Ay * Q + A * Qy);
                e32[3 * cs + o] = (float)(Az * Q + A * Qz);
            }
        }
    }
}

// Diagnostic of the bounded waits: one CTA sets up as the tensor-core
// kernels do (their mbarriers and 512 TMEM columns), one thread waits on a
// barrier that nothing ever arrives on, for budget_ns, flags the timeout in
// err as the pipelines do and the CTA unwinds, releasing TMEM.  No TMA load
// or MMA is issued, so nothing is in flight when the wait gives up.
__global__ void __launch_bounds__(128, 1) wait_probe_kernel(unsigned long long budget_ns, int* err) {
    __shared__ Smem sm;
    init_cta(sm, 1, 1);
    const uint32_t tmem = sm.tmem;
    if (threadIdx.x == 32 && !tc::mbar_wait_budget(&sm.full[0], 0, budget_ns)) flag_timeout(err, &sm);
    tc::fence_before_sync();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) tc::tmem_dealloc(tmem, kTmemCols);
}

}  // namespace

void launch_wait_probe(double budget_ms, int* err, cudaStream_t s) {
    wait_probe_kernel<<<1, 128, 0, s>>>((unsigned long long)(budget_ms * 1e6), err);
    CGB_CUDA(cudaGetLastError());
}

void launch_ao_mixed(const MixedDev& md, DevShells sh, const int* tile_shells, const int* tile_shell_off, const double* x,
                     const double* y, const double* z, const double* shtab, int ao_comp, float* e32, cudaStream_t s) {
    if (md.ntiles == 0) return;
    ao_mixed_kernel<<<md.ntiles, 128, 0, s>>>(md, sh, tile_shells, tile_shell_off, x, y, z, shtab, ao_comp, e32);
    CGB_CUDA(cudaGetLastError());
}

void launch_split_d(const double* D, const MolRange* mols, int nmol, int nspin, long drows, int dcols, int /*maxn*/,
                    bf16* Dp, cudaStream_t s) {
    CGB_CHECK(dcols % 64 == 0, XC_ERR_INTERNAL, "density strip width is not a multiple of 64");
    const long threads = (long)nspin * drows * (dcols / 64) * 32;
    if (threads == 0) return;
    split_d_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(D, mols, nmol, nspin, drows, dcols, Dp);
    CGB_CUDA(cudaGetLastError());
}


size_t mixed_smem_bytes() { return (size_t)kSmemBytes + 1024; }

void set_mixed_kernel_attributes() {
    const int smem = (int)mixed_smem_bytes();
    CGB_CUDA(cudaFuncSetAttribute(density_tc_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    CGB_CUDA(cudaFuncSetAttribute(density_tc_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    CGB_CUDA(cudaFuncSetAttribute(density_tc_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    CGB_CUDA(cudaFuncSetAttribute(fock_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    const int smem16 = (int)(2 * kStageBytes + 1024);
    CGB_CUDA(cudaFuncSetAttribute(fock16_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem16));
    CGB_CUDA(cudaFuncSetAttribute(density16_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem16));
    CGB_CUDA(cudaFuncSetAttribute(density16_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem16));
    CGB_CUDA(cudaFuncSetAttribute(density16_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem16));
}

void launch_density_tc(const CUtensorMap& tm_d, const CUtensorMap& tm_raw, const MixedDev& md, int ctas,
                       const int* job_off, const DensJob* jobs, int epi, int acomp, int spin, double* rho,
                       double* rho1, double* tau, double* rho_b, double* rho1_b, double* tau_b, int* err,
                       cudaStream_t s) {
    if (ctas == 0) return;
    CGB_CHECK(md.nchunk <= kMaxChunks, XC_ERR_UNSUPPORTED, "more than 16384 basis functions in one molecule");
    const size_t smem = mixed_smem_bytes();
    DensOut o{rho, rho1, tau, rho_b, rho1_b, tau_b};
    if (epi == 0)
        density_tc_kernel<0><<<ctas, kThreads, smem, s>>>(tm_d, tm_raw, md, job_off, jobs, acomp, spin, o, err);
    else if (epi == 1)
        density_tc_kernel<1><<<ctas, kThreads, smem, s>>>(tm_d, tm_raw, md, job_off, jobs, acomp, spin, o, err);
    else
        density_tc_kernel<2><<<ctas, kThreads, smem, s>>>(tm_d, tm_raw, md, job_off, jobs, acomp, spin, o, err);
    CGB_CUDA(cudaGetLastError());
}

void launch_density16(const CUtensorMap& tm_d, const CUtensorMap& tm_e16, const MixedDev& md, int ctas,
                      const int* job_off, const DensJob* jobs, int epi, int acomp, int spin, double* rho,
                      double* rho1, double* tau, double* rho_b, double* rho1_b, double* tau_b, int* err,
                      cudaStream_t s) {
    if (ctas == 0) return;
    CGB_CHECK(md.nchunk <= kMaxChunks, XC_ERR_UNSUPPORTED, "more than 16384 basis functions in one molecule");
    const size_t smem = 2 * kStageBytes + 1024;
    DensOut o{rho, rho1, tau, rho_b, rho1_b, tau_b};
    if (epi == 0)
        density16_kernel<0><<<ctas, kF16Threads, smem, s>>>(tm_d, tm_e16, md, job_off, jobs, acomp, spin, o, err);
    else if (epi == 1)
        density16_kernel<1><<<ctas, kF16Threads, smem, s>>>(tm_d, tm_e16, md, job_off, jobs, acomp, spin, o, err);
    else
        density16_kernel<2><<<ctas, kF16Threads, smem, s>>>(tm_d, tm_e16, md, job_off, jobs, acomp, spin, o, err);
    CGB_CUDA(cudaGetLastError());
}

void launch_combine(long n1, double* rho, const double* rho_b, double* rho1, const double* rho1_b, double* tau,
                    const double* tau_b, int type, cudaStream_t s) {
    const long n3 = 3 * n1;
    combine_kernel<<<(unsigned)((n3 + 255) / 256), 256, 0, s>>>(n1, n3, rho, rho_b, rho1, rho1_b, tau, tau_b, type);
    CGB_CUDA(cudaGetLastError());
}

void launch_prep_z(const MixedDev& md, int type, const double* fcoef, float* Z, float* c2, cudaStream_t s) {
    if (md.ntiles == 0) return;
    prep_z_kernel<<<md.ntiles, 128, 0, s>>>(md, type, fcoef, Z, c2);
    CGB_CUDA(cudaGetLastError());
}

void launch_fock_tc(const CUtensorMap& tm_e32, const CUtensorMap& tm_z, long rows, int ctas, const int* job_off,
                    const FockJob* jobs, const float* c2, int ncomp, double* wpart, int* err, cudaStream_t s) {
    if (ctas == 0) return;
    fock_tc_kernel<<<ctas, kThreads, mixed_smem_bytes(), s>>>(tm_e32, tm_z, rows, job_off, jobs, c2, ncomp, wpart,
                                                             err);
    CGB_CUDA(cudaGetLastError());
}

void launch_split_store_fixed(const float* e32, long rows, int ncomp, bf16* e16d, cudaStream_t s) {
    const long blocks = (long)ncomp * (rows / 64);  // kept rows come in 64-row slots
    if (blocks == 0) return;
    split_store_fixed_kernel<<<(unsigned)blocks, 128, 0, s>>>(e32, rows, ncomp, e16d);
    CGB_CUDA(cudaGetLastError());
}

void launch_split_store(const float* e32, long n, int ncomp, bf16* e16, cudaStream_t s) {
    const long total = n * ncomp;
    if (total == 0) return;
    split_store_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(e32, n, ncomp, e16);
    CGB_CUDA(cudaGetLastError());
}

void launch_prep16(const MixedDev& md, int type, const double* fcoef, bf16* R16, cudaStream_t s) {
    if (md.ntiles == 0) return;
    if (type >= 2)
        prep16_kernel<2><<<md.ntiles, 256, 0, s>>>(md, type, fcoef, R16);
    else
        prep16_kernel<4><<<md.ntiles, 256, 0, s>>>(md, type, fcoef, R16);
    CGB_CUDA(cudaGetLastError());
}

void launch_fock16(const CUtensorMap& tm_l, const CUtensorMap& tm_r, long rows, int ctas, const int* job_off,
                   const FockJob* jobs, int ncomp, double* wpart, int* err, cudaStream_t s) {
    if (ctas == 0) return;
    fock16_kernel<<<ctas, kF16Threads, 2 * kStageBytes + 1024, s>>>(tm_l, tm_r, rows, job_off, jobs, ncomp, wpart,
                                                                     err);
    CGB_CUDA(cudaGetLastError());
}

void launch_axpby(long n, double a, const double* x, double b, const double* y, double* out, cudaStream_t s) {
    if (n <= 0) return;
    axpby_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, a, x, b, y, out);
    CGB_CUDA(cudaGetLastError());
}

void launch_wsum(const double* wpart, const int* item_live, const MolRange* mols, int nmol, int maxn, int spin,
                 int /*nspin*/, double* V, cudaStream_t s) {
    CGB_CHECK(nmol <= 65535, XC_ERR_ARG, "too many molecules in one batch");
    const unsigned t = (unsigned)((maxn + 31) / 32);
    wsum_kernel<<<dim3(t, t, (unsigned)nmol), dim3(32, 32), 0, s>>>(wpart, item_live, mols, spin, V);
    CGB_CUDA(cudaGetLastError());
}

void launch_gather(const long* perm, long Gt, long Gp, int ncomp, const double* src, double* dst, bool zero_pads,
                   cudaStream_t s) {
    if (Gt <= 0) return;
    gather_kernel<<<(unsigned)((Gt + 255) / 256), 256, 0, s>>>(perm, Gt, Gp, ncomp, src, dst, zero_pads);
    CGB_CUDA(cudaGetLastError());
}

void launch_energy_mols(const double* partial, const MolRange* mols, int nmol, double* E, cudaStream_t s) {
    energy_mols_kernel<<<nmol, 256, 0, s>>>(partial, mols, E);
    CGB_CUDA(cudaGetLastError());
}

}  // namespace cgb
