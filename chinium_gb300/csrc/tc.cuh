// Blackwell (sm_103a) building blocks in inline PTX: mbarriers with bounded
// waits, TMA tile loads, tcgen05 TMEM allocation / MMA / commit / load, and
// the shared-memory and instruction descriptors of tcgen05.mma kind::f16.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace cgb {
namespace tc {

// Time budget of one bounded wait (ns of %globaltimer); on exhaustion the
// caller records XC_ERR_TIMEOUT in a global flag and unwinds.
constexpr uint64_t kWaitNs = 2000000000ull;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait for the phase of the given parity; false after budget_ns.
__device__ __forceinline__ bool mbar_wait_budget(uint64_t* bar, uint32_t parity, uint64_t budget_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    for (;;) {
        for (int i = 0; i < 256; i++)
            if (mbar_try_wait(bar, parity)) return true;
        if (globaltimer_ns() - t0 > budget_ns) return false;
    }
}
// The pipelines' wait: false after kWaitNs.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) { return mbar_wait_budget(bar, parity, kWaitNs); }

// 2D TMA tile load global -> shared, completing bytes on bar.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// Shared-memory accesses by 32-bit shared-window address.
__device__ __forceinline__ void sts128(uint32_t addr, const uint4& v) {
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w)
                 : "memory");
}
__device__ __forceinline__ float4 lds128f(uint32_t addr) {
    float4 v;
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(addr));
    return v;
}
__device__ __forceinline__ float lds32f(uint32_t addr) {
    float v;
    asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(addr));
    return v;
}

// --- tcgen05 -----------------------------------------------------------
__device__ __forceinline__ void tmem_alloc(uint32_t* slot_smem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot_smem)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// D(tmem) (+)= A(smem desc) * B(smem desc)^T, issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// D = A B + D / 2 (scale-input-d = 1): halves the accumulator before adding.
__device__ __forceinline__ void mma_bf16_halve_d(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, 1, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p, 1;\n\t}" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc)
        : "memory");
}

// Arrive once on bar when all previously issued MMAs of this thread complete.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 16 consecutive 32-bit TMEM columns of this thread's lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// 16 TMEM columns, load and wait in one statement without a memory clobber:
// TMEM is not memory the compiler tracks, so global loads may be scheduled
// across it (the register outputs are valid when the statement completes).
__device__ __forceinline__ void tmem_ld16_nomem(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// Two 16-column TMEM loads (a at ta, b at tb) and one wait, no memory clobber.
__device__ __forceinline__ void tmem_ld16x2_nomem(uint32_t ta, uint32_t tb, float* a, float* b) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%32];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, "
        "[%33];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(ta), "r"(tb));
#pragma unroll
    for (int i = 0; i < 16; i++) {
        a[i] = __uint_as_float(r[i]);
        b[i] = __uint_as_float(r[16 + i]);
    }
}

// 8 consecutive 32-bit TMEM columns of this thread's lane.
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* v) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 8; i++) v[i] = __uint_as_float(r[i]);
}

// Shared-memory matrix descriptor, K-major operand staged by TMA with 128-byte
// swizzle: rows of 128 B (64 bf16 along K), 8-row atoms 1024 B apart (SBO).
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)(1) << 16;             // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;     // stride byte offset: 8 rows x 128 B
    d |= (uint64_t)1 << 46;               // descriptor version for tcgen05
    d |= (uint64_t)2 << 61;               // 128-byte swizzle
    return d;
}

// MN-major operand staged by TMA with 128-byte swizzle from a [K][MN] array:
// K rows of 128 B (64 bf16 along MN), 8-row groups 1024 B apart (SBO), the
// next 64 MN elements `lbo` bytes on (LBO); a K step of 16 is +2048 B.
__device__ __forceinline__ uint64_t smem_desc_sw128_mn(uint32_t saddr, uint32_t lbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;  // leading byte offset: between 64-element MN blocks
    d |= (uint64_t)(1024 >> 4) << 32;            // stride byte offset: 8 K rows x 128 B
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

// Instruction descriptor of kind::f16: BF16 A and B (K-major), FP32 D.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4)                      // D = F32
           | (1u << 7)                    // A = BF16
           | (1u << 10)                   // B = BF16
           | ((uint32_t)(N >> 3) << 17)   // N / 8
           | ((uint32_t)(M >> 4) << 24);  // M / 16
}
// The same with A MN-major (transpose-A bit).
__host__ __device__ constexpr uint32_t idesc_bf16_amn(int M, int N) { return idesc_bf16(M, N) | (1u << 15); }

// Three-term BF16 split of a double: x ~= h + m + l (relative error ~2^-24).
__device__ __forceinline__ void split3(double x, __nv_bfloat16& h, __nv_bfloat16& m, __nv_bfloat16& l) {
    h = __double2bfloat16(x);
    double r = x - (double)__bfloat162float(h);
    m = __double2bfloat16(r);
    r -= (double)__bfloat162float(m);
    l = __double2bfloat16(r);
}

// Same for a float (the three parts represent it exactly).
__device__ __forceinline__ void split3f(float x, __nv_bfloat16& h, __nv_bfloat16& m, __nv_bfloat16& l) {
    h = __float2bfloat16_rn(x);
    float r = x - __bfloat162float(h);
    m = __float2bfloat16_rn(r);
    r -= __bfloat162float(m);
    l = __float2bfloat16_rn(r);
}

// Binary exponent shared by a group of values for split3_fixed: e with
// 2^e <= max|x| < 2^(e+1), or kFixedZero when the group is negligible
// (max|x| < 2^-100: its slices are zero).
constexpr int kFixedZero = -100000;
__device__ __forceinline__ int fixed_exponent(double maxabs) {
    return maxabs >= 0x1p-100 ? ilogb(maxabs) : kFixedZero;
}

// Three-term split on the fixed-point grid of a group (x ~= h + m + l, error
// <= 2^(e-24)): h, m and l are integer multiples of 2^(e-7), 2^(e-15) and
// 2^(e-23) with at most 8 significant bits (|h| <= 256 units, |m|, |l| <= 128),
// each rounded to nearest and so exact in BF16.  When both operands of a
// product are split this way with one exponent per row of A and per column
// of B over the K range of an accumulation, every hh product of that sum is
// an integer (|.| <= 2^16) times one common power of two, so a K <= 256 sum
// of them is exact in FP32 whatever the order or rounding mode of the
// accumulator: the tensor core's FP32 accumulation adds no error (and no
// truncation bias) to the leading term.
__device__ __forceinline__ void split3_fixed(double x, int e, __nv_bfloat16& h, __nv_bfloat16& m,
                                             __nv_bfloat16& l) {
    if (e == kFixedZero) {
        h = m = l = __double2bfloat16(0.0);
        return;
    }
    const double a = ldexp(rint(ldexp(x, 7 - e)), e - 7);
    const double r1 = x - a;
    const double b = ldexp(rint(ldexp(r1, 15 - e)), e - 15);
    const double r2 = r1 - b;
    const double c = ldexp(rint(ldexp(r2, 23 - e)), e - 23);
    h = __double2bfloat16(a);
    m = __double2bfloat16(b);
    l = __double2bfloat16(c);
}

// 2^k as a float for -126 <= k <= 127.
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((127 + k) << 23); }

// fixed_exponent of a float group maximum from its bits (no FP64): the same
// value as ilogb for every float >= 2^-100.
__device__ __forceinline__ int fixed_exponent_f(float maxabs) {
    return maxabs >= 0x1p-100f ? (int)((__float_as_uint(maxabs) >> 23) & 0xffu) - 127 : kFixedZero;
}

// x rounded to the nearest integer, ties to even (as rintf), for |x| < 2^22:
// adding and removing 1.5 * 2^23 on the FMA pipe (rintf runs on the
// eight-times-slower conversion pipe).
__device__ __forceinline__ float round_small(float x) {
    const float big = 12582912.f;  // 1.5 * 2^23
    return __fsub_rn(__fadd_rn(x, big), big);
}

// The BF16 of a float whose low 16 significand bits are zero (exact: the top
// half of its bits), without a conversion instruction.
__device__ __forceinline__ __nv_bfloat16 bf16_exact(float x) {
    return __ushort_as_bfloat16((unsigned short)(__float_as_uint(x) >> 16));
}

// split3_fixed for a float x, in float arithmetic: every step is exact (scaling
// by powers of two within the normal range, rounding to an integer, exact
// differences), so it gives the same slices as the double version.  The
// scaled values are below 2^8 in magnitude, so round_small rounds them, and
// each slice has at most 8 significant bits, so bf16_exact converts it.
// Needs -100 <= e <= 103 or e == kFixedZero (fixed_exponent of a float group).
__device__ __forceinline__ void split3_fixed_f(float x, int e, __nv_bfloat16& h, __nv_bfloat16& m,
                                               __nv_bfloat16& l) {
    if (e == kFixedZero) {
        h = m = l = __float2bfloat16_rn(0.f);
        return;
    }
    // slice = round_small(v * 2^k) * 2^-k as two exact FMAs: t = v 2^k + B
    // rounds the (exact) scaled value to an integer offset by B = 1.5 * 2^23,
    // and t 2^-k - B 2^-k is that integer times 2^-k, exactly representable
    const float big = 12582912.f;
    const float s1 = pow2f(7 - e), s2 = pow2f(15 - e), s3 = pow2f(23 - e);
    const float i1 = pow2f(e - 7), i2 = pow2f(e - 15), i3 = pow2f(e - 23);
    const float a = __fmaf_rn(__fmaf_rn(x, s1, big), i1, -big * i1);
    const float r1 = __fsub_rn(x, a);
    const float b = __fmaf_rn(__fmaf_rn(r1, s2, big), i2, -big * i2);
    const float r2 = __fsub_rn(r1, b);
    const float c = __fmaf_rn(__fmaf_rn(r2, s3, big), i3, -big * i3);
    h = bf16_exact(a);
    m = bf16_exact(b);
    l = bf16_exact(c);
}

// split3_fixed_f of two values that share the exponent e (adjacent functions
// of one point), with packed FP32x2 instructions: the same slices bit for
// bit (each lane rounds to nearest as the scalar operations do), as BF16
// pairs (x in the low half, as __halves2bfloat162).
__device__ __forceinline__ uint32_t bf16x2_exact(float2 a) {
    return __byte_perm(__float_as_uint(a.x), __float_as_uint(a.y), 0x7632);
}
__device__ __forceinline__ void split3_fixed_f2(float2 x, int e, uint32_t& h, uint32_t& m, uint32_t& l) {
    if (e == kFixedZero) {
        h = m = l = 0u;  // +0 in both halves
        return;
    }
    const float big = 12582912.f;
    const float2 B = make_float2(big, big), neg1 = make_float2(-1.f, -1.f);
    const float p1 = pow2f(7 - e), p2 = pow2f(15 - e), p3 = pow2f(23 - e);
    const float q1 = pow2f(e - 7), q2 = pow2f(e - 15), q3 = pow2f(e - 23);
    const float2 a = __ffma2_rn(__ffma2_rn(x, make_float2(p1, p1), B), make_float2(q1, q1),
                                make_float2(-big * q1, -big * q1));
    const float2 r1 = __ffma2_rn(a, neg1, x);  // x - a, exact
    const float2 b = __ffma2_rn(__ffma2_rn(r1, make_float2(p2, p2), B), make_float2(q2, q2),
                                make_float2(-big * q2, -big * q2));
    const float2 r2 = __ffma2_rn(b, neg1, r1);
    const float2 c = __ffma2_rn(__ffma2_rn(r2, make_float2(p3, p3), B), make_float2(q3, q3),
                                make_float2(-big * q3, -big * q3));
    h = bf16x2_exact(a);
    m = bf16x2_exact(b);
    l = bf16x2_exact(c);
}

}  // namespace tc
}  // namespace cgb
