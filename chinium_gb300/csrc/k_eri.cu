// Electron-repulsion integrals (McMurchie-Davidson, FP64) and their
// contraction into Coulomb and exchange matrices: the GPU counterpart of the
// reference's in-core Int4C2E (CalculateIntegrals, then ContractInts /
// Gunified every SCF iteration, src/Integral/Int4C2E.cpp:567-683).
//
// eri_kernel: one CTA (128 threads) per shell quartet of the screened list.
// Per primitive quartet the threads evaluate the Boys function F_0..F_L
// (tabulated Taylor expansion), the Hermite Coulomb integrals R_tuv by the
// MD recursion level by level in shared memory, the ket half-transform
//   X[cd][h] = sum_h' (-1)^|h'| Ep_cd[cd][h'] R_{h + h'}
// and the bra contraction I[ab][cd] += pre sum_h Ep_ab[ab][h] X[cd][h].
// The block of pure integrals [fa][fb][fc][fd] is written once.
//
// jk_slab_kernel (in-core store, split once into float-float pairs): one CTA
// per run of quartets of one bra pair; lanes form elements of the six J / K
// sub-blocks each quartet feeds (2 J, 4 K) in float-float arithmetic on the
// FP32 pipe, the exchange elements summed in a shared-memory slab of the bra
// shells' rows and added to HBM once per run.  jk_contract_kernel (FP64
// store: integral-direct chunks, or slabs too large for shared memory): one
// warp per quartet block, one FP64 atomic per element.  Small molecules take J from
// a dense Coulomb operator over function pairs filled once from the blocks
// (coulomb_scatter_kernel, then split into float-float pairs) and a GEMV per
// build in float-float arithmetic on the FP32 pipe (coulomb_gemv_kernel).
#include "common.h"
#include "eri.h"

namespace cgb {
namespace {

constexpr int kEriThreads = 128;
constexpr int kHMax = herm_count(kEriMaxLt);        // 455
constexpr int kHabMax = herm_count(2 * kEriMaxL);   // 84
constexpr int kNf = 2 * kEriMaxL + 1;               // 7 pure functions per shell at most
constexpr int kXMax = kNf * kNf * kHabMax;          // 4116
constexpr int kIMax = kNf * kNf * kNf * kNf;        // 2401

// (t | u << 8 | v << 16 | (t + u + v) << 24) of Hermite index h.
__constant__ unsigned c_tuv[kHMax];

__device__ __forceinline__ int hidx(int t, int u, int v) {
    const int N = t + u + v, a = N - t;
    return N * (N + 1) * (N + 2) / 6 + a * (a + 1) / 2 + (a - u);
}

// F_n(T): Taylor expansion about the nearest table point (|dT| <= 0.025,
// seven terms: relative error ~1e-15), asymptotic form beyond the table.
__device__ __forceinline__ double boys_n(int n, double T, const double* __restrict__ tab) {
    if (T >= kBoysTmax) {
        double f = 0.5 * sqrt(3.14159265358979323846 / T);
        for (int k = 1; k <= n; k++) f *= (2 * k - 1) / (2.0 * T);
        return f;
    }
    const int i = (int)(T * (1.0 / kBoysStep) + 0.5);
    const double x = i * kBoysStep - T;
    const double* row = tab + (size_t)i * kBoysCols + n;
    double r = __ldg(row + 6);
#pragma unroll
    for (int k = 5; k >= 0; k--) r = __ldg(row + k) + r * x * (1.0 / (k + 1));
    return r;
}

struct EriSmem {
    double R[2][kHMax];
    double X[kXMax];
    double I[kIMax];
    double F[kEriMaxLt + 1];
    double sc[6];  // alpha, X_PQ, Y_PQ, Z_PQ, T, prefactor
};

__global__ void __launch_bounds__(kEriThreads) eri_kernel(EriDev e, const int2* __restrict__ quartets,
                                                          const long long* __restrict__ out_off, long long q0,
                                                          long long base, double* __restrict__ out) {
    extern __shared__ double smem_d[];
    EriSmem& sm = *reinterpret_cast<EriSmem*>(smem_d);
    const long long q = q0 + blockIdx.x;
    const int tid = threadIdx.x;
    const int2 pq = quartets[q];
    const EriPair P = e.pairs[pq.x], Q = e.pairs[pq.y];
    const int Lab = P.la + P.lb, Lcd = Q.la + Q.lb, L = Lab + Lcd;
    const int Hab = herm_count(Lab), Hcd = herm_count(Lcd);
    const int nab = P.na * P.nb, ncd = Q.na * Q.nb, nI = nab * ncd, nX = ncd * Hab;
    for (int i = tid; i < nI; i += kEriThreads) sm.I[i] = 0.0;
    for (int ij = 0; ij < P.npp; ij++) {
        const int pi = P.pp0 + ij;
        const double p = e.pp_p[pi];
        const double* __restrict__ Eab = e.ep + P.ep0 + (long long)ij * nab * Hab;
        for (int kl = 0; kl < Q.npp; kl++) {
            const int qi = Q.pp0 + kl;
            const double* __restrict__ Ecd = e.ep + Q.ep0 + (long long)kl * ncd * Hcd;
            if (tid == 0) {
                const double qq = e.pp_p[qi];
                const double alpha = p * qq / (p + qq);
                const double X = e.pp_P[3 * pi] - e.pp_P[3 * qi], Y = e.pp_P[3 * pi + 1] - e.pp_P[3 * qi + 1],
                             Z = e.pp_P[3 * pi + 2] - e.pp_P[3 * qi + 2];
                sm.sc[0] = alpha;
                sm.sc[1] = X;
                sm.sc[2] = Y;
                sm.sc[3] = Z;
                sm.sc[4] = alpha * (X * X + Y * Y + Z * Z);
                sm.sc[5] = 34.98683665524972 / (p * qq * sqrt(p + qq));  // 2 pi^(5/2)
            }
            __syncthreads();
            const double alpha = sm.sc[0], Xp = sm.sc[1], Yp = sm.sc[2], Zp = sm.sc[3], T = sm.sc[4];
            if (tid <= L) {
                // (-2 alpha)^n F_n(T): the level-n value of R_000
                double m = 1.0;
                for (int k = 0; k < tid; k++) m *= -2.0 * alpha;
                sm.F[tid] = m * boys_n(tid, T, e.boys);
            }
            __syncthreads();
            // MD recursion, level n = L .. 0 (level n holds N <= L - n), ping-pong buffers
            if (tid == 0) sm.R[L & 1][0] = sm.F[L];
            __syncthreads();
            for (int n = L - 1; n >= 0; n--) {
                const int b = n & 1, hn = herm_count(L - n);
                const double* __restrict__ up = sm.R[b ^ 1];
                for (int h = tid; h < hn; h += kEriThreads) {
                    double v;
                    if (h == 0) {
                        v = sm.F[n];
                    } else {
                        const unsigned c = c_tuv[h];
                        const int t = c & 255, u = (c >> 8) & 255, w = (c >> 16) & 255;
                        if (t > 0) {
                            v = Xp * up[hidx(t - 1, u, w)];
                            if (t > 1) v += (t - 1) * up[hidx(t - 2, u, w)];
                        } else if (u > 0) {
                            v = Yp * up[hidx(t, u - 1, w)];
                            if (u > 1) v += (u - 1) * up[hidx(t, u - 2, w)];
                        } else {
                            v = Zp * up[hidx(t, u, w - 1)];
                            if (w > 1) v += (w - 1) * up[hidx(t, u, w - 2)];
                        }
                    }
                    sm.R[b][h] = v;
                }
                __syncthreads();
            }
            const double* __restrict__ R0 = sm.R[0];
            // ket half-transform
            for (int i = tid; i < nX; i += kEriThreads) {
                const int cd = i / Hab, ha = i - cd * Hab;
                const unsigned c1 = c_tuv[ha];
                const int t1 = c1 & 255, u1 = (c1 >> 8) & 255, v1 = (c1 >> 16) & 255;
                const double* __restrict__ ec = Ecd + cd * Hcd;
                double acc = 0.0;
                for (int hc = 0; hc < Hcd; hc++) {
                    const unsigned c2 = c_tuv[hc];
                    const double term = __ldg(ec + hc) * R0[hidx(t1 + (c2 & 255), u1 + ((c2 >> 8) & 255),
                                                                v1 + ((c2 >> 16) & 255))];
                    acc += ((c2 >> 24) & 1) ? -term : term;
                }
                sm.X[i] = acc;
            }
            __syncthreads();
            const double pre = sm.sc[5];
            for (int i = tid; i < nI; i += kEriThreads) {
                const int ab = i / ncd, cd = i - ab * ncd;
                const double* __restrict__ ea = Eab + ab * Hab;
                const double* __restrict__ x = sm.X + cd * Hab;
                double acc = 0.0;
                for (int h = 0; h < Hab; h++) acc = fma(__ldg(ea + h), x[h], acc);
                sm.I[i] = fma(pre, acc, sm.I[i]);
            }
            __syncthreads();
        }
    }
    double* o = out + (out_off[q] - base);
    for (int i = tid; i < nI; i += kEriThreads) o[i] = sm.I[i];
}

// One warp per quartet block (persistent grid, quartets strided over the
// warps): each lane forms elements of the sub-blocks rawJ(a, b), rawJ(c, d),
// rawK(a, c), rawK(b, d), rawK(a, d), rawK(b, c) of every matrix -- one
// slice sum of the block times D each -- and adds it with one FP64 atomic.
// The block's lines are read from HBM once and re-read from L1 by the six
// slices (D symmetric, n x n; row-major and column-major alike).  rawJ or
// rawK may be null (that half is skipped).
constexpr int kJkWarps = 8;
__global__ void __launch_bounds__(32 * kJkWarps) jk_contract_kernel(EriDev e, const int2* __restrict__ quartets,
                                                                    const long long* __restrict__ out_off,
                                                                    long long q0, long long nq, long long base,
                                                                    const double* __restrict__ ints, int n, int nmat,
                                                                    const double* __restrict__ D,
                                                                    double* __restrict__ rawJ,
                                                                    double* __restrict__ rawK) {
    const int lane = threadIdx.x & 31;
    const long long w0 = (long long)blockIdx.x * kJkWarps + (threadIdx.x >> 5);
    const long long nw = (long long)gridDim.x * kJkWarps;
    const size_t nn = (size_t)n * n;
    for (long long qq = w0; qq < nq; qq += nw) {
        const long long q = q0 + qq;
        const int2 pq = quartets[q];
        const EriPair P = e.pairs[pq.x], Q = e.pairs[pq.y];
        const int na = P.na, nb = P.nb, nc = Q.na, nd = Q.nb;
        const double* __restrict__ blk = ints + (out_off[q] - base);
        // degeneracy of the canonical quartet (a >= b, c >= d, bra pair >= ket pair)
        const int sa = P.fa, sb = P.fb, sc = Q.fa, sd = Q.fb;
        double f = 1.0;
        if (sa == sb) f *= 0.5;
        if (sc == sd) f *= 0.5;
        if (pq.x == pq.y) f *= 0.5;
        const int nJ1 = na * nb, nJ2 = nc * nd, nK1 = na * nc, nK2 = nb * nd, nK3 = na * nd, nK4 = nb * nc;
        const int nJ = rawJ ? nJ1 + nJ2 : 0;
        const int tot = nJ + (rawK ? nK1 + nK2 + nK3 + nK4 : 0);
        const int sab = nb * nc * nd, sbb = nc * nd;  // strides of ia, ib in the block
        for (int m = 0; m < nmat; m++) {
            const double* __restrict__ Dm = D + m * nn;
            for (int k = lane; k < tot; k += 32) {
                double acc = 0.0;
                size_t dst;
                double* out;
                if (k < nJ && k < nJ1) {  // rawJ(a, b) += f sum_cd I D(c, d)
                    const int ia = k / nb, ib = k - ia * nb;
                    const double* bl = blk + ia * sab + ib * sbb;
                    for (int ic = 0; ic < nc; ic++)
                        for (int id = 0; id < nd; id++)
                            acc = fma(__ldg(bl + ic * nd + id), __ldg(Dm + (size_t)(sc + ic) * n + sd + id), acc);
                    dst = (size_t)(sa + ia) * n + sb + ib;
                    out = rawJ;
                } else if (k < nJ) {  // rawJ(c, d) += f sum_ab I D(a, b)
                    const int r = k - nJ1, ic = r / nd, id = r - ic * nd;
                    const double* bl = blk + ic * nd + id;
                    for (int ia = 0; ia < na; ia++)
                        for (int ib = 0; ib < nb; ib++)
                            acc = fma(__ldg(bl + ia * sab + ib * sbb), __ldg(Dm + (size_t)(sa + ia) * n + sb + ib), acc);
                    dst = (size_t)(sc + ic) * n + sd + id;
                    out = rawJ;
                } else {
                    int r = k - nJ;
                    out = rawK;
                    if (r < nK1) {  // rawK(a, c) += f sum_bd I D(b, d)
                        const int ia = r / nc, ic = r - ia * nc;
                        for (int ib = 0; ib < nb; ib++)
                            for (int id = 0; id < nd; id++)
                                acc = fma(__ldg(blk + ia * sab + ib * sbb + ic * nd + id),
                                          __ldg(Dm + (size_t)(sb + ib) * n + sd + id), acc);
                        dst = (size_t)(sa + ia) * n + sc + ic;
                    } else if ((r -= nK1) < nK2) {  // rawK(b, d) += f sum_ac I D(a, c)
                        const int ib = r / nd, id = r - ib * nd;
                        for (int ia = 0; ia < na; ia++)
                            for (int ic = 0; ic < nc; ic++)
                                acc = fma(__ldg(blk + ia * sab + ib * sbb + ic * nd + id),
                                          __ldg(Dm + (size_t)(sa + ia) * n + sc + ic), acc);
                        dst = (size_t)(sb + ib) * n + sd + id;
                    } else if ((r -= nK2) < nK3) {  // rawK(a, d) += f sum_bc I D(b, c)
                        const int ia = r / nd, id = r - ia * nd;
                        for (int ib = 0; ib < nb; ib++)
                            for (int ic = 0; ic < nc; ic++)
                                acc = fma(__ldg(blk + ia * sab + ib * sbb + ic * nd + id),
                                          __ldg(Dm + (size_t)(sb + ib) * n + sc + ic), acc);
                        dst = (size_t)(sa + ia) * n + sd + id;
                    } else {  // rawK(b, c) += f sum_ad I D(a, d)
                        r -= nK3;
                        const int ib = r / nc, ic = r - ib * nc;
                        for (int ia = 0; ia < na; ia++)
                            for (int id = 0; id < nd; id++)
                                acc = fma(__ldg(blk + ia * sab + ib * sbb + ic * nd + id),
                                          __ldg(Dm + (size_t)(sa + ia) * n + sd + id), acc);
                        dst = (size_t)(sb + ib) * n + sc + ic;
                    }
                }
                atomicAdd(out + m * nn + dst, f * acc);
            }
        }
    }
}

// Dense Coulomb operator of small molecules: M[(mu nu), (la si)] =
// (mu nu|la si) over packed pairs mu >= nu (p = mu (mu + 1) / 2 + nu), filled
// once from the in-core quartet blocks (warp per quartet, both (P, Q) and
// (Q, P) entries; screened-out quartets stay zero), rows of stride ld (npair
// rounded up to even, the pad column zero).  J of a density is then M d with
// d_p = D(mu, nu) (x 2 off the diagonal): a GEMV that streams M from HBM once
// per build.
__device__ __forceinline__ long long pair_index(int i, int j) {
    return i >= j ? (long long)i * (i + 1) / 2 + j : (long long)j * (j + 1) / 2 + i;
}

__global__ void __launch_bounds__(256) coulomb_scatter_kernel(EriDev e, const int2* __restrict__ quartets,
                                                              const long long* __restrict__ out_off, long long nq,
                                                              const double* __restrict__ ints, long long ld,
                                                              double* __restrict__ M) {
    const int lane = threadIdx.x & 31;
    const long long w0 = (long long)blockIdx.x * 8 + (threadIdx.x >> 5), nw = (long long)gridDim.x * 8;
    for (long long q = w0; q < nq; q += nw) {
        const int2 pq = quartets[q];
        const EriPair P = e.pairs[pq.x], Q = e.pairs[pq.y];
        const int nb = P.nb, nc = Q.na, nd = Q.nb, ncd = nc * nd, nI = P.na * nb * ncd;
        const double* __restrict__ blk = ints + out_off[q];
        for (int k = lane; k < nI; k += 32) {
            const int ab = k / ncd, cd = k - ab * ncd;
            const int ia = ab / nb, ib = ab - ia * nb, ic = cd / nd, id = cd - ic * nd;
            const long long p1 = pair_index(P.fa + ia, P.fb + ib), p2 = pair_index(Q.fa + ic, Q.fb + id);
            const double v = blk[k];
            M[p1 * ld + p2] = v;
            M[p2 * ld + p1] = v;
        }
    }
}

// The dense operator and the packed densities are float-float pairs: an FP64
// value v is held as (hi, lo) = (fl32(v), fl32(v - hi)), 48 significant bits,
// so the GEMV runs on the FP32 pipe (GB300's FP64 rate is 1/64 of it) at
// FP64-level accuracy, in the same 8 bytes per element as FP64.
__device__ __forceinline__ float2 ff_split(double v) {
    const float hi = (float)v;
    return make_float2(hi, (float)(v - (double)hi));
}

// In place: M[i] (FP64) -> (hi, lo) float pair in the same 8 bytes.
__global__ void coulomb_split_kernel(long long n, double* __restrict__ M) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double v = M[i];
        reinterpret_cast<float2*>(M)[i] = ff_split(v);
    }
}

// d_p of nmat densities (n x n each) -> x[m][p] as float-float pairs
// (vectors of stride ld)
__global__ void coulomb_pack_kernel(int n, int nmat, long long npair, const double* __restrict__ D,
                                    float2* __restrict__ x) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n * n * nmat) return;
    const int m = (int)(t / ((long long)n * n));
    const long long r = t - (long long)m * n * n;
    const int i = (int)(r / n), j = (int)(r - (long long)i * n);
    if (j > i) return;
    x[m * npair + pair_index(i, j)] = ff_split((i == j ? 1.0 : 2.0) * D[t]);
}

// s + c += (mh + ml)(xh + xl) in float-float: the product's rounding error
// exactly (FMA), the sum's by TwoSum (Knuth); explicit _rn intrinsics keep
// the compiler from contracting the error-free transformations.
__device__ __forceinline__ void ff_fma(float mh, float ml, float xh, float xl, float& s, float& c) {
    const float p = __fmul_rn(mh, xh);
    const float e = __fmaf_rn(mh, xh, -p);
    const float t = __fadd_rn(s, p);
    const float z = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z));
    s = t;
    c = __fadd_rn(c, __fadd_rn(__fadd_rn(err, e), __fmaf_rn(mh, xl, __fmul_rn(ml, xh))));
}

// float -> double from the bit pattern (integer pipe; GB300's FP64 pipe,
// which also converts, runs at 1/64 of the FP32 rate).  Normal numbers are
// exact; zero and subnormals (below 1.2e-38) give 0.
__device__ __forceinline__ double f32_to_f64(float x) {
    const unsigned u = __float_as_uint(x);
    const unsigned ex = (u >> 23) & 0xffu;
    if (ex == 0) return 0.0;
    const unsigned long long b = ((unsigned long long)(u & 0x80000000u) << 32) |
                                 ((unsigned long long)(ex + 896u) << 52) |
                                 ((unsigned long long)(u & 0x7fffffu) << 29);
    return __longlong_as_double((long long)b);
}

// FP64 value of the float-float pair (s, c) scaled by f, a power of two
// (exact in FP32): one FP64 add.
__device__ __forceinline__ double ff_scaled(float s, float c, float f) {
    return f32_to_f64(s * f) + f32_to_f64(c * f);
}

// Exchange and Coulomb by bra pair (in-core list, float-float store).  The
// quartets of one bra pair P = (a, b) are consecutive in the list, and every
// exchange element they feed lies in a row of shell a or of shell b:
// K(a, c), K(a, d), K(b, c), K(b, d).  A CTA takes one run of them (a
// chunk), adds its K contributions into a shared-memory slab of those
// na + nb rows x n columns (per matrix) and its J(a, b) contributions into a
// small shared buffer, and adds both to the raw accumulators once at the
// end: one FP64 global atomic per touched slab element instead of one per
// element and quartet.  The J(c, d) contributions (a different ket pair per
// quartet) stay global atomics.  Warps take the chunk's quartets in turn,
// lanes the sub-block elements (one slice sum of the block times D each, as
// in jk_contract_kernel).  The integrals and densities are float-float pairs
// (hi, lo) and the slice sums run in float-float on the FP32 pipe; each sum
// enters the FP64 slab with one FP64 add.  Shared layout: nmat x kNf^2
// J(a, b) entries, then (kK) nmat x rows x n slab entries (rows = na + nb
// <= rows_cap, the launch's size).
template <bool kJ, bool kK>
__global__ void __launch_bounds__(32 * kJkWarps) jk_slab_kernel(EriDev e, const int2* __restrict__ quartets,
                                                                const long long* __restrict__ out_off,
                                                                const longlong2* __restrict__ chunks, int rows_cap,
                                                                const float2* __restrict__ ints, int n, int nmat,
                                                                const float2* __restrict__ D,
                                                                double* __restrict__ rawJ,
                                                                double* __restrict__ rawK) {
    extern __shared__ double sm_slab[];
    const longlong2 ch = chunks[blockIdx.x];
    const int2 pq0 = quartets[ch.x];
    const EriPair P = e.pairs[pq0.x];
    const int na = P.na, nb = P.nb, sa = P.fa, sb = P.fb, rows = na + nb;
    if (kK && rows > rows_cap) return;  // chunks are grouped by rows on the host; never taken
    const int slab = kK ? rows * n : 0;
    const size_t nn = (size_t)n * n;
    double* __restrict__ j1 = sm_slab;                             // [m][ia * nb + ib]
    double* __restrict__ ks = sm_slab + (size_t)nmat * kNf * kNf;  // [m][row][col]
    for (int t = threadIdx.x; t < nmat * (kNf * kNf + slab); t += blockDim.x) sm_slab[t] = 0.0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const float fab = sa == sb ? 0.5f : 1.0f;
    const int nJ1 = na * nb;
    for (long long q = ch.x + (threadIdx.x >> 5); q < ch.y; q += kJkWarps) {
        const int2 pq = quartets[q];
        const EriPair Q = e.pairs[pq.y];
        const int nc = Q.na, nd = Q.nb, sc = Q.fa, sd = Q.fb;
        const float2* __restrict__ blk = ints + out_off[q];
        float f = fab;
        if (sc == sd) f *= 0.5f;
        if (pq.x == pq.y) f *= 0.5f;
        const int nJ2 = nc * nd, nK1 = na * nc, nK2 = nb * nd, nK3 = na * nd;
        const int nJ = kJ ? nJ1 + nJ2 : 0;
        const int tot = nJ + (kK ? nK1 + nK2 + nK3 + nb * nc : 0);
        const int sab = nb * nc * nd, sbb = nc * nd;  // strides of ia, ib in the block
        for (int m = 0; m < nmat; m++) {
            const float2* __restrict__ Dm = D + m * nn;
            double* __restrict__ km = ks + (size_t)m * slab;
            for (int k = lane; k < tot; k += 32) {
                float s = 0.f, c = 0.f;
                double* dst;
                if (k < nJ && k < nJ1) {  // J(a, b) += f sum_cd I D(c, d): shared
                    const int ia = k / nb, ib = k - ia * nb;
                    const float2* bl = blk + ia * sab + ib * sbb;
                    for (int ic = 0; ic < nc; ic++)
                        for (int id = 0; id < nd; id++) {
                            const float2 v = bl[ic * nd + id], x = Dm[(size_t)(sc + ic) * n + sd + id];
                            ff_fma(v.x, v.y, x.x, x.y, s, c);
                        }
                    dst = j1 + m * kNf * kNf + k;
                } else if (k < nJ) {  // J(c, d) += f sum_ab I D(a, b): global
                    const int r = k - nJ1, ic = r / nd, id = r - ic * nd;
                    const float2* bl = blk + ic * nd + id;
                    for (int ia = 0; ia < na; ia++)
                        for (int ib = 0; ib < nb; ib++) {
                            const float2 v = bl[ia * sab + ib * sbb], x = Dm[(size_t)(sa + ia) * n + sb + ib];
                            ff_fma(v.x, v.y, x.x, x.y, s, c);
                        }
                    dst = rawJ + m * nn + (size_t)(sc + ic) * n + sd + id;
                } else {
                    int r = k - nJ;
                    if (r < nK1) {  // K(a, c) += f sum_bd I D(b, d): slab row ia
                        const int ia = r / nc, ic = r - ia * nc;
                        for (int ib = 0; ib < nb; ib++)
                            for (int id = 0; id < nd; id++) {
                                const float2 v = blk[ia * sab + ib * sbb + ic * nd + id];
                                const float2 x = Dm[(size_t)(sb + ib) * n + sd + id];
                                ff_fma(v.x, v.y, x.x, x.y, s, c);
                            }
                        dst = km + ia * n + sc + ic;
                    } else if ((r -= nK1) < nK2) {  // K(b, d) += f sum_ac I D(a, c): slab row na + ib
                        const int ib = r / nd, id = r - ib * nd;
                        for (int ia = 0; ia < na; ia++)
                            for (int ic = 0; ic < nc; ic++) {
                                const float2 v = blk[ia * sab + ib * sbb + ic * nd + id];
                                const float2 x = Dm[(size_t)(sa + ia) * n + sc + ic];
                                ff_fma(v.x, v.y, x.x, x.y, s, c);
                            }
                        dst = km + (na + ib) * n + sd + id;
                    } else if ((r -= nK2) < nK3) {  // K(a, d) += f sum_bc I D(b, c): slab row ia
                        const int ia = r / nd, id = r - ia * nd;
                        for (int ib = 0; ib < nb; ib++)
                            for (int ic = 0; ic < nc; ic++) {
                                const float2 v = blk[ia * sab + ib * sbb + ic * nd + id];
                                const float2 x = Dm[(size_t)(sb + ib) * n + sc + ic];
                                ff_fma(v.x, v.y, x.x, x.y, s, c);
                            }
                        dst = km + ia * n + sd + id;
                    } else {  // K(b, c) += f sum_ad I D(a, d): slab row na + ib
                        r -= nK3;
                        const int ib = r / nc, ic = r - ib * nc;
                        for (int ia = 0; ia < na; ia++)
                            for (int id = 0; id < nd; id++) {
                                const float2 v = blk[ia * sab + ib * sbb + ic * nd + id];
                                const float2 x = Dm[(size_t)(sa + ia) * n + sd + id];
                                ff_fma(v.x, v.y, x.x, x.y, s, c);
                            }
                        dst = km + (na + ib) * n + sc + ic;
                    }
                }
                atomicAdd(dst, ff_scaled(s, c, f));
            }
        }
    }
    __syncthreads();
    if constexpr (kK) {
        // slab row r < na is function sa + r, row na + r' is function sb + r'
        for (int t = threadIdx.x; t < nmat * slab; t += blockDim.x) {
            const double v = ks[t];
            if (v == 0.0) continue;  // columns no ket of the chunk touched
            const int m = t / slab, r = t - m * slab, row = r / n, col = r - row * n;
            const int fn = row < na ? sa + row : sb + (row - na);
            atomicAdd(rawK + m * nn + (size_t)fn * n + col, v);
        }
    }
    if constexpr (kJ) {
        for (int t = threadIdx.x; t < nmat * nJ1; t += blockDim.x) {
            const int m = t / nJ1, r = t - m * nJ1, ia = r / nb, ib = r - ia * nb;
            const double v = j1[m * kNf * kNf + r];
            if (v != 0.0) atomicAdd(rawJ + m * nn + (size_t)(sa + ia) * n + sb + ib, v);
        }
    }
}

// nmat densities (FP64) -> float-float pairs, out of place
__global__ void jk_split_density_kernel(long long count, const double* __restrict__ D, float2* __restrict__ out) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x)
        out[i] = ff_split(D[i]);
}

// y[m] = M x[m] for NM <= 4 vectors in one pass over M (npair rows of
// stride npair here being the even row stride ld): one warp per row, four
// independent 16-byte loads (two float-float elements each) of M per lane in
// flight per step (a single outstanding load per warp leaves HBM at ~10% of
// its rate).  Lanes accumulate in float-float and reduce in FP64.
constexpr int kGemvMaxVec = 4;
template <int NM>
__global__ void __launch_bounds__(256) coulomb_gemv_kernel(long long npair, const float2* __restrict__ M,
                                                           const float2* __restrict__ x, double* __restrict__ y) {
    const int lane = threadIdx.x & 31;
    const long long w0 = (long long)blockIdx.x * 8 + (threadIdx.x >> 5), nw = (long long)gridDim.x * 8;
    const long long nc2 = npair / 2;
    for (long long r = w0; r < npair; r += nw) {
        const float4* __restrict__ row2 = reinterpret_cast<const float4*>(M + r * npair);
        float s[NM], c[NM];
#pragma unroll
        for (int m = 0; m < NM; m++) s[m] = c[m] = 0.f;
        long long k = lane;
        for (; k + 96 < nc2; k += 128) {
            float4 v[4];
#pragma unroll
            for (int u = 0; u < 4; u++) v[u] = __ldcs(row2 + k + 32 * u);
#pragma unroll
            for (int m = 0; m < NM; m++) {
                const float4* __restrict__ x2 = reinterpret_cast<const float4*>(x + m * npair);
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    const float4 xv = __ldg(x2 + k + 32 * u);
                    ff_fma(v[u].x, v[u].y, xv.x, xv.y, s[m], c[m]);
                    ff_fma(v[u].z, v[u].w, xv.z, xv.w, s[m], c[m]);
                }
            }
        }
        for (; k < nc2; k += 32) {
            const float4 v = __ldcs(row2 + k);
#pragma unroll
            for (int m = 0; m < NM; m++) {
                const float4 xv = __ldg(reinterpret_cast<const float4*>(x + m * npair) + k);
                ff_fma(v.x, v.y, xv.x, xv.y, s[m], c[m]);
                ff_fma(v.z, v.w, xv.z, xv.w, s[m], c[m]);
            }
        }
#pragma unroll
        for (int m = 0; m < NM; m++) {
            double v = (double)s[m] + (double)c[m];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if (lane == 0) y[m * npair + r] = v;
        }
    }
}

// J[m](i, j) = y[m][p(i, j)]
__global__ void coulomb_unpack_kernel(int n, int nmat, long long npair, const double* __restrict__ y,
                                      double* __restrict__ J) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n * n * nmat) return;
    const int m = (int)(t / ((long long)n * n));
    const long long r = t - (long long)m * n * n;
    const int i = (int)(r / n), j = (int)(r - (long long)i * n);
    J[t] = y[m * npair + pair_index(i, j)];
}

__global__ void jk_symmetrise_kernel(int n, int nmat, const double* __restrict__ rawJ, const double* __restrict__ rawK,
                                     double* __restrict__ J, double* __restrict__ K) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long nn = (long long)n * n;
    if (i >= nn * nmat) return;
    const long long m = i / nn, r = i - m * nn;
    const int a = (int)(r / n), b = (int)(r - (long long)a * n);
    const long long t = m * nn + (long long)b * n + a;
    if (J) J[i] = 2.0 * (rawJ[i] + rawJ[t]);
    if (K) K[i] = rawK[i] + rawK[t];
}

}  // namespace

void set_eri_kernel_attributes() {
    CGB_CUDA(cudaFuncSetAttribute(eri_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(EriSmem)));
    CGB_CUDA(cudaFuncSetAttribute(jk_slab_kernel<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kJkSlabMaxBytes));
    CGB_CUDA(cudaFuncSetAttribute(jk_slab_kernel<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kJkSlabMaxBytes));
    CGB_CUDA(cudaFuncSetAttribute(jk_slab_kernel<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kJkSlabMaxBytes));
    static bool tables = false;
    if (!tables) {
        unsigned h[kHMax];
        for (int N = 0; N <= kEriMaxLt; N++)
            for (int t = N; t >= 0; t--)
                for (int u = N - t; u >= 0; u--) {
                    const int v = N - t - u, a = N - t;
                    const int i = N * (N + 1) * (N + 2) / 6 + a * (a + 1) / 2 + (a - u);
                    h[i] = (unsigned)t | ((unsigned)u << 8) | ((unsigned)v << 16) | ((unsigned)N << 24);
                }
        CGB_CUDA(cudaMemcpyToSymbol(c_tuv, h, sizeof(h)));
        tables = true;
    }
}

void launch_eri(const EriDev& e, const int2* quartets, const long long* out_off, long long q0, long long nq,
                long long base, double* out, cudaStream_t s) {
    for (long long c = 0; c < nq; c += (1LL << 30)) {
        const long long m = nq - c < (1LL << 30) ? nq - c : (1LL << 30);
        eri_kernel<<<(unsigned)m, kEriThreads, sizeof(EriSmem), s>>>(e, quartets, out_off, q0 + c, base, out);
        CGB_CUDA(cudaGetLastError());
    }
}

void launch_jk_contract(const EriDev& e, const int2* quartets, const long long* out_off, long long q0, long long nq,
                        long long base, const double* ints, int n, int nmat, const double* D, double* rawJ,
                        double* rawK, cudaStream_t s) {
    if (nq <= 0 || (!rawJ && !rawK)) return;
    int dev = 0, sms = 0;
    CGB_CUDA(cudaGetDevice(&dev));
    CGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const long long want = (nq + kJkWarps - 1) / kJkWarps;
    const unsigned blocks = (unsigned)(want < (long long)sms * 8 ? want : (long long)sms * 8);
    jk_contract_kernel<<<blocks, 32 * kJkWarps, 0, s>>>(e, quartets, out_off, q0, nq, base, ints, n, nmat, D, rawJ,
                                                      rawK);
    CGB_CUDA(cudaGetLastError());
}

size_t jk_slab_bytes(int rows, int n, int nmat) {
    return (size_t)nmat * ((size_t)kNf * kNf + (size_t)rows * n) * sizeof(double);
}

void launch_jk_slab(const EriDev& e, const int2* quartets, const long long* out_off, const longlong2* chunks,
                    const std::vector<int>& cls_rows, const std::vector<long long>& cls_c0, const float2* ints, int n,
                    int nmat, const double* D, float2* Dff, double* rawJ, double* rawK, cudaStream_t s) {
    CGB_CHECK((rawJ || rawK) && cls_c0.size() == cls_rows.size() + 1, XC_ERR_INTERNAL, "bad exchange slab launch");
    const size_t nn = (size_t)n * n;
    const long long count = (long long)nn * nmat;
    jk_split_density_kernel<<<(unsigned)std::min<long long>((count + 255) / 256, 4096), 256, 0, s>>>(count, D, Dff);
    CGB_CUDA(cudaGetLastError());
    for (size_t k = 0; k < cls_rows.size(); k++) {
        const long long nc = cls_c0[k + 1] - cls_c0[k];
        if (nc <= 0) continue;
        CGB_CHECK(nc < (1LL << 31), XC_ERR_INTERNAL, "too many exchange chunks");
        const int rows = rawK ? cls_rows[k] : 0;
        // matrices per launch: as many as the slab holds (at least one)
        int mg = nmat;
        while (mg > 1 && jk_slab_bytes(rows, n, mg) > kJkSlabMaxBytes) mg--;
        const size_t bytes = jk_slab_bytes(rows, n, mg);
        CGB_CHECK(bytes <= kJkSlabMaxBytes, XC_ERR_INTERNAL, "exchange slab too large");
        const longlong2* c = chunks + cls_c0[k];
        for (int m0 = 0; m0 < nmat; m0 += mg) {
            const int nm = std::min(mg, nmat - m0);
            const float2* Dm = Dff + m0 * nn;
            double* Jm = rawJ ? rawJ + m0 * nn : nullptr;
            double* Km = rawK ? rawK + m0 * nn : nullptr;
            if (Jm && Km)
                jk_slab_kernel<true, true><<<(unsigned)nc, 32 * kJkWarps, bytes, s>>>(e, quartets, out_off, c, rows,
                                                                                      ints, n, nm, Dm, Jm, Km);
            else if (Km)
                jk_slab_kernel<false, true><<<(unsigned)nc, 32 * kJkWarps, bytes, s>>>(e, quartets, out_off, c, rows,
                                                                                       ints, n, nm, Dm, nullptr, Km);
            else
                jk_slab_kernel<true, false><<<(unsigned)nc, 32 * kJkWarps, bytes, s>>>(e, quartets, out_off, c, rows,
                                                                                       ints, n, nm, Dm, Jm, nullptr);
            CGB_CUDA(cudaGetLastError());
        }
    }
}

static unsigned persistent_blocks(long long items, int per_block) {
    int dev = 0, sms = 0;
    CGB_CUDA(cudaGetDevice(&dev));
    CGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const long long want = (items + per_block - 1) / per_block;
    return (unsigned)(want < (long long)sms * 8 ? (want > 0 ? want : 1) : (long long)sms * 8);
}

void launch_coulomb_scatter(const EriDev& e, const int2* quartets, const long long* out_off, long long nq,
                            const double* ints, long long ld, double* M, cudaStream_t s) {
    if (nq <= 0) return;
    coulomb_scatter_kernel<<<persistent_blocks(nq, 8), 256, 0, s>>>(e, quartets, out_off, nq, ints, ld, M);
    CGB_CUDA(cudaGetLastError());
}

void launch_coulomb_split(long long n, double* M, cudaStream_t s) {
    coulomb_split_kernel<<<persistent_blocks(n, 2048), 256, 0, s>>>(n, M);
    CGB_CUDA(cudaGetLastError());
}
void launch_coulomb_dense(int n, int nmat, long long ld, const double* M, const double* D, double* x, double* y,
                          double* J, cudaStream_t s) {
    CGB_CHECK(ld % 2 == 0 && ld >= (long long)n * (n + 1) / 2, XC_ERR_INTERNAL, "bad dense Coulomb row stride");
    const long long tot = (long long)n * n * nmat;
    // x: nmat float-float vectors of stride ld whose pad entry stays zero (the caller zeroes x once)
    float2* xf = reinterpret_cast<float2*>(x);
    const float2* Mf = reinterpret_cast<const float2*>(M);
    coulomb_pack_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(n, nmat, ld, D, xf);
    CGB_CUDA(cudaGetLastError());
    // one CTA per 8 rows (not persistent): CTAs retire every few microseconds,
    // so kernels of a higher-priority stream (an SCF's XC build beside J) get
    // SMs without waiting for the whole GEMV
    const unsigned blocks = (unsigned)((ld + 7) / 8);
    for (int m0 = 0; m0 < nmat; m0 += kGemvMaxVec) {
        const int nm = nmat - m0 < kGemvMaxVec ? nmat - m0 : kGemvMaxVec;
        const float2* xm = xf + m0 * ld;
        double* ym = y + m0 * ld;
        if (nm == 1) coulomb_gemv_kernel<1><<<blocks, 256, 0, s>>>(ld, Mf, xm, ym);
        else if (nm == 2) coulomb_gemv_kernel<2><<<blocks, 256, 0, s>>>(ld, Mf, xm, ym);
        else if (nm == 3) coulomb_gemv_kernel<3><<<blocks, 256, 0, s>>>(ld, Mf, xm, ym);
        else coulomb_gemv_kernel<4><<<blocks, 256, 0, s>>>(ld, Mf, xm, ym);
        CGB_CUDA(cudaGetLastError());
    }
    coulomb_unpack_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(n, nmat, ld, y, J);
    CGB_CUDA(cudaGetLastError());
}

void launch_jk_symmetrise(int n, int nmat, const double* rawJ, const double* rawK, double* J, double* K,
                          cudaStream_t s) {
    const long long tot = (long long)n * n * nmat;
    if (tot == 0) return;
    jk_symmetrise_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(n, nmat, rawJ, rawK, J, K);
    CGB_CUDA(cudaGetLastError());
}

}  // namespace cgb
