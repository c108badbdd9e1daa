// Electron-repulsion integrals and their J / K contraction on the GPU (the
// role of the reference's Int4C2E: CalculateIntegrals + ContractInts,
// src/Integral/Int4C2E.cpp:567-683).  Host-side description of the device
// data; the kernels are in k_eri.cu, the set-up and the C ABI in jk.cpp.
//
// Method: McMurchie-Davidson in FP64.  Per shell pair (a >= b) and
// primitive pair (i, j) the Hermite expansion of every product of pure
// functions is stored once ("Ep", the contraction coefficients and the
// Gaussian product factor folded in):
//   Ep[fa * nb + fb][h(t, u, v)] = c_i c_j sum_{Cartesian ka, kb}
//        T_a(fa, ka) T_b(fb, kb) E^x_{t} E^y_{u} E^z_{v},
// so that a primitive quartet is
//   (ab|cd) += 2 pi^(5/2) / (p q sqrt(p + q)) sum_h Ep_ab[ab][h]
//              sum_h' (-1)^|h'| Ep_cd[cd][h'] R_{h + h'}(alpha, P - Q).
// Hermite index h(t, u, v) orders (t, u, v) by N = t + u + v, so the
// entries with N <= L are the first H(L) = (L+1)(L+2)(L+3)/6.
#pragma once

#include <cstdint>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

namespace cgb {

constexpr int kEriMaxL = 3;                  // f shells
constexpr int kEriMaxLt = 4 * kEriMaxL;      // highest total angular momentum of a quartet
constexpr int kBoysCols = kEriMaxLt + 8;     // Boys table orders 0 .. kEriMaxLt + 7
constexpr double kBoysStep = 0.05;           // table spacing in T
constexpr double kBoysTmax = 80.0;           // asymptotic form beyond
constexpr int kBoysRows = 1601;              // kBoysTmax / kBoysStep + 1

__host__ __device__ constexpr int herm_count(int L) { return (L + 1) * (L + 2) * (L + 3) / 6; }

// One shell pair (shell a >= shell b) of the screened pair list.
struct EriPair {
    int fa, fb;       // first basis function of shell a, b
    int na, nb;       // pure functions per shell
    int la, lb;
    int npp, pp0;     // primitive pairs: count, first index in the primitive-pair arrays
    long long ep0;    // first Ep element of the pair (primitive pairs consecutive, na nb H(la+lb) each)
};

struct EriDev {
    const EriPair* pairs;
    const double* pp_p;   // exponent sum p per primitive pair
    const double* pp_P;   // Gaussian product centre (3 per primitive pair)
    const double* ep;     // Hermite coefficients of the pure function products
    const double* boys;   // kBoysRows x kBoysCols table of F_n(T_i)
};

// Integrals of quartets q0 .. q0 + nq - 1 of the list (bra pair x, ket pair
// y), each block [fa][fb][fc][fd] written to out + out_off[q] - base.
void launch_eri(const EriDev& e, const int2* quartets, const long long* out_off, long long q0, long long nq,
                long long base, double* out, cudaStream_t s);

// J / K of nmat density matrices (n x n, symmetric) from the integral blocks
// of quartets q0 .. q0 + nq - 1: raw accumulators (symmetrised by the caller:
// J = 2 (rawJ + rawJ^T), K = rawK + rawK^T), FP64 atomics.
void launch_jk_contract(const EriDev& e, const int2* quartets, const long long* out_off, long long q0, long long nq,
                        long long base, const double* ints, int n, int nmat, const double* D, double* rawJ,
                        double* rawK, cudaStream_t s);

// Coulomb and / or exchange (rawJ, rawK; either may be null) of the in-core
// list (base 0) from the float-float store (the FP64 blocks split in place
// by launch_coulomb_split, which nothing else reads afterwards) by bra-pair
// chunks: chunks[c] = [first, end) quartets of one bra pair, at most a few
// thousand; the chunks are grouped by the bra pair's na + nb, class k
// (na + nb = cls_rows[k]) holding chunks cls_c0[k] .. cls_c0[k + 1] - 1.
// D (FP64, nmat x n x n) is split into Dff (same size in float pairs) first.
// One CTA per chunk sums its exchange contributions in a shared-memory slab
// of jk_slab_bytes(rows, n, m) bytes for m matrices at a time, which must
// not exceed kJkSlabMaxBytes for m = 1.  Same raw accumulators as
// launch_jk_contract.
constexpr size_t kJkSlabMaxBytes = 200 * 1024;
size_t jk_slab_bytes(int rows, int n, int nmat);
void launch_jk_slab(const EriDev& e, const int2* quartets, const long long* out_off, const longlong2* chunks,
                    const std::vector<int>& cls_rows, const std::vector<long long>& cls_c0, const float2* ints, int n,
                    int nmat, const double* D, float2* Dff, double* rawJ, double* rawK, cudaStream_t s);

// Dense Coulomb operator M (ld x ld, ld = n (n + 1) / 2 rounded up to even,
// packed pairs mu >= nu) from the in-core blocks of all quartets; M must
// start at zero.  launch_coulomb_split then turns each FP64 element in place
// into a float-float pair (hi, lo), the form launch_coulomb_dense reads.
// J of nmat densities: pack (x2 off-diagonal) into x (nmat float-float
// vectors of stride ld in a buffer of nmat * ld doubles, zeroed once by the
// caller), GEMV into y (FP64), unpack.
void launch_coulomb_scatter(const EriDev& e, const int2* quartets, const long long* out_off, long long nq,
                            const double* ints, long long ld, double* M, cudaStream_t s);
void launch_coulomb_split(long long n, double* M, cudaStream_t s);
void launch_coulomb_dense(int n, int nmat, long long ld, const double* M, const double* D, double* x, double* y,
                          double* J, cudaStream_t s);

// rawJ, rawK -> J = 2 (rawJ + rawJ^T), K = rawK + rawK^T (nmat matrices each, either may be null).
void launch_jk_symmetrise(int n, int nmat, const double* rawJ, const double* rawK, double* J, double* K,
                          cudaStream_t s);

void set_eri_kernel_attributes();

struct BasisSet;
// Host side (integrals.cpp): Hermite data of shell pairs (first >= second),
// and the Boys table.
struct PairHermite {
    std::vector<double> p, P, ep;  // per kept primitive pair: p; centre (3); Ep block (na nb H)
};
void eri_pairs_hermite(const BasisSet& b, const std::vector<std::pair<int, int>>& pairs, double prim_cut,
                       std::vector<PairHermite>& out);
void boys_table(int rows, int cols, double step, double* out);

}  // namespace cgb
