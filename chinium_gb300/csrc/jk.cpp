// Coulomb and exchange matrices on the GPU for the SCF caller of the XC
// build: the reference's Int4C2E (src/Integral/Int4C2E.cpp) -- Schwarz
// bounds from the diagonal integrals (getRepulsionDiag, :19-77), the
// screened list of unique shell quartets (getRepulsionLength /
// getRepulsionIndices, :79-130), the integrals (CalculateIntegrals, :567-584)
// and their contraction with the density matrices every SCF iteration
// (ContractInts / Gunified, :601-683).
//
// Set-up (xc_jk_create): per shell pair a >= b the Hermite data of its kept
// primitive pairs (host, OpenMP) goes to HBM; the diagonal quartets (ab|ab)
// run on the GPU and give Q_ab = sqrt(max |(mu nu|mu nu)|); pairs are sorted
// by Q and the unique quartets (bra pair >= ket pair in that order) with
// Q_bra Q_ket >= threshold form the list.  When the integrals of the list
// fit in the memory budget they are computed once and kept in HBM
// ("in-core", as the reference keeps RepulsionInts in memory); otherwise
// each build recomputes them chunk by chunk ("direct").  A build contracts
// every quartet block with the density matrices into J and K: in-core stores
// of large quartets (>= 24 integrals on average) are split once into
// float-float pairs and contracted per bra pair on the FP32 pipe
// (jk_slab_kernel); the others per quartet in FP64 (jk_contract_kernel).
// Small molecules take J from a dense Coulomb operator instead.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "../../include/chinium_int.h"
#include "common.h"
#include "eri.h"
#include "model.h"
#include "xc_state.h"

namespace cgb {

struct JkEngine {
    int n = 0;
    double threshold = 0;
    cudaStream_t stream = nullptr;
    std::vector<EriPair> pairs;  // screened, sorted by Schwarz bound (descending)
    std::vector<double> Q;       // Schwarz bound per pair (same order)
    long long nquartets = 0, nints = 0;
    bool incore = false;
    long long chunk_ints = 0;                 // direct mode: integrals per chunk buffer
    std::vector<long long> chunk_q;           // direct mode: first quartet of every chunk (+ end)
    std::vector<long long> chunk_base;        // direct mode: block offset of each chunk's first quartet
    DevBuf<EriPair> d_pairs;
    DevBuf<double> d_pp_p, d_pp_P, d_ep, d_boys;
    DevBuf<int2> d_quartets;
    DevBuf<long long> d_off;
    bool dense_j = false;                     // J from the dense Coulomb operator over function pairs
    long long npair = 0;                      // row stride of the dense operator (pairs, rounded up to even)
    int dense_nmat = 0;
    DevBuf<double> d_M, d_x, d_y;             // dense operator and packed densities (float-float pairs
                                              // in 8-byte elements); results (FP64)
    DevBuf<double> d_ints;                    // in-core integrals, or the direct-mode chunk buffer
    DevBuf<double> d_D, d_rawJ, d_rawK, d_J, d_K;
    // in-core J / K by bra-pair chunks (launch_jk_slab) from the store split
    // into float-float pairs, when one matrix's slab of the largest bra
    // shells fits in shared memory: chunks grouped by the bra pair's na + nb,
    // largest first
    bool ff_store = false;
    DevBuf<longlong2> d_chunks;
    std::vector<int> cls_rows;
    std::vector<long long> cls_c0;
    DevBuf<float2> d_Dff;
    int nmat_alloc = 0;
    void make_chunks(const std::vector<int2>& quart);
    void dense_coulomb(int nmat, const double* dD, double* dJ);  // J from the dense operator into dJ
    EriDev dev() const { return EriDev{d_pairs.p, d_pp_p.p, d_pp_P.p, d_ep.p, d_boys.p}; }
    void setup(const BasisSet& b, double thr, double max_bytes);
    void build_device(int nmat, const double* dD, double* dJ, double* dK);
};

namespace {
constexpr double kPrimCut = 1e-20;
constexpr long long kSlabChunk = 2048;  // quartets per exchange chunk at most
// The slab kernel pays one shared-memory FP64 add (the warp waits for it)
// per sub-block element, the per-quartet kernel one global atomic add (not
// waited for) and FP64 products.  Measured: C18 def2-TZVP, 61 integrals per
// quartet, J + K 0.18 s (slab) vs 0.23 s; (H2O)8 def2-SVP, 13 per quartet,
// K 7.3 ms (slab) vs 4.7 ms.  The slab kernel is taken from this average up
// (between the measured points; the crossover itself was not measured).
constexpr double kSlabMinIntsPerQuartet = 24.0;

inline int nfunc_of(const Shell& s) { return shell_size(s.type); }
}  // namespace

void JkEngine::setup(const BasisSet& b, double thr, double max_bytes) {
    ensure_device();
    set_eri_kernel_attributes();
    n = b.nbasis;
    threshold = thr;
    for (const Shell& s : b.shells)
        CGB_CHECK(s.l <= kEriMaxL, XC_ERR_UNSUPPORTED, "the GPU integral engine supports s, p, d and f shells");
    const int ns = (int)b.shells.size();
    std::vector<std::pair<int, int>> sp;
    for (int a = 0; a < ns; a++)
        for (int c = 0; c <= a; c++) sp.emplace_back(a, c);
    std::vector<PairHermite> ph;
    eri_pairs_hermite(b, sp, kPrimCut, ph);
    // pairs with at least one primitive pair kept
    std::vector<EriPair> all;
    std::vector<double> pp_p, pp_P, ep;
    for (size_t i = 0; i < sp.size(); i++) {
        if (ph[i].p.empty()) continue;
        const Shell &A = b.shells[sp[i].first], &B = b.shells[sp[i].second];
        EriPair e{};
        e.fa = A.first;
        e.fb = B.first;
        e.na = nfunc_of(A);
        e.nb = nfunc_of(B);
        e.la = A.l;
        e.lb = B.l;
        e.npp = (int)ph[i].p.size();
        e.pp0 = (int)pp_p.size();
        e.ep0 = (long long)ep.size();
        pp_p.insert(pp_p.end(), ph[i].p.begin(), ph[i].p.end());
        pp_P.insert(pp_P.end(), ph[i].P.begin(), ph[i].P.end());
        ep.insert(ep.end(), ph[i].ep.begin(), ph[i].ep.end());
        all.push_back(e);
        std::vector<double>().swap(ph[i].ep);
    }
    CGB_CHECK(!all.empty(), XC_ERR_ARG, "basis without significant shell pairs");
    d_pp_p.upload(pp_p.data(), pp_p.size(), stream);
    d_pp_P.upload(pp_P.data(), pp_P.size(), stream);
    d_ep.upload(ep.data(), ep.size(), stream);
    {
        std::vector<double> tab((size_t)kBoysRows * kBoysCols);
        boys_table(kBoysRows, kBoysCols, kBoysStep, tab.data());
        d_boys.upload(tab.data(), tab.size(), stream);
    }
    d_pairs.upload(all.data(), all.size(), stream);
    // Schwarz bounds from the diagonal quartets (ab|ab)
    const int np = (int)all.size();
    {
        std::vector<int2> dq(np);
        std::vector<long long> doff(np);
        long long tot = 0;
        for (int i = 0; i < np; i++) {
            dq[i] = make_int2(i, i);
            doff[i] = tot;
            const long long nab = (long long)all[i].na * all[i].nb;
            tot += nab * nab;
        }
        DevBuf<int2> d_dq;
        DevBuf<long long> d_doff;
        DevBuf<double> d_diag;
        d_dq.upload(dq.data(), dq.size(), stream);
        d_doff.upload(doff.data(), doff.size(), stream);
        d_diag.alloc(tot);
        launch_eri(dev(), d_dq.p, d_doff.p, 0, np, 0, d_diag.p, stream);
        std::vector<double> diag(tot);
        CGB_CUDA(cudaMemcpyAsync(diag.data(), d_diag.p, tot * sizeof(double), cudaMemcpyDeviceToHost, stream));
        CGB_CUDA(cudaStreamSynchronize(stream));
        Q.assign(np, 0.0);
        for (int i = 0; i < np; i++) {
            const long long nab = (long long)all[i].na * all[i].nb;
            double m = 0;
            for (long long k = 0; k < nab; k++) m = std::max(m, std::fabs(diag[doff[i] + k * nab + k]));
            Q[i] = std::sqrt(m);
        }
    }
    // screen and sort the pairs by their bound
    const double qmax = *std::max_element(Q.begin(), Q.end());
    std::vector<int> order;
    for (int i = 0; i < np; i++)
        if (Q[i] * qmax >= thr && Q[i] > 0) order.push_back(i);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return Q[x] > Q[y]; });
    pairs.clear();
    std::vector<double> Qs;
    for (int i : order) {
        pairs.push_back(all[i]);
        Qs.push_back(Q[i]);
    }
    Q.swap(Qs);
    d_pairs.upload(pairs.data(), pairs.size(), stream);
    // unique quartets (bra >= ket in the sorted order), offsets of their blocks
    std::vector<int2> quart;
    std::vector<long long> off;
    long long tot = 0;
    const int npk = (int)pairs.size();
    for (int i = 0; i < npk; i++) {
        const long long nab = (long long)pairs[i].na * pairs[i].nb;
        for (int j = 0; j <= i; j++) {
            if (Q[i] * Q[j] < thr) break;  // Q sorted descending: no later ket passes
            quart.push_back(make_int2(i, j));
            off.push_back(tot);
            tot += nab * pairs[j].na * pairs[j].nb;
        }
    }
    nquartets = (long long)quart.size();
    nints = tot;
    CGB_CHECK(nquartets > 0, XC_ERR_ARG, "no shell quartet above the threshold");
    d_quartets.upload(quart.data(), quart.size(), stream);
    d_off.upload(off.data(), off.size(), stream);
    // in-core when the integrals fit in the budget (default: half of the free memory)
    size_t freeb = 0, totalb = 0;
    CGB_CUDA(cudaMemGetInfo(&freeb, &totalb));
    const double budget = max_bytes > 0 ? max_bytes : 0.5 * (double)freeb;
    incore = (double)nints * sizeof(double) <= budget;
    chunk_q.clear();
    if (incore) {
        d_ints.alloc(nints);
        launch_eri(dev(), d_quartets.p, d_off.p, 0, nquartets, 0, d_ints.p, stream);
        // small molecules: the dense Coulomb operator when it takes at most a
        // quarter of the memory left (J then streams it once per build)
        npair = (long long)n * (n + 1) / 2;
        npair += npair & 1;  // even row stride (16-byte rows for the GEMV)
        CGB_CUDA(cudaStreamSynchronize(stream));
        CGB_CUDA(cudaMemGetInfo(&freeb, &totalb));
        // (and the operator plus the integrals within the caller's budget)
        const double mbytes = (double)npair * npair * sizeof(double);
        dense_j = mbytes <= 0.25 * (double)freeb && (double)nints * sizeof(double) + mbytes <= budget;
        if (dense_j) {
            d_M.alloc((size_t)npair * npair);
            d_M.zero(stream);
            launch_coulomb_scatter(dev(), d_quartets.p, d_off.p, nquartets, d_ints.p, npair, d_M.p, stream);
            launch_coulomb_split((long long)npair * npair, d_M.p, stream);
        }
        make_chunks(quart);
        ff_store = jk_slab_bytes(cls_rows[0], n, 1) <= kJkSlabMaxBytes &&
                   (double)nints >= kSlabMinIntsPerQuartet * (double)nquartets;
        if (ff_store) launch_coulomb_split(nints, d_ints.p, stream);  // after the scatter read the FP64 blocks
        CGB_CUDA(cudaStreamSynchronize(stream));
    } else {
        // chunks of consecutive quartets whose blocks fit in the chunk buffer
        const long long cap = std::max<long long>((long long)(std::min(budget, 2e9) / sizeof(double)), 2401);
        chunk_q.push_back(0);
        long long start = off[0];
        for (long long q = 0; q < nquartets; q++) {
            const long long end = (q + 1 < nquartets ? off[q + 1] : nints);
            if (end - start > cap) {
                chunk_q.push_back(q);
                start = off[q];
            }
        }
        chunk_q.push_back(nquartets);
        chunk_base.clear();
        for (size_t c = 0; c + 1 < chunk_q.size(); c++) chunk_base.push_back(off[chunk_q[c]]);
        chunk_ints = cap;
        d_ints.alloc(cap);
    }
}

void JkEngine::make_chunks(const std::vector<int2>& quart) {
    // the quartets of a bra pair are consecutive (bra-major list); runs of at
    // most kSlabChunk of them, grouped by the bra pair's na + nb
    std::vector<std::vector<longlong2>> by_rows(2 * (2 * kEriMaxL + 1) + 1);
    const long long nq = (long long)quart.size();
    for (long long q = 0; q < nq;) {
        const int i = quart[q].x;
        long long e = q;
        while (e < nq && quart[e].x == i) e++;
        const int rows = pairs[i].na + pairs[i].nb;
        for (long long c = q; c < e; c += kSlabChunk)
            by_rows[rows].push_back(make_longlong2(c, std::min(e, c + kSlabChunk)));
        q = e;
    }
    std::vector<longlong2> all;
    cls_rows.clear();
    cls_c0.clear();
    for (int rows = (int)by_rows.size() - 1; rows >= 0; rows--) {
        if (by_rows[rows].empty()) continue;
        cls_rows.push_back(rows);
        cls_c0.push_back((long long)all.size());
        all.insert(all.end(), by_rows[rows].begin(), by_rows[rows].end());
    }
    cls_c0.push_back((long long)all.size());
    d_chunks.upload(all.data(), all.size(), stream);
    CGB_CUDA(cudaStreamSynchronize(stream));
}

void JkEngine::dense_coulomb(int nmat, const double* dD, double* dJ) {
    if (nmat > dense_nmat) {
        d_x.alloc((size_t)npair * nmat);
        d_x.zero(stream);  // pad entries stay zero
        d_y.alloc((size_t)npair * nmat);
        dense_nmat = nmat;
    }
    launch_coulomb_dense(n, nmat, npair, d_M.p, dD, d_x.p, d_y.p, dJ, stream);
}

void JkEngine::build_device(int nmat, const double* dD, double* dJ, double* dK) {
    const size_t nn = (size_t)n * n;
    if (nmat > nmat_alloc) {
        d_rawJ.alloc(nn * nmat);
        d_rawK.alloc(nn * nmat);
        nmat_alloc = nmat;
    }
    // J from the dense operator (straight into dJ) where there is one, else
    // from the blocks into the raw accumulator with K
    const bool j_dense = incore && dense_j && dJ;
    double* rJ = dJ && !j_dense ? d_rawJ.p : nullptr;
    double* rK = dK ? d_rawK.p : nullptr;
    if (rJ) CGB_CUDA(cudaMemsetAsync(rJ, 0, nn * nmat * sizeof(double), stream));
    if (rK) CGB_CUDA(cudaMemsetAsync(rK, 0, nn * nmat * sizeof(double), stream));
    if (j_dense) dense_coulomb(nmat, dD, dJ);
    if (incore && ff_store) {
        if (rJ || rK) {
            if (d_Dff.n < nn * nmat) d_Dff.alloc(nn * nmat);
            launch_jk_slab(dev(), d_quartets.p, d_off.p, d_chunks.p, cls_rows, cls_c0,
                           reinterpret_cast<const float2*>(d_ints.p), n, nmat, dD, d_Dff.p, rJ, rK, stream);
        }
    } else if (incore) {
        launch_jk_contract(dev(), d_quartets.p, d_off.p, 0, nquartets, 0, d_ints.p, n, nmat, dD, rJ, rK, stream);
    } else {
        for (size_t c = 0; c + 1 < chunk_q.size(); c++) {
            const long long q0 = chunk_q[c], q1 = chunk_q[c + 1];
            if (q1 <= q0) continue;
            const long long base = chunk_base[c];
            launch_eri(dev(), d_quartets.p, d_off.p, q0, q1 - q0, base, d_ints.p, stream);
            launch_jk_contract(dev(), d_quartets.p, d_off.p, q0, q1 - q0, base, d_ints.p, n, nmat, dD, rJ, rK,
                               stream);
        }
    }
    launch_jk_symmetrise(n, nmat, rJ, rK, rJ ? dJ : nullptr, dK, stream);
}

}  // namespace cgb

using namespace cgb;

struct xc_jk {
    JkEngine e;
};

extern "C" int xc_jk_create(const xc_basis* b, double threshold, double max_bytes, xc_jk** out) {
    return guard([&] {
        CGB_CHECK(b && out, XC_ERR_ARG, "null argument");
        CGB_CHECK(threshold >= 0 && std::isfinite(threshold), XC_ERR_ARG, "threshold must be >= 0");
        auto* h = new xc_jk;
        try {
            h->e.setup(b->b, threshold, max_bytes);
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
    });
}

extern "C" int xc_jk_destroy(xc_jk* h) {
    delete h;
    return XC_OK;
}

extern "C" int xc_jk_info(const xc_jk* h, long long* nquartets, long long* nints, int* incore) {
    return guard([&] {
        CGB_CHECK(h, XC_ERR_ARG, "null handle");
        if (nquartets) *nquartets = h->e.nquartets;
        if (nints) *nints = h->e.nints;
        if (incore) *incore = h->e.incore ? 1 : 0;
    });
}

extern "C" int xc_jk_set_stream(xc_jk* h, void* stream) {
    return guard([&] {
        CGB_CHECK(h, XC_ERR_ARG, "null handle");
        h->e.stream = (cudaStream_t)stream;
    });
}

extern "C" int xc_jk_build_device(xc_jk* h, int nmat, const double* dD, double* dJ, double* dK) {
    return guard([&] {
        CGB_CHECK(h && dD && nmat > 0 && (dJ || dK), XC_ERR_ARG, "bad J/K arguments");
        h->e.build_device(nmat, dD, dJ, dK);
    });
}

extern "C" int xc_jk_build(xc_jk* h, int nmat, const double* D, double* J, double* K) {
    return guard([&] {
        CGB_CHECK(h && D && nmat > 0 && (J || K), XC_ERR_ARG, "bad J/K arguments");
        JkEngine& e = h->e;
        const size_t nn = (size_t)e.n * e.n * nmat;
        e.d_D.alloc(nn);
        CGB_CUDA(cudaMemcpyAsync(e.d_D.p, D, nn * sizeof(double), cudaMemcpyHostToDevice, e.stream));
        if (J) e.d_J.alloc(nn);
        if (K) e.d_K.alloc(nn);
        e.build_device(nmat, e.d_D.p, J ? e.d_J.p : nullptr, K ? e.d_K.p : nullptr);
        if (J) CGB_CUDA(cudaMemcpyAsync(J, e.d_J.p, nn * sizeof(double), cudaMemcpyDeviceToHost, e.stream));
        if (K) CGB_CUDA(cudaMemcpyAsync(K, e.d_K.p, nn * sizeof(double), cudaMemcpyDeviceToHost, e.stream));
        CGB_CUDA(cudaStreamSynchronize(e.stream));
    });
}
