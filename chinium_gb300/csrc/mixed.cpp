// Host orchestration of the mixed-precision build: molecule sources, point
// tiles (k-d cells of each molecule), chunk screening, the FP32 AO store,
// cost-balanced persistent work lists, the TMA map of the density strip, and
// the per-build launch sequence (D split -> tensor-core density ->
// functional -> per-molecule E_xc -> Z operand -> tensor-core V partials ->
// FP64 reduction), optionally replayed from a CUDA graph.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <numeric>
#include <queue>

#include "mixed.h"
#include "nvtx.h"
#include "xc_state.h"

namespace cgb {

namespace {
using PFN_encode = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

PFN_encode encoder() {
    static PFN_encode fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        CGB_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
        CGB_CHECK(p && q == cudaDriverEntryPointSuccess, XC_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
        fn = (PFN_encode)p;
    }
    return fn;
}

// Orders idx[lo, hi) so that consecutive runs of 128 points are k-d cells:
// each split cuts the longest extent at a tile-aligned rank, so every left
// part holds a multiple of 128 points and only the last run is partial.
void kd_order(const double* x, const double* y, const double* z, int* idx, long lo, long hi) {
    if (hi - lo <= kTilePts) return;
    double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
    for (long k = lo; k < hi; k++) {
        const double p[3] = {x[idx[k]], y[idx[k]], z[idx[k]]};
        for (int a = 0; a < 3; a++) {
            mn[a] = std::min(mn[a], p[a]);
            mx[a] = std::max(mx[a], p[a]);
        }
    }
    int axis = 0;
    for (int a = 1; a < 3; a++)
        if (mx[a] - mn[a] > mx[axis] - mn[axis]) axis = a;
    const double* c = axis == 0 ? x : (axis == 1 ? y : z);
    const long n = hi - lo;
    long left = ((n + 1) / 2 + kTilePts - 1) / kTilePts * kTilePts;
    if (left >= n) left = (n - 1) / kTilePts * kTilePts;
    const long mid = lo + left;
    std::nth_element(idx + lo, idx + mid, idx + hi, [&](int a, int b) { return c[a] < c[b] || (c[a] == c[b] && a < b); });
    kd_order(x, y, z, idx, lo, mid);
    kd_order(x, y, z, idx, mid, hi);
}

// Longest-processing-time binning: items by decreasing cost, each to the
// least-loaded bin (ties: lower bin).  CSR output, deterministic.
void lpt(const std::vector<long>& cost, const std::vector<int>& ids, int nbins, std::vector<int>& off,
         std::vector<int>& list) {
    std::vector<int> order(ids.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[ids[a]] > cost[ids[b]]; });
    using Load = std::pair<long, int>;
    std::priority_queue<Load, std::vector<Load>, std::greater<Load>> pq;
    for (int b = 0; b < nbins; b++) pq.push({0, b});
    std::vector<std::vector<int>> bins(nbins);
    for (int i : order) {
        const Load l = pq.top();
        pq.pop();
        bins[l.second].push_back(ids[i]);
        pq.push({l.first + cost[ids[i]], l.second});
    }
    off.assign(1, 0);
    list.clear();
    for (auto& b : bins) {
        list.insert(list.end(), b.begin(), b.end());
        off.push_back((int)list.size());
    }
}

int sm_count() {
    int dev = 0, nsm = 148;
    CGB_CUDA(cudaGetDevice(&dev));
    CGB_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    return nsm;
}
}  // namespace

void make_tmap_bf16(CUtensorMap* map, const void* base, uint64_t cols, uint64_t rows, uint32_t box_cols,
                    uint32_t box_rows) {
    CGB_CHECK(((uintptr_t)base & 15) == 0 && (cols * 2) % 16 == 0, XC_ERR_INTERNAL, "TMA base/stride alignment");
    const cuuint64_t dims[2] = {cols, rows};
    const cuuint64_t strides[1] = {cols * 2};
    const cuuint32_t box[2] = {box_cols, box_rows};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = encoder()(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    CGB_CHECK(r == CUDA_SUCCESS, XC_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
}

void make_tmap_f32(CUtensorMap* map, const void* base, uint64_t cols, uint64_t rows, uint32_t box_cols,
                   uint32_t box_rows) {
    CGB_CHECK(((uintptr_t)base & 15) == 0 && (cols * 4) % 16 == 0, XC_ERR_INTERNAL, "TMA base/stride alignment");
    CGB_CHECK(rows < (1ull << 31), XC_ERR_UNSUPPORTED, "FP32 AO store too tall for a TMA coordinate");
    const cuuint64_t dims[2] = {cols, rows};
    const cuuint64_t strides[1] = {cols * 4};
    const cuuint32_t box[2] = {box_cols, box_rows};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = encoder()(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    CGB_CHECK(r == CUDA_SUCCESS, XC_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
}

MixedState::~MixedState() { drop_graph(); }

void MixedState::drop_graph() {
    if (graph) cudaGraphExecDestroy(graph);
    graph = nullptr;
    graph_ids.clear();
    graph_type = -1;
}

long Grid::packed_size() const {
    if (mol_n.empty()) return (long)nspin * basis.nbasis * basis.nbasis;
    long s = 0;
    for (int n : mol_n) s += (long)nspin * n * n;
    return s;
}

// The one molecule of an ordinary grid: the real points of its blocks.
void Grid::collect_sources() {
    if (batched || !sources.empty()) return;
    std::vector<double> w(Gp);
    if (Gp) CGB_CUDA(cudaMemcpyAsync(w.data(), d_w.p, Gp * sizeof(double), cudaMemcpyDeviceToHost, stream));
    CGB_CUDA(cudaStreamSynchronize(stream));
    MolSource m;
    m.n = basis.nbasis;
    m.f0 = 0;
    m.sh0 = 0;
    m.sh1 = (int)basis.shells.size();
    for (const BlockDesc& bd : blocks)
        for (int k = 0; k < bd.nreal; k++) {
            const long i = bd.pt_off + k;
            m.x.push_back(hx[i]);
            m.y.push_back(hy[i]);
            m.z.push_back(hz[i]);
            m.w.push_back(w[i]);
            m.src.push_back(i);
        }
    sources.assign(1, std::move(m));
    mol_n.assign(1, basis.nbasis);
}

void Grid::prepare_mixed(const MixedConfig& cfg) {
    NvtxRange nvtx_("xc.mixed.prepare");
    MixedState& m = mx;
    m.drop_graph();
    m.ready = false;
    m.have_ref = false;
    m.cfg = cfg;
    m.nspin = nspin;
    collect_sources();
    const int nmol = (int)sources.size();
    CGB_CHECK(nmol > 0, XC_ERR_STATE, "no molecules");
    const int nsm = sm_count();

    // ---- tiles: k-d cells of each molecule's real points, padded to 128
    std::vector<double> tx, ty, tz, tw;
    std::vector<long> perm;
    std::vector<int> tile_real;
    m.have_perm = true;
    m.mols.assign(nmol, MolRange{});
    long voff = 0, drows = 0;
    int maxchunk = 1, dcols = 64;
    m.real_points = 0;
    for (int i = 0; i < nmol; i++) {
        const MolSource& S = sources[i];
        MolRange& R = m.mols[i];
        R.n = S.n;
        R.f0 = S.f0;
        R.sh0 = S.sh0;
        R.sh1 = S.sh1;
        R.nchunk = (S.n + kChunk - 1) / kChunk;
        R.nblk = (R.nchunk + 1) / 2;
        R.voff = voff;
        voff += (long)nspin * S.n * S.n;
        maxchunk = std::max(maxchunk, R.nchunk);
        drows = std::max(drows, (long)S.f0 + (long)R.nchunk * kChunk);
        dcols = std::max(dcols, R.nchunk * kChunk);
        const long np = (long)S.x.size();
        m.real_points += np;
        if (S.src.size() != S.x.size()) m.have_perm = false;
        std::vector<int> idx(np);
        std::iota(idx.begin(), idx.end(), 0);
        if (cfg.spatial) kd_order(S.x.data(), S.y.data(), S.z.data(), idx.data(), 0, np);
        R.t0 = (int)(tx.size() / kTilePts);
        for (long k0 = 0; k0 < np; k0 += kTilePts) {
            const long k1 = std::min(np, k0 + kTilePts);
            tile_real.push_back((int)(k1 - k0));
            for (long k = k0; k < k0 + kTilePts; k++) {
                const bool pad = k >= k1;
                const int j = idx[pad ? k0 : k];  // padding: copies of the tile's first point, weight 0
                tx.push_back(S.x[j]);
                ty.push_back(S.y[j]);
                tz.push_back(S.z[j]);
                tw.push_back(pad ? 0.0 : S.w[j]);
                const long src = m.have_perm ? S.src[j] : 0;
                perm.push_back(pad ? -src - 1 : src);
            }
        }
        R.t1 = (int)(tx.size() / kTilePts);
    }
    const int ntiles = (int)(tx.size() / kTilePts);
    MixedDev& md = m.md;
    md = MixedDev{};
    md.ntiles = ntiles;
    md.nchunk = maxchunk;
    md.Gt = (long)ntiles * kTilePts;
    md.drows = drows;
    m.dcols = dcols;

    // ---- chunk screening per tile (bounding sphere of its real points)
    const int nsh = (int)basis.shells.size();
    std::vector<double> ext(nsh);
    for (int s = 0; s < nsh; s++) ext[s] = shell_extent(basis, basis.shells[s], cfg.screen);
    m.h_nkept.assign(ntiles, 0);
    m.h_chunks.assign((size_t)ntiles * md.nchunk, 0);
    m.h_slot.assign((size_t)ntiles * md.nchunk, -1);
    m.h_row.assign(ntiles, 0);
    std::vector<int> c0s(ntiles, 0), tile_shells, tile_off(1, 0);
    long rows = 0;
    m.kept_pairs = 0;
    for (int i = 0; i < nmol; i++) {
        const MolRange& R = m.mols[i];
        for (int t = R.t0; t < R.t1; t++) {
            const long lo = (long)t * kTilePts, nr = tile_real[t];
            double cx = 0, cy = 0, cz = 0;
            for (long k = lo; k < lo + nr; k++) {
                cx += tx[k];
                cy += ty[k];
                cz += tz[k];
            }
            cx /= (double)nr;
            cy /= (double)nr;
            cz /= (double)nr;
            double rad = 0;
            for (long k = lo; k < lo + nr; k++)
                rad = std::max(rad, std::sqrt((tx[k] - cx) * (tx[k] - cx) + (ty[k] - cy) * (ty[k] - cy) +
                                              (tz[k] - cz) * (tz[k] - cz)));
            std::vector<char> keep(R.nchunk, 0);
            for (int s = R.sh0; s < R.sh1; s++) {
                const Shell& sh = basis.shells[s];
                const double d =
                    std::sqrt((sh.x - cx) * (sh.x - cx) + (sh.y - cy) * (sh.y - cy) + (sh.z - cz) * (sh.z - cz));
                if (cfg.screen > 0 && d - rad > ext[s]) continue;
                const int f0 = sh.first - R.f0, f1 = f0 + shell_size(sh.type) - 1;
                for (int c = f0 / kChunk; c <= f1 / kChunk; c++) keep[c] = 1;
            }
            int nk = 0;
            for (int c = 0; c < R.nchunk; c++)
                if (keep[c]) {
                    m.h_chunks[(size_t)t * md.nchunk + nk] = c;
                    m.h_slot[(size_t)t * md.nchunk + c] = nk;
                    nk++;
                }
            m.h_nkept[t] = nk;
            m.h_row[t] = rows;
            rows += (long)nk * kChunk;
            c0s[t] = R.f0 / kChunk;
            m.kept_pairs += (long)(nk * kChunk) * (nk * kChunk);
            for (int s = R.sh0; s < R.sh1; s++) {
                const Shell& sh = basis.shells[s];
                const int f0 = sh.first - R.f0, f1 = f0 + shell_size(sh.type) - 1;
                bool any = false;
                for (int c = f0 / kChunk; c <= f1 / kChunk; c++) any |= keep[c] != 0;
                if (any) tile_shells.push_back(s);
            }
            tile_off.push_back((int)tile_shells.size());
        }
    }
    md.rows = std::max(rows, 1L);

    // pre-split operands (BF16 planes of the AO store and of the per-build R
    // operands) when they fit in half of the memory left after the FP32 store
    m.ao_comp = type >= 1 ? 4 : 1;
    {
        const int ncv = type >= 2 ? 4 : 1;
        const size_t n16 = (size_t)md.rows * kTilePts;
        const int ncd = type >= 2 ? 4 : 1;  // components the density kernel takes as its A operand
        const size_t need = (size_t)(3 * m.ao_comp + 3 * ncv + 3 * ncd) * n16 * sizeof(__nv_bfloat16);
        const size_t e32b = (size_t)m.ao_comp * n16 * sizeof(float);
        size_t freeb = 0, totalb = 0;
        CGB_CUDA(cudaMemGetInfo(&freeb, &totalb));
        const size_t room = freeb > e32b ? (freeb - e32b) / 2 : 0;
        const bool coord_ok = (long)(3 * std::max(m.ao_comp, ncv)) * md.rows < (1L << 31);
        m.use16 = coord_ok && (cfg.v_operands == 2 || (cfg.v_operands == 0 && need < room));
        CGB_CHECK(cfg.v_operands != 2 || m.use16, XC_ERR_UNSUPPORTED,
                  "pre-split V operands do not fit (TMA row coordinate)");
    }

    // ---- persistent work lists
    std::vector<long> dcost(ntiles);
    std::vector<int> dids;
    m.units_full = m.units_sym = 0;
    for (int t = 0; t < ntiles; t++) {
        const int nk = m.h_nkept[t], nvb = (nk + 1) / 2;
        dcost[t] = (long)nvb * nk;
        m.units_full += (long)nvb * nk;
        m.units_sym += (long)nvb * nk - (long)nvb * (nvb - 1);
        if (nk > 0) dids.push_back(t);
    }
    m.empty_tiles = ntiles - (long)dids.size();
    std::vector<int> doff, dlist;
    m.dens_ctas = std::min((int)dids.size(), nsm);
    lpt(dcost, dids, m.dens_ctas, doff, dlist);
    CGB_CHECK(4 * rows < (1L << 31), XC_ERR_UNSUPPORTED, "FP32 AO store rows exceed the 32-bit TMA row coordinate");
    std::vector<DensJob> djobs;
    for (int t : dlist) djobs.push_back(DensJob{t, m.h_nkept[t], (int)m.h_row[t], c0s[t]});

    long L = cfg.fock_tiles;
    if (L <= 0) {
        long work = 0;
        for (auto& R : m.mols) work += (long)(R.t1 - R.t0) * R.nblk * R.nblk;
        L = std::max(1L, (work + 6L * nsm - 1) / (6L * nsm));
    }
    std::vector<FockItem> items;
    std::vector<int> live, fids;
    std::vector<long> fcost;
    auto slot = [&](int t, int c) { return c < md.nchunk ? m.h_slot[(size_t)t * md.nchunk + c] : -1; };
    for (auto& R : m.mols) {
        const long nt = R.t1 - R.t0;
        R.nsplit = (int)std::max(1L, (nt + L - 1) / L);
        R.item0 = (long)items.size();
        for (int I = 0; I < R.nblk; I++)
            for (int J = 0; J < R.nblk; J++)
                for (int s = 0; s < R.nsplit; s++) {
                    FockItem it;
                    it.I = I;
                    it.J = J;
                    it.t0 = (int)(R.t0 + nt * s / R.nsplit);
                    it.t1 = (int)(R.t0 + nt * (s + 1) / R.nsplit);
                    long wanted = 0;
                    for (int t = it.t0; t < it.t1; t++)
                        wanted += (slot(t, 2 * I) >= 0 || slot(t, 2 * I + 1) >= 0) &&
                                  (slot(t, 2 * J) >= 0 || slot(t, 2 * J + 1) >= 0);
                    if (wanted) fids.push_back((int)items.size());
                    live.push_back(wanted > 0);
                    fcost.push_back(wanted * (type >= 2 && I <= J ? 4 : 1));
                    items.push_back(it);
                }
    }
    m.nitems = (long)items.size();
    m.live_items = (long)fids.size();
    std::vector<int> foff, flist;
    m.fock_ctas = std::min((int)fids.size(), nsm);
    {
        // L2 locality of the pre-split kernel (which streams 96 KB of planes
        // per stage): items fall into S segments by the position of their
        // tile range in the molecule (S keeps >= 2 items per CTA in each);
        // every CTA takes its segment-0 items first, then segment 1, ..., so
        // concurrently running items read the same stretch of the operand
        // stores.  Each segment is cost-balanced on its own (LPT).  The
        // in-kernel-split kernel keeps one LPT over all items (faster there).
        const int S = !m.use16 ? 1 : std::max(1, std::min(64, (int)(fids.size() / (2 * (size_t)std::max(m.fock_ctas, 1)))));
        std::vector<std::vector<int>> seg(S);
        std::vector<int> item_mol(items.size(), 0);
        for (int i = 0; i < nmol; i++)
            for (long k = m.mols[i].item0; k < (i + 1 < nmol ? m.mols[i + 1].item0 : (long)items.size()); k++)
                item_mol[k] = i;
        for (int id : fids) {
            const MolRange& R = m.mols[item_mol[id]];
            const long span = std::max(1, R.t1 - R.t0);
            seg[std::min(S - 1, (int)((long)(items[id].t0 - R.t0) * S / span))].push_back(id);
        }
        std::vector<std::vector<int>> per_cta(m.fock_ctas);
        for (int k = 0; k < S; k++) {
            if (seg[k].empty()) continue;
            std::vector<int> so, sl;
            lpt(fcost, seg[k], m.fock_ctas, so, sl);
            for (int b = 0; b < m.fock_ctas; b++) per_cta[b].insert(per_cta[b].end(), sl.begin() + so[b], sl.begin() + so[b + 1]);
        }
        foff.assign(1, 0);
        for (auto& v : per_cta) {
            flist.insert(flist.end(), v.begin(), v.end());
            foff.push_back((int)flist.size());
        }
    }
    // per CTA: the wanted tiles of its items, in order, with their slots
    std::vector<FockJob> fjobs;
    std::vector<int> fjoff(1, 0);
    for (int b = 0; b < m.fock_ctas; b++) {
        for (int k = foff[b]; k < foff[b + 1]; k++) {
            const int id = flist[k];
            const FockItem& it = items[id];
            const size_t first = fjobs.size();
            for (int t = it.t0; t < it.t1; t++) {
                const int sa0 = slot(t, 2 * it.I), sa1 = slot(t, 2 * it.I + 1);
                const int sb0 = slot(t, 2 * it.J), sb1 = slot(t, 2 * it.J + 1);
                if ((sa0 < 0 && sa1 < 0) || (sb0 < 0 && sb1 < 0)) continue;
                const int tau = (it.I <= it.J ? 4 : 0) | (it.I < it.J ? 8 : 0);
                fjobs.push_back(FockJob{t, (int)m.h_row[t], sa0, sa1, sb0, sb1, id, tau});
            }
            fjobs[first].flags |= 1;
            fjobs.back().flags |= 2;
        }
        fjoff.push_back((int)fjobs.size());
    }

    // ---- device structures
    cudaStream_t s = stream;
    m.d_nkept.upload(m.h_nkept.data(), ntiles, s);
    m.d_chunks.upload(m.h_chunks.data(), m.h_chunks.size(), s);
    m.d_slot.upload(m.h_slot.data(), m.h_slot.size(), s);
    m.d_row.upload(m.h_row.data(), ntiles, s);
    m.d_c0.upload(c0s.data(), ntiles, s);
    m.d_tile_shells.upload(tile_shells.data(), std::max<size_t>(tile_shells.size(), 1), s);
    m.d_tile_shell_off.upload(tile_off.data(), tile_off.size(), s);
    m.d_x.upload(tx.data(), tx.size(), s);
    m.d_y.upload(ty.data(), ty.size(), s);
    m.d_z.upload(tz.data(), tz.size(), s);
    m.d_w.upload(tw.data(), tw.size(), s);
    if (m.have_perm) m.d_perm.upload(perm.data(), perm.size(), s);
    m.d_mols.upload(m.mols.data(), m.mols.size(), s);
    m.d_item_live.upload(live.data(), std::max<size_t>(live.size(), 1), s);
    m.d_dens_off.upload(doff.data(), doff.size(), s);
    if (djobs.empty()) djobs.push_back(DensJob{0, 1, 0, 0});
    m.d_dens_jobs.upload(djobs.data(), djobs.size(), s);
    m.d_fock_off.upload(fjoff.data(), fjoff.size(), s);
    m.fock_jobs = (long)fjobs.size();
    m.fock_tau_jobs = 0;
    for (const FockJob& j : fjobs) m.fock_tau_jobs += (j.flags & 4) != 0;
    if (fjobs.empty()) fjobs.push_back(FockJob{0, 0, -1, -1, -1, -1, 0, 0});
    m.d_fock_jobs.upload(fjobs.data(), fjobs.size(), s);
    {
        static double table[kMaxL + 1][2 * kMaxL + 1][(kMaxL + 1) * (kMaxL + 2) / 2];
        solid_harmonic_table(table);
        m.d_shtab.upload(&table[0][0][0], sizeof(table) / sizeof(double), s);
    }
    md.tile_nkept = m.d_nkept.p;
    md.tile_chunks = m.d_chunks.p;
    md.tile_slot = m.d_slot.p;
    md.tile_row = m.d_row.p;
    md.tile_c0 = m.d_c0.p;
    m.d_e32.alloc((size_t)m.ao_comp * md.rows * kTilePts);
    m.d_e32.zero(s);
    md.e32 = m.d_e32.p;
    launch_ao_mixed(md, dev_shells(), m.d_tile_shells.p, m.d_tile_shell_off.p, m.d_x.p, m.d_y.p, m.d_z.p, m.d_shtab.p,
                    m.ao_comp, m.d_e32.p, s);
    // pre-split operands: AO planes (3 per component) and R planes (3 for Z,
    // 9 more for the meta-GGA components)
    {
        const int ncv = type >= 2 ? 4 : 1;
        const size_t n16 = (size_t)md.rows * kTilePts;
        if (m.use16) {
            const int ncd = type >= 2 ? 4 : 1;
            m.d_e16.alloc((size_t)3 * m.ao_comp * n16);
            m.d_e16d.alloc((size_t)3 * ncd * n16);
            m.d_R16.alloc((size_t)3 * ncv * n16);
            launch_split_store(m.d_e32.p, (long)n16, m.ao_comp, m.d_e16.p, s);
            launch_split_store_fixed(m.d_e32.p, md.rows, ncd, m.d_e16d.p, s);
            make_tmap_bf16(&m.tm_e16, m.d_e16.p, kTilePts, (uint64_t)3 * m.ao_comp * md.rows, 64, 64);
            make_tmap_bf16(&m.tm_e16d, m.d_e16d.p, kTilePts, (uint64_t)3 * ncd * md.rows, 64, 64);
            make_tmap_bf16(&m.tm_r16, m.d_R16.p, kTilePts, (uint64_t)3 * ncv * md.rows, 64, 64);
            m.d_Z.alloc(1);
            m.d_c2.alloc(1);
        } else {
            m.d_e16.alloc(1);
            m.d_e16d.alloc(1);
            m.d_R16.alloc(1);
            m.d_Z.alloc((size_t)md.rows * kTilePts);
            m.d_c2.alloc(type >= 2 ? (size_t)md.Gt : 1);
        }
    }
    m.d_Dp.alloc((size_t)nspin * 3 * drows * dcols);
    m.d_wpart.alloc((size_t)std::max(m.nitems, 1L) * 16384);
    m.d_err.alloc(1);
    m.d_err.zero(s);
    make_tmap_bf16(&m.tm_d, m.d_Dp.p, dcols, (uint64_t)nspin * 3 * drows, 64, 64);
    make_tmap_f32(&m.tm_raw_d, m.d_e32.p, kTilePts, (uint64_t)m.ao_comp * md.rows, 128, 64);
    make_tmap_f32(&m.tm_raw_f, m.d_e32.p, kTilePts, (uint64_t)m.ao_comp * md.rows, 32, 64);
    if (!m.use16) make_tmap_f32(&m.tm_z, m.d_Z.p, kTilePts, (uint64_t)md.rows, 32, 64);
    const long Gt = md.Gt;
    const int nsig = nspin == 1 ? 1 : 3;
    m.rho.alloc(nspin * Gt);
    m.rho1.alloc(3 * nspin * Gt);
    m.tau.alloc(nspin * Gt);
    m.sigma.alloc(nsig * Gt);
    m.eps.alloc(Gt);
    m.vrho.alloc(nspin * Gt);
    m.vsigma.alloc(nsig * Gt);
    m.vtau.alloc(nspin * Gt);
    m.fcoef.alloc(5 * nspin * Gt);
    m.partial.alloc(ntiles + 1);
    m.rho_b.alloc(nspin * Gt);
    m.rho1_b.alloc(3 * nspin * Gt);
    m.tau_b.alloc(nspin * Gt);
    m.rho.zero(s);
    m.rho_b.zero(s);
    m.tau.zero(s);
    m.rho1.zero(s);
    m.tau_b.zero(s);
    m.rho1_b.zero(s);
    d_Emol.alloc(nmol);
    static bool attrs = false;
    if (!attrs) {
        set_mixed_kernel_attributes();
        attrs = true;
    }
    CGB_CUDA(cudaStreamSynchronize(s));
    m.ready = true;
}

void Grid::mixed_ready() {
    CGB_CHECK(batched || ao_order >= type, XC_ERR_STATE, "getAO must run (for the current type) before a build");
    if (!mx.ready || mx.ao_comp != (type >= 1 ? 4 : 1) || mx.nspin != nspin) prepare_mixed(mx.cfg);
}

// rho (+ grad rho, tau) of every tile point from the split density planes.
void Grid::density_passes(const __nv_bfloat16*) {
    MixedState& m = mx;
    const MixedDev& md = m.md;
    const long Gt = md.Gt;
    if (type >= 2) {
        CGB_CUDA(cudaMemsetAsync(m.tau.p, 0, sizeof(double) * nspin * Gt, stream));
        CGB_CUDA(cudaMemsetAsync(m.tau_b.p, 0, sizeof(double) * nspin * Gt, stream));
    }
    if (m.empty_tiles) {
        // points of tiles that keep no chunk have zero density; no kernel
        // writes them, so clear what an earlier build (or an incremental
        // reconstruction) left there
        CGB_CUDA(cudaMemsetAsync(m.rho.p, 0, sizeof(double) * nspin * Gt, stream));
        CGB_CUDA(cudaMemsetAsync(m.rho_b.p, 0, sizeof(double) * nspin * Gt, stream));
        if (type >= 1) {
            CGB_CUDA(cudaMemsetAsync(m.rho1.p, 0, sizeof(double) * 3 * nspin * Gt, stream));
            CGB_CUDA(cudaMemsetAsync(m.rho1_b.p, 0, sizeof(double) * 3 * nspin * Gt, stream));
        }
    }
    const auto pass = [&](int epi, int acomp, int s) {
        if (m.use16)
            launch_density16(m.tm_d, m.tm_e16d, md, m.dens_ctas, m.d_dens_off.p, m.d_dens_jobs.p, epi, acomp, s, m.rho.p,
                             m.rho1.p, m.tau.p, m.rho_b.p, m.rho1_b.p, m.tau_b.p, m.d_err.p, stream);
        else
            launch_density_tc(m.tm_d, m.tm_raw_d, md, m.dens_ctas, m.d_dens_off.p, m.d_dens_jobs.p, epi, acomp, s,
                              m.rho.p, m.rho1.p, m.tau.p, m.rho_b.p, m.rho1_b.p, m.tau_b.p, m.d_err.p, stream);
    };
    for (int s = 0; s < nspin; s++) {
        pass(type >= 1 ? 1 : 0, 0, s);
        if (type >= 2)
            for (int r = 1; r <= 3; r++) pass(2, r, s);
    }
    launch_combine((long)nspin * Gt, m.rho.p, m.rho_b.p, m.rho1.p, m.rho1_b.p, m.tau.p, m.tau_b.p, type, stream);
}

void Grid::build_mixed(const double* dD, const Functional& f, double* dE, double* dV, double float_above) {
    NvtxRange nvtx_("xc.mixed.build");
    mixed_ready();
    MixedState& m = mx;
    const MixedDev& md = m.md;
    const long Gt = md.Gt;
    const int nmol = (int)m.mols.size();
    int maxn = 0;
    for (auto& R : m.mols) maxn = std::max(maxn, R.n);
    mark(0);
    launch_split_d(dD, m.d_mols.p, nmol, nspin, md.drows, m.dcols, maxn, m.d_Dp.p, stream);
    density_passes(m.d_Dp.p);
    mark(1);
    launch_functional_fp64(f.desc, f.family, nspin, Gt, m.d_w.p, m.rho.p, m.rho1.p, m.tau.p, m.sigma.p, m.eps.p,
                           m.vrho.p, m.vsigma.p, m.vtau.p, m.fcoef.p, m.partial.p, &m.n_partial, stream,
                           float_above < 0 ? m.cfg.func_float_above : float_above);
    mark(2);
    launch_energy_mols(m.partial.p, m.d_mols.p, nmol, dE, stream);
    mark(3);
    const int ncomp = f.family >= 2 ? 4 : 1;
    for (int s = 0; s < nspin; s++) {
        v_prep(m.fcoef.p + (size_t)s * 5 * Gt, f.family);
        mark(5 + 3 * s);
        v_partials(ncomp);
        mark(6 + 3 * s);
        launch_wsum(m.d_wpart.p, m.d_item_live.p, m.d_mols.p, nmol, maxn, s, nspin, dV, stream);
        mark(7 + 3 * s);
    }
    mark(4);
}

// d_D -> d_Emol, d_V.  The launch sequence of one build is captured once
// (per functional and grid type) on a private stream and replayed on the
// grid's stream; profiling runs it eagerly so that the stage events exist.
void Grid::build_mixed_graph(const Functional& f) {
    mixed_ready();
    ensure_work();
    MixedState& m = mx;
    if (profiling) {
        build_mixed(d_D.p, f, d_Emol.p, d_V.p);
        return;
    }
    if (!m.graph || m.graph_ids != f.ids || m.graph_type != type) {
        m.drop_graph();
        if (!capture_stream) CGB_CUDA(cudaStreamCreateWithFlags(&capture_stream, cudaStreamNonBlocking));
        cudaStream_t saved = stream;
        stream = capture_stream;
        CGB_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        cudaGraph_t g = nullptr;
        try {
            build_mixed(d_D.p, f, d_Emol.p, d_V.p);
        } catch (...) {
            cudaStreamEndCapture(stream, &g);
            if (g) cudaGraphDestroy(g);
            stream = saved;
            throw;
        }
        const cudaError_t e1 = cudaStreamEndCapture(stream, &g);
        stream = saved;
        CGB_CUDA(e1);
        const cudaError_t e2 = cudaGraphInstantiate(&m.graph, g, 0);
        cudaGraphDestroy(g);
        CGB_CUDA(e2);
        m.graph_ids = f.ids;
        m.graph_type = type;
    }
    CGB_CUDA(cudaGraphLaunch(m.graph, stream));
}

// Incremental build: the density is linear in D and V_xc is linear in the
// per-point coefficients, so rho(D) = rho_ref + rho(D - D_ref) and
// V = V_ref + V(c - c_ref), with only the differences on the tensor cores.
// Their split-BF16 error is relative to the (shrinking, in an SCF) change;
// the functional and E_xc are evaluated on the reconstructed densities, in
// FP64 or (flag XC_INCREMENTAL_FP32_POTENTIALS) with FP32 potentials above
// the config's func_float_above and an FP64 energy density.  An anchor resets
// the references: a full FP64 build (anchor 1, or the first call), FP64
// densities, functional and E_xc with V on the tensor cores (anchor 2) -- both
// gathered into tile order -- or a full tensor-core build (anchor 3).
void Grid::build_incremental(const double* dD, const Functional& f, double* dE, double* dV, int anchor_flags) {
    NvtxRange nvtx_("xc.mixed.incremental");
    CGB_CHECK(!batched, XC_ERR_UNSUPPORTED, "incremental builds need the FP64 path (one molecule per grid)");
    CGB_CHECK(ao_order >= type, XC_ERR_STATE, "getAO must run (for the current type) before a build");
    ensure_work();
    mixed_ready();
    MixedState& m = mx;
    const MixedDev& md = m.md;
    const int n = basis.nbasis;
    const long Gt = md.Gt;
    const size_t nn = (size_t)n * n * nspin, G1 = (size_t)nspin * Gt;
    const auto alloc_refs = [&] {
        m.d_Dref.alloc(nn);
        m.d_rho_ref.alloc(G1);
        m.d_rho1_ref.alloc(3 * G1);
        m.d_tau_ref.alloc(G1);
        m.d_fcoef_ref.alloc(5 * G1);
        m.d_Vref.alloc(nn);
        m.d_dD.alloc(nn);
        m.d_dfcoef.alloc(5 * G1);
    };
    const int anchor = anchor_flags & 15;
    const double float_above =
        (anchor_flags & XC_INCREMENTAL_FP32_POTENTIALS) ? m.cfg.func_float_above : __builtin_huge_val();
    if (anchor == XC_ANCHOR_MIXED) {
        alloc_refs();
        build_mixed(dD, f, dE, dV);
        save_refs(dD, dV);
        m.have_ref = true;
        return;
    }
    if (anchor == 2) {
        // float-float (FP64-level) densities, FP64 functional and E_xc; V
        // from the full coefficients on the tensor cores
        density_device(dD, true);
        evaluate(f);
        energy_device(dE);
        alloc_refs();
        launch_gather(m.d_perm.p, Gt, Gp, nspin, d_rho.p, m.d_rho_ref.p, false, stream);
        launch_gather(m.d_perm.p, Gt, Gp, 3 * nspin, d_rho1.p, m.d_rho1_ref.p, false, stream);
        launch_gather(m.d_perm.p, Gt, Gp, nspin, d_tau.p, m.d_tau_ref.p, false, stream);
        launch_gather(m.d_perm.p, Gt, Gp, 5 * nspin, d_fcoef.p, m.d_fcoef_ref.p, true, stream);
        mark(3);
        const int ncomp = f.family >= 2 ? 4 : 1;
        for (int s = 0; s < nspin; s++) {
            v_prep(m.d_fcoef_ref.p + (size_t)s * 5 * Gt, f.family);
            v_partials(ncomp);
            launch_wsum(m.d_wpart.p, m.d_item_live.p, m.d_mols.p, 1, n, s, nspin, dV, stream);
        }
        mark(4);
        CGB_CUDA(cudaMemcpyAsync(m.d_Dref.p, dD, nn * 8, cudaMemcpyDeviceToDevice, stream));
        CGB_CUDA(cudaMemcpyAsync(m.d_Vref.p, dV, nn * 8, cudaMemcpyDeviceToDevice, stream));
        m.have_ref = true;
        return;
    }
    if (anchor == 1 || !m.have_ref) {
        density_device(dD);
        evaluate(f);
        energy_device(dE);
        fock_device(dV, f.family);
        alloc_refs();
        CGB_CUDA(cudaMemcpyAsync(m.d_Dref.p, dD, nn * 8, cudaMemcpyDeviceToDevice, stream));
        CGB_CUDA(cudaMemcpyAsync(m.d_Vref.p, dV, nn * 8, cudaMemcpyDeviceToDevice, stream));
        launch_gather(m.d_perm.p, Gt, Gp, nspin, d_rho.p, m.d_rho_ref.p, false, stream);
        launch_gather(m.d_perm.p, Gt, Gp, 3 * nspin, d_rho1.p, m.d_rho1_ref.p, false, stream);
        launch_gather(m.d_perm.p, Gt, Gp, nspin, d_tau.p, m.d_tau_ref.p, false, stream);
        launch_gather(m.d_perm.p, Gt, Gp, 5 * nspin, d_fcoef.p, m.d_fcoef_ref.p, true, stream);
        m.have_ref = true;
        return;
    }
    int maxn = n;
    mark(0);
    launch_axpby((long)nn, 1.0, dD, -1.0, m.d_Dref.p, m.d_dD.p, stream);
    launch_split_d(m.d_dD.p, m.d_mols.p, 1, nspin, md.drows, m.dcols, maxn, m.d_Dp.p, stream);
    density_passes(m.d_Dp.p);
    launch_axpby((long)G1, 1.0, m.rho.p, 1.0, m.d_rho_ref.p, m.rho.p, stream);
    if (type >= 1) launch_axpby((long)(3 * G1), 1.0, m.rho1.p, 1.0, m.d_rho1_ref.p, m.rho1.p, stream);
    if (type >= 2) launch_axpby((long)G1, 1.0, m.tau.p, 1.0, m.d_tau_ref.p, m.tau.p, stream);
    mark(1);
    // FP64 functional on the reconstructed densities
    launch_functional_fp64(f.desc, f.family, nspin, Gt, m.d_w.p, m.rho.p, m.rho1.p, m.tau.p, m.sigma.p, m.eps.p,
                           m.vrho.p, m.vsigma.p, m.vtau.p, m.fcoef.p, m.partial.p, &m.n_partial, stream, float_above);
    mark(2);
    launch_energy_mols(m.partial.p, m.d_mols.p, 1, dE, stream);
    mark(3);
    launch_axpby((long)(5 * G1), 1.0, m.fcoef.p, -1.0, m.d_fcoef_ref.p, m.d_dfcoef.p, stream);
    const int ncomp = f.family >= 2 ? 4 : 1;
    for (int s = 0; s < nspin; s++) {
        v_prep(m.d_dfcoef.p + (size_t)s * 5 * Gt, f.family);
        v_partials(ncomp);
        launch_wsum(m.d_wpart.p, m.d_item_live.p, m.d_mols.p, 1, maxn, s, nspin, dV, stream);
    }
    launch_axpby((long)nn, 1.0, dV, 1.0, m.d_Vref.p, dV, stream);
    mark(4);
    save_refs(dD, dV);
}

// The current D, tile-order densities, coefficients and V become the references.
void Grid::save_refs(const double* dD, const double* dV) {
    MixedState& m = mx;
    const size_t nn = (size_t)basis.nbasis * basis.nbasis * nspin, G1 = (size_t)nspin * m.md.Gt;
    CGB_CUDA(cudaMemcpyAsync(m.d_Dref.p, dD, nn * 8, cudaMemcpyDeviceToDevice, stream));
    CGB_CUDA(cudaMemcpyAsync(m.d_rho_ref.p, m.rho.p, G1 * 8, cudaMemcpyDeviceToDevice, stream));
    if (type >= 1) CGB_CUDA(cudaMemcpyAsync(m.d_rho1_ref.p, m.rho1.p, 3 * G1 * 8, cudaMemcpyDeviceToDevice, stream));
    if (type >= 2) CGB_CUDA(cudaMemcpyAsync(m.d_tau_ref.p, m.tau.p, G1 * 8, cudaMemcpyDeviceToDevice, stream));
    CGB_CUDA(cudaMemcpyAsync(m.d_fcoef_ref.p, m.fcoef.p, 5 * G1 * 8, cudaMemcpyDeviceToDevice, stream));
    CGB_CUDA(cudaMemcpyAsync(m.d_Vref.p, dV, nn * 8, cudaMemcpyDeviceToDevice, stream));
}

// The R operands of V for one spin's coefficients (tile order).
void Grid::v_prep(const double* fcoef_s, int family) {
    MixedState& m = mx;
    if (m.use16)
        launch_prep16(m.md, family, fcoef_s, m.d_R16.p, stream);
    else
        launch_prep_z(m.md, family, fcoef_s, m.d_Z.p, m.d_c2.p, stream);
}

// W partials of every V work item on the tensor cores (components 0..ncomp-1).
void Grid::v_partials(int ncomp) {
    MixedState& m = mx;
    if (m.use16)
        launch_fock16(m.tm_e16, m.tm_r16, m.md.rows, m.fock_ctas, m.d_fock_off.p, m.d_fock_jobs.p, ncomp, m.d_wpart.p,
                      m.d_err.p, stream);
    else
        launch_fock_tc(m.tm_raw_f, m.tm_z, m.md.rows, m.fock_ctas, m.d_fock_off.p, m.d_fock_jobs.p, m.d_c2.p, ncomp,
                       m.d_wpart.p, m.d_err.p, stream);
}

int Grid::mixed_error() {
    if (!mx.ready) return 0;
    int e = 0;
    CGB_CUDA(cudaMemcpyAsync(&e, mx.d_err.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
    CGB_CUDA(cudaStreamSynchronize(stream));
    if (e) CGB_CUDA(cudaMemsetAsync(mx.d_err.p, 0, sizeof(int), stream));
    return e;
}

}  // namespace cgb

namespace cgb {

// Ground-state grad rho, vsigma and the second derivatives of the last
// Evaluate("ev") / Evaluate("f") (FP64 grid) in tile order, for response_mixed.
void Grid::response_tiles_prepare() {
    CGB_CHECK(!batched, XC_ERR_UNSUPPORTED, "response builds are per molecule");
    CGB_CHECK(have_fxc && (fxc_family == 0 || (have_potential && eval_family >= 1)), XC_ERR_STATE,
              "the response needs Evaluate(\"ev\") and Evaluate(\"f\") on the current density");
    mixed_ready();
    MixedState& m = mx;
    const long Gt = m.md.Gt;
    const int nsig = nspin == 1 ? 1 : 3, nf2 = nspin == 1 ? 3 : 15;
    const size_t nn = (size_t)basis.nbasis * basis.nbasis;
    d_rt_rho1.alloc((size_t)3 * nspin * Gt);
    d_rt_vsig.alloc((size_t)nsig * Gt);
    d_rt_f2.alloc((size_t)nf2 * Gt);
    d_rt_fcU.alloc((size_t)5 * nspin * Gt);
    d_rt_D.alloc(nspin * nn);
    d_rt_V.alloc(nspin * nn);
    if (fxc_family >= 1) {
        launch_gather(m.d_perm.p, Gt, Gp, 3 * nspin, d_rho1.p, d_rt_rho1.p, true, stream);
        launch_gather(m.d_perm.p, Gt, Gp, nsig, d_vsigma.p, d_rt_vsig.p, true, stream);
    }
    launch_gather(m.d_perm.p, Gt, Gp, nf2, d_f2.p, d_rt_f2.p, true, stream);
}

// V_U of nmat matrices D_U (s, nmat, n, n) on the tensor cores: per matrix the
// split-BF16 density of its symmetric part (rho_U, grad rho_U in tile order),
// the response coefficients (FP64) and V_U through the V kernels, FP64 sums.
void Grid::response_mixed(const double* dDU, int nmat, double* dFU) {
    NvtxRange nvtx_("xc.mixed.response");
    MixedState& m = mx;
    const MixedDev& md = m.md;
    const long Gt = md.Gt;
    const int n = basis.nbasis;
    const size_t nn = (size_t)n * n;
    for (int k = 0; k < nmat; k++) {
        // stage timers (xc_grid_profile) on the first matrix: [split_d + density + combine,
        // coefficients + R planes, V partials, V sum] of spin 0
        const bool first = k == 0;
        for (int s = 0; s < nspin; s++)
            CGB_CUDA(cudaMemcpyAsync(d_rt_D.p + s * nn, dDU + ((size_t)s * nmat + k) * nn, nn * sizeof(double),
                                     cudaMemcpyDeviceToDevice, stream));
        if (first) mark(0);
        launch_split_d(d_rt_D.p, m.d_mols.p, 1, nspin, md.drows, m.dcols, n, m.d_Dp.p, stream);
        density_passes(m.d_Dp.p);
        if (first) mark(1);
        launch_response_coef(fxc_family, nspin, Gt, 1, m.d_w.p, d_rt_rho1.p, d_rt_vsig.p, d_rt_f2.p, m.rho.p,
                             m.rho1.p, d_rt_fcU.p, stream);
        for (int s = 0; s < nspin; s++) {
            v_prep(d_rt_fcU.p + (size_t)s * 5 * Gt, fxc_family);
            if (first && s == 0) mark(2);
            v_partials(1);
            if (first && s == 0) mark(3);
            launch_wsum(m.d_wpart.p, m.d_item_live.p, m.d_mols.p, 1, n, s, nspin, d_rt_V.p, stream);
            if (first && s == 0) mark(4);
        }
        for (int s = 0; s < nspin; s++)
            CGB_CUDA(cudaMemcpyAsync(dFU + ((size_t)s * nmat + k) * nn, d_rt_V.p + s * nn, nn * sizeof(double),
                                     cudaMemcpyDeviceToDevice, stream));
    }
}

}  // namespace cgb
