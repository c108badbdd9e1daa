// Host orchestration of the mixed-precision build: tile/chunk screening,
// split-BF16 AO stores in both layouts, TMA tensor maps, and the per-build
// launch sequence (D split -> tensor-core density -> functional -> E_xc ->
// R operand -> tensor-core V partials -> FP64 reduction).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "mixed.h"
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

void Grid::prepare_mixed(double thr) {
    MixedState& m = mx;
    m.ready = false;
    m.thr = thr;
    const int n = basis.nbasis;
    MixedDev& md = m.md;
    md.ntiles = (int)((Gp + kTilePts - 1) / kTilePts);
    md.Gt = (long)md.ntiles * kTilePts;
    md.nchunk = (n + kChunk - 1) / kChunk;
    md.npad = md.nchunk * kChunk;
    // shell significance per tile (bounding sphere of the tile's points)
    const int nsh = (int)basis.shells.size();
    std::vector<double> ext(nsh);
    for (int s = 0; s < nsh; s++) ext[s] = shell_extent(basis, basis.shells[s], thr);
    m.h_nkept.assign(md.ntiles, 0);
    m.h_chunks.assign((size_t)md.ntiles * md.nchunk, 0);
    m.h_slot.assign((size_t)md.ntiles * md.nchunk, -1);
    std::vector<int> tile_shells, tile_off(1, 0);
    int maxkept = 0;
    m.kept_pairs = 0;
    for (int t = 0; t < md.ntiles; t++) {
        const long lo = (long)t * kTilePts, hi = std::min(Gp, lo + kTilePts);
        double cx = 0, cy = 0, cz = 0;
        for (long k = lo; k < hi; k++) {
            cx += hx[k];
            cy += hy[k];
            cz += hz[k];
        }
        const double inv = 1.0 / (double)(hi - lo);
        cx *= inv; cy *= inv; cz *= inv;
        double rad = 0;
        for (long k = lo; k < hi; k++)
            rad = std::max(rad, std::sqrt((hx[k] - cx) * (hx[k] - cx) + (hy[k] - cy) * (hy[k] - cy) + (hz[k] - cz) * (hz[k] - cz)));
        std::vector<char> keep(md.nchunk, 0);
        for (int s = 0; s < nsh; s++) {
            const Shell& sh = basis.shells[s];
            const double d = std::sqrt((sh.x - cx) * (sh.x - cx) + (sh.y - cy) * (sh.y - cy) + (sh.z - cz) * (sh.z - cz));
            if (thr > 0 && d - rad > ext[s]) continue;
            const int f0 = sh.first, f1 = sh.first + shell_size(sh.type) - 1;
            for (int c = f0 / kChunk; c <= f1 / kChunk; c++) keep[c] = 1;
        }
        int nk = 0;
        for (int c = 0; c < md.nchunk; c++)
            if (keep[c]) {
                m.h_chunks[(size_t)t * md.nchunk + nk] = c;
                m.h_slot[(size_t)t * md.nchunk + c] = nk;
                nk++;
            }
        m.h_nkept[t] = nk;
        maxkept = std::max(maxkept, nk);
        m.kept_pairs += (long)(nk * kChunk) * (nk * kChunk);
        for (int s = 0; s < nsh; s++) {
            const Shell& sh = basis.shells[s];
            const int f0 = sh.first, f1 = sh.first + shell_size(sh.type) - 1;
            bool any = false;
            for (int c = f0 / kChunk; c <= f1 / kChunk; c++) any |= keep[c] != 0;
            if (any) tile_shells.push_back(s);
        }
        tile_off.push_back((int)tile_shells.size());
    }
    md.kmax = std::max(1, maxkept) * kChunk;
    m.d_nkept.upload(m.h_nkept.data(), m.h_nkept.size(), stream);
    m.d_chunks.upload(m.h_chunks.data(), m.h_chunks.size(), stream);
    m.d_slot.upload(m.h_slot.data(), m.h_slot.size(), stream);
    m.d_tile_shells.upload(tile_shells.data(), tile_shells.size(), stream);
    m.d_tile_shell_off.upload(tile_off.data(), tile_off.size(), stream);
    {
        static double table[kMaxL + 1][2 * kMaxL + 1][(kMaxL + 1) * (kMaxL + 2) / 2];
        solid_harmonic_table(table);
        m.d_shtab.upload(&table[0][0][0], sizeof(table) / sizeof(double), stream);
    }
    const long TK = (long)md.ntiles * md.kmax;
    m.d_pf.alloc((size_t)12 * md.Gt * md.kmax);
    m.d_fp.alloc((size_t)(12 * TK + 64) * 128);
    m.d_e32.alloc((size_t)4 * TK * 128);
    m.d_pf.zero(stream);
    m.d_fp.zero(stream);
    m.d_e32.zero(stream);
    md.tile_nkept = m.d_nkept.p;
    md.tile_chunks = m.d_chunks.p;
    md.tile_slot = m.d_slot.p;
    md.pf = m.d_pf.p;
    md.fp = m.d_fp.p;
    md.e32 = m.d_e32.p;
    launch_ao_mixed(md, dev_shells(), m.d_tile_shells.p, m.d_tile_shell_off.p, d_x.p, d_y.p, d_z.p, Gp, m.d_shtab.p,
                    m.d_pf.p, m.d_fp.p, m.d_e32.p, stream);
    // per-build operands
    m.r_ncomp = type >= 2 ? 4 : 1;
    m.d_R.alloc((size_t)(m.r_ncomp * 3 * TK + 64) * 128);
    m.d_R.zero(stream);
    m.d_Dp.alloc((size_t)nspin * 3 * md.npad * md.npad);
    m.nblk = (md.nchunk + 1) / 2;
    int dev = 0, nsm = 148;
    CGB_CUDA(cudaGetDevice(&dev));
    CGB_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = m.nblk * m.nblk;
    m.nsplit = std::max(1, std::min(md.ntiles, (2 * nsm + blocks - 1) / blocks));
    const size_t npadw = (size_t)m.nblk * 128;
    m.d_wpart.alloc((size_t)nspin * m.nsplit * npadw * npadw);
    m.d_err.alloc(1);
    m.d_err.zero(stream);
    make_tmap_bf16(&m.tm_pf, m.d_pf.p, md.kmax, 12 * md.Gt, 64, 128);
    make_tmap_bf16(&m.tm_fp, m.d_fp.p, 128, 12 * TK + 64, 64, 64);
    make_tmap_bf16(&m.tm_r, m.d_R.p, 128, m.r_ncomp * 3 * TK + 64, 64, 64);
    make_tmap_bf16(&m.tm_d, m.d_Dp.p, md.npad, (uint64_t)nspin * 3 * md.npad, 64, 64);
    CGB_CUDA(cudaStreamSynchronize(stream));
    m.ready = true;
}

void Grid::build_mixed(const double* dD, const Functional& f, double* dE, double* dV) {
    MixedState& m = mx;
    CGB_CHECK(ao_order >= type, XC_ERR_STATE, "getAO must run (for the current type) before a build");
    if (!m.ready || m.r_ncomp != (type >= 2 ? 4 : 1)) prepare_mixed(m.ready ? m.thr : kMixedScreen);
    ensure_work();
    const MixedDev& md = m.md;
    const int n = basis.nbasis;
    mark(0);
    launch_split_d(dD, n, md.npad, nspin, m.d_Dp.p, stream);
    if (type >= 2) CGB_CUDA(cudaMemsetAsync(d_tau.p, 0, sizeof(double) * nspin * Gp, stream));
    for (int s = 0; s < nspin; s++) {
        launch_density_tc(m.tm_pf, m.tm_d, md, type >= 1 ? 1 : 0, 0, s, d_rho.p, d_rho1.p, d_tau.p, Gp, m.d_err.p,
                          stream);
        if (type >= 2)
            for (int r = 1; r <= 3; r++)
                launch_density_tc(m.tm_pf, m.tm_d, md, 2, r, s, d_rho.p, d_rho1.p, d_tau.p, Gp, m.d_err.p, stream);
    }
    have_density = true;
    evaluate(f, kMixedFuncFloat);  // marks 1
    energy_device(dE);  // marks 2
    mark(3);
    const size_t npadw = (size_t)m.nblk * 128;
    const int ncomp = f.family >= 2 ? 4 : 1;
    for (int s = 0; s < nspin; s++) {
        launch_prep_r(md, ncomp, f.family, d_fcoef.p + (size_t)s * 5 * Gp, Gp, m.d_R.p, stream);
        double* wp = m.d_wpart.p + (size_t)s * m.nsplit * npadw * npadw;
        const int r_rows = (int)((long)m.r_ncomp * 3 * md.ntiles * md.kmax);
        launch_fock_tc(m.tm_fp, m.tm_r, md, ncomp, r_rows, m.nblk, m.nsplit, wp, m.d_err.p, stream);
        launch_wsum(wp, m.nsplit, (int)npadw, n, dV + (size_t)s * n * n, stream);
    }
    mark(4);
}

// Incremental build: the density is linear in D and V_xc is linear in the
// per-point coefficients, so rho(D) = rho_ref + rho(D - D_ref) and
// V = V_ref + V(c - c_ref), with only the differences on the tensor cores.
// Their split-BF16 error is relative to the (shrinking, in an SCF) change;
// the functional and E_xc are evaluated in FP64 on the reconstructed
// densities.  An anchor (or the first call) is a full FP64 build that resets
// the references.
void Grid::build_incremental(const double* dD, const Functional& f, double* dE, double* dV, bool anchor) {
    MixedState& m = mx;
    CGB_CHECK(ao_order >= type, XC_ERR_STATE, "getAO must run (for the current type) before a build");
    ensure_work();
    const int n = basis.nbasis;
    const size_t nn = (size_t)n * n * nspin, G1 = (size_t)nspin * Gp;
    if (anchor || !m.have_ref) {
        density_device(dD);
        evaluate(f);
        energy_device(dE);
        fock_device(dV, f.family);
        m.d_Dref.alloc(nn);
        m.d_rho_ref.alloc(G1);
        m.d_rho1_ref.alloc(3 * G1);
        m.d_tau_ref.alloc(G1);
        m.d_fcoef_ref.alloc(5 * G1);
        m.d_Vref.alloc(nn);
        m.d_dD.alloc(nn);
        m.d_dfcoef.alloc(5 * G1);
        CGB_CUDA(cudaMemcpyAsync(m.d_Dref.p, dD, nn * 8, cudaMemcpyDeviceToDevice, stream));
        CGB_CUDA(cudaMemcpyAsync(m.d_rho_ref.p, d_rho.p, G1 * 8, cudaMemcpyDeviceToDevice, stream));
        CGB_CUDA(cudaMemcpyAsync(m.d_rho1_ref.p, d_rho1.p, 3 * G1 * 8, cudaMemcpyDeviceToDevice, stream));
        CGB_CUDA(cudaMemcpyAsync(m.d_tau_ref.p, d_tau.p, G1 * 8, cudaMemcpyDeviceToDevice, stream));
        CGB_CUDA(cudaMemcpyAsync(m.d_fcoef_ref.p, d_fcoef.p, 5 * G1 * 8, cudaMemcpyDeviceToDevice, stream));
        CGB_CUDA(cudaMemcpyAsync(m.d_Vref.p, dV, nn * 8, cudaMemcpyDeviceToDevice, stream));
        m.have_ref = true;
        return;
    }
    if (!m.ready || m.r_ncomp != (type >= 2 ? 4 : 1)) prepare_mixed(m.ready ? m.thr : kMixedScreen);
    const MixedDev& md = m.md;
    mark(0);
    launch_axpby((long)nn, 1.0, dD, -1.0, m.d_Dref.p, m.d_dD.p, stream);
    launch_split_d(m.d_dD.p, n, md.npad, nspin, m.d_Dp.p, stream);
    if (type >= 2) CGB_CUDA(cudaMemsetAsync(d_tau.p, 0, sizeof(double) * G1, stream));
    for (int s = 0; s < nspin; s++) {
        launch_density_tc(m.tm_pf, m.tm_d, md, type >= 1 ? 1 : 0, 0, s, d_rho.p, d_rho1.p, d_tau.p, Gp, m.d_err.p,
                          stream);
        if (type >= 2)
            for (int r = 1; r <= 3; r++)
                launch_density_tc(m.tm_pf, m.tm_d, md, 2, r, s, d_rho.p, d_rho1.p, d_tau.p, Gp, m.d_err.p, stream);
    }
    launch_axpby((long)G1, 1.0, d_rho.p, 1.0, m.d_rho_ref.p, d_rho.p, stream);
    if (type >= 1) launch_axpby((long)(3 * G1), 1.0, d_rho1.p, 1.0, m.d_rho1_ref.p, d_rho1.p, stream);
    if (type >= 2) launch_axpby((long)G1, 1.0, d_tau.p, 1.0, m.d_tau_ref.p, d_tau.p, stream);
    have_density = true;
    evaluate(f);  // FP64 functional on the reconstructed densities
    energy_device(dE);
    mark(3);
    launch_axpby((long)(5 * G1), 1.0, d_fcoef.p, -1.0, m.d_fcoef_ref.p, m.d_dfcoef.p, stream);
    const size_t npadw = (size_t)m.nblk * 128;
    const int ncomp = f.family >= 2 ? 4 : 1;
    for (int s = 0; s < nspin; s++) {
        launch_prep_r(md, ncomp, f.family, m.d_dfcoef.p + (size_t)s * 5 * Gp, Gp, m.d_R.p, stream);
        double* wp = m.d_wpart.p + (size_t)s * m.nsplit * npadw * npadw;
        const int r_rows = (int)((long)m.r_ncomp * 3 * md.ntiles * md.kmax);
        launch_fock_tc(m.tm_fp, m.tm_r, md, ncomp, r_rows, m.nblk, m.nsplit, wp, m.d_err.p, stream);
        launch_wsum(wp, m.nsplit, (int)npadw, n, dV + (size_t)s * n * n, stream);
    }
    launch_axpby((long)nn, 1.0, dV, 1.0, m.d_Vref.p, dV, stream);
    mark(4);
    // the new references
    CGB_CUDA(cudaMemcpyAsync(m.d_Dref.p, dD, nn * 8, cudaMemcpyDeviceToDevice, stream));
    CGB_CUDA(cudaMemcpyAsync(m.d_rho_ref.p, d_rho.p, G1 * 8, cudaMemcpyDeviceToDevice, stream));
    if (type >= 1) CGB_CUDA(cudaMemcpyAsync(m.d_rho1_ref.p, d_rho1.p, 3 * G1 * 8, cudaMemcpyDeviceToDevice, stream));
    if (type >= 2) CGB_CUDA(cudaMemcpyAsync(m.d_tau_ref.p, d_tau.p, G1 * 8, cudaMemcpyDeviceToDevice, stream));
    CGB_CUDA(cudaMemcpyAsync(m.d_fcoef_ref.p, d_fcoef.p, 5 * G1 * 8, cudaMemcpyDeviceToDevice, stream));
    CGB_CUDA(cudaMemcpyAsync(m.d_Vref.p, dV, nn * 8, cudaMemcpyDeviceToDevice, stream));
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
