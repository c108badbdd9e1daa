// C-ABI implementation: the Grid / ExchangeCorrelation objects and every
// extern "C" entry point of include/chinium_xc.h.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <functional>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "common.h"
#include "kernels.h"
#include "model.h"
#include "nvtx.h"
#include "xc_state.h"

namespace cgb {

namespace {
thread_local std::string g_last_error;
std::once_flag g_sh_once;
}  // namespace

void set_last_error(const std::string& msg) { g_last_error = msg; }

void ensure_device() {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0)
        throw Error(XC_ERR_CUDA, std::string("no CUDA device available: ") + cudaGetErrorString(e));
    std::call_once(g_sh_once, [] { upload_solid_harmonics(); });
}

// ------------------------------------------------------------ grid build
// SphericalGrid (GridGeneration.cpp:73-133) for one atom: points in
// generation order with radial * 4 pi * Lebedev weights.
static void atom_points(const std::string& grid, int Z, const double* c, int atom, std::vector<double>& X,
                        std::vector<double>& Y, std::vector<double>& Zc, std::vector<double>& W, std::vector<int>& owner) {
    const GridRecipe& r = grid_recipe(grid, Z);
    const int nt = r.nshells_total;
    std::function<double(double)> ri, rw;
    if (r.formula == "de2") {
        CGB_CHECK(r.params.size() >= 3, XC_ERR_IO, "corrupt de2 recipe");
        const double a = r.params[0], t2 = r.params[1], t3 = r.params[2];
        const double h = (t3 - t2) / (double)(nt - 1);
        ri = [=](double i) {
            const double xi = h * i + t2;
            return std::exp(a * xi - std::exp(-xi));
        };
        rw = [=](double i) {
            const double xi = h * i + t2;
            return std::exp(3 * a * xi - 3 * std::exp(-xi)) * (a + std::exp(-xi)) * h;
        };
    } else if (r.formula == "em") {
        CGB_CHECK(r.params.size() >= 1, XC_ERR_IO, "corrupt em recipe");
        const double R = r.params[0];
        ri = [=](double i) {
            const double ii = i + 1;
            return R * std::pow(ii / (nt + 1 - ii), 2);
        };
        rw = [=](double i) {
            const double ii = i + 1;
            return 2 * std::pow(R, 3) * (nt + 1) * std::pow(ii, 5) / std::pow(nt + 1 - ii, 7);
        };
    } else {
        throw Error(XC_ERR_IO, "Unrecognized radial formula!");
    }
    int ish = 0;
    for (auto [npts, nsh] : r.groups) {
        const std::vector<double>& leb = lebedev_rule(npts);
        for (int s = 0; s < nsh; s++, ish++) {
            const double rad = ri(ish), wr = rw(ish);
            for (int k = 0; k < npts; k++) {
                X.push_back(leb[4 * k] * rad + c[0]);
                Y.push_back(leb[4 * k + 1] * rad + c[1]);
                Zc.push_back(leb[4 * k + 2] * rad + c[2]);
                W.push_back(wr * (4 * M_PI * leb[4 * k + 3]));
                owner.push_back(atom);
            }
        }
    }
}

// RecursiveCut (GridGeneration.cpp:177-210) as it behaves: leaves are
// recursive halves of generation order (its partition step only reorders
// the first four points, which stay in the left half).
static void halve(long lo, long n, std::vector<std::pair<long, long>>& out) {
    if (n <= kMaxBlockPts) {
        out.emplace_back(lo, n);
        return;
    }
    const long h = n / 2;
    halve(lo, h, out);
    halve(lo + h, n - h, out);
}

void Grid::build(const BasisSet& bs, const std::string& grid_name, int ns, double thr) {
    NvtxRange nvtx_("xc.grid");
    basis = bs;
    nspin = ns;
    screen_thr = thr;
    const int natoms = bs.natoms();
    std::vector<double> X, Y, Z, Win;
    std::vector<int> own;
    for (int a = 0; a < natoms; a++) atom_points(grid_name, bs.Z[a], &bs.xyz[3 * a], a, X, Y, Z, Win, own);
    npoints = (long)X.size();
    std::vector<std::pair<long, long>> ranges;
    halve(0, npoints, ranges);
    // SubGrid::SubGrid (GridGeneration.cpp:212-230): pad to a multiple of 8,
    // padded coordinates copy the first points, padded weights zero.
    hx.clear(); hy.clear(); hz.clear();
    std::vector<double> hw;
    std::vector<int> hown;
    blocks.clear();
    for (auto [lo, n] : ranges) {
        BlockDesc bd{};
        bd.pt_off = (int)hx.size();
        bd.nreal = (int)n;
        bd.ng = (int)((n + 7) & ~7L);
        for (int k = 0; k < bd.ng; k++) {
            const long src = lo + (k < n ? k : k - n);
            hx.push_back(X[src]);
            hy.push_back(Y[src]);
            hz.push_back(Z[src]);
            hw.push_back(k < n ? Win[src] : 0.0);
            hown.push_back(own[src]);
        }
        blocks.push_back(bd);
    }
    Gp = (long)hx.size();
    // shell screening per block: bounding sphere of the block's real points
    std::vector<double> ext(bs.shells.size());
    for (size_t s = 0; s < bs.shells.size(); s++) ext[s] = shell_extent(bs, bs.shells[s], thr);
    basis_lists.clear();
    shell_lists.clear();
    max_nb = 0;
    screened_pairs = 0;
    for (auto& bd : blocks) {
        double cx = 0, cy = 0, cz = 0;
        for (int k = 0; k < bd.nreal; k++) {
            cx += hx[bd.pt_off + k];
            cy += hy[bd.pt_off + k];
            cz += hz[bd.pt_off + k];
        }
        cx /= bd.nreal; cy /= bd.nreal; cz /= bd.nreal;
        double rad = 0;
        for (int k = 0; k < bd.ng; k++) {
            const double dx = hx[bd.pt_off + k] - cx, dy = hy[bd.pt_off + k] - cy, dz = hz[bd.pt_off + k] - cz;
            rad = std::max(rad, std::sqrt(dx * dx + dy * dy + dz * dz));
        }
        bd.sh_off = (int)shell_lists.size();
        bd.bas_off = (int)basis_lists.size();
        int nb = 0, nsh = 0;
        for (size_t s = 0; s < bs.shells.size(); s++) {
            const Shell& sh = bs.shells[s];
            const double d = std::sqrt((sh.x - cx) * (sh.x - cx) + (sh.y - cy) * (sh.y - cy) + (sh.z - cz) * (sh.z - cz));
            if (thr > 0 && d - rad > ext[s]) continue;
            shell_lists.push_back((int)s);
            for (int f = 0; f < shell_size(sh.type); f++) basis_lists.push_back(sh.first + f);
            nb += shell_size(sh.type);
            nsh++;
        }
        bd.nb = nb;
        bd.nsh = nsh;
        max_nb = std::max(max_nb, nb);
        screened_pairs += (long)nb * nb;
    }
    // device: points, Becke weights
    ensure_device();
    d_x.upload(hx.data(), Gp, stream);
    d_y.upload(hy.data(), Gp, stream);
    d_z.upload(hz.data(), Gp, stream);
    DevBuf<double> d_win;
    DevBuf<int> d_own;
    d_win.upload(hw.data(), Gp, stream);
    d_own.upload(hown.data(), Gp, stream);
    d_atoms.upload(bs.xyz.data(), bs.xyz.size(), stream);
    d_w.alloc(Gp);
    launch_becke(natoms, d_atoms.p, Gp, d_x.p, d_y.p, d_z.p, d_own.p, d_win.p, d_w.p, stream);
    // shells
    std::vector<int> st, sl, snp, spo, sf;
    std::vector<double> sxyz;
    for (auto& sh : bs.shells) {
        st.push_back(sh.type);
        sl.push_back(sh.l);
        snp.push_back(sh.nprim);
        spo.push_back(sh.prim_off);
        sf.push_back(sh.first);
        sxyz.push_back(sh.x);
        sxyz.push_back(sh.y);
        sxyz.push_back(sh.z);
    }
    d_sh_type.upload(st.data(), st.size(), stream);
    d_sh_l.upload(sl.data(), sl.size(), stream);
    d_sh_nprim.upload(snp.data(), snp.size(), stream);
    d_sh_poff.upload(spo.data(), spo.size(), stream);
    d_sh_first.upload(sf.data(), sf.size(), stream);
    d_sh_xyz.upload(sxyz.data(), sxyz.size(), stream);
    d_exps.upload(bs.exps.data(), bs.exps.size(), stream);
    d_coefs.upload(bs.coefs.data(), bs.coefs.size(), stream);
    d_lists.upload(basis_lists.data(), basis_lists.size(), stream);
    d_shell_lists.upload(shell_lists.data(), shell_lists.size(), stream);
    CGB_CUDA(cudaStreamSynchronize(stream));
}

// Batch of molecules: each molecule's grid is generated (and Becke
// partitioned) on its own; their real points become the molecule sources of
// the mixed path, and their shells one combined basis in which every
// molecule's functions start at a multiple of 64.
void Grid::build_batch(const std::vector<BasisSet>& mols, const std::string& grid_name, int ns) {
    CGB_CHECK(!mols.empty(), XC_ERR_ARG, "empty batch");
    nspin = ns;
    screen_thr = 0;
    batched = true;
    BasisSet comb;
    sources.clear();
    mol_n.clear();
    npoints = 0;
    int f0 = 0;
    for (const BasisSet& b : mols) {
        Grid g;
        g.stream = stream;
        g.build(b, grid_name, ns, 0.0);
        std::vector<double> w(g.Gp);
        CGB_CUDA(cudaMemcpyAsync(w.data(), g.d_w.p, g.Gp * sizeof(double), cudaMemcpyDeviceToHost, stream));
        CGB_CUDA(cudaStreamSynchronize(stream));
        MolSource S;
        S.n = b.nbasis;
        S.f0 = f0;
        S.sh0 = (int)comb.shells.size();
        const int atom0 = comb.natoms(), prim0 = (int)comb.exps.size();
        comb.Z.insert(comb.Z.end(), b.Z.begin(), b.Z.end());
        comb.xyz.insert(comb.xyz.end(), b.xyz.begin(), b.xyz.end());
        comb.exps.insert(comb.exps.end(), b.exps.begin(), b.exps.end());
        comb.coefs.insert(comb.coefs.end(), b.coefs.begin(), b.coefs.end());
        for (Shell sh : b.shells) {
            sh.atom += atom0;
            sh.first += f0;
            sh.prim_off += prim0;
            comb.shells.push_back(sh);
        }
        S.sh1 = (int)comb.shells.size();
        for (const BlockDesc& bd : g.blocks)
            for (int k = 0; k < bd.nreal; k++) {
                const long i = bd.pt_off + k;
                S.x.push_back(g.hx[i]);
                S.y.push_back(g.hy[i]);
                S.z.push_back(g.hz[i]);
                S.w.push_back(w[i]);
            }
        npoints += (long)S.x.size();
        sources.push_back(std::move(S));
        mol_n.push_back(b.nbasis);
        f0 += (b.nbasis + 63) / 64 * 64;
    }
    comb.nbasis = f0;
    basis = comb;
    Gp = 0;
    blocks.clear();
    basis_lists.clear();
    shell_lists.clear();
    hx.clear();
    hy.clear();
    hz.clear();
    ensure_device();
    std::vector<int> st, sl, snp, spo, sf;
    std::vector<double> sxyz;
    for (auto& sh : basis.shells) {
        st.push_back(sh.type);
        sl.push_back(sh.l);
        snp.push_back(sh.nprim);
        spo.push_back(sh.prim_off);
        sf.push_back(sh.first);
        sxyz.push_back(sh.x);
        sxyz.push_back(sh.y);
        sxyz.push_back(sh.z);
    }
    d_sh_type.upload(st.data(), st.size(), stream);
    d_sh_l.upload(sl.data(), sl.size(), stream);
    d_sh_nprim.upload(snp.data(), snp.size(), stream);
    d_sh_poff.upload(spo.data(), spo.size(), stream);
    d_sh_first.upload(sf.data(), sf.size(), stream);
    d_sh_xyz.upload(sxyz.data(), sxyz.size(), stream);
    d_exps.upload(basis.exps.data(), basis.exps.size(), stream);
    d_coefs.upload(basis.coefs.data(), basis.coefs.size(), stream);
    d_atoms.upload(basis.xyz.data(), basis.xyz.size(), stream);
    CGB_CUDA(cudaStreamSynchronize(stream));
}

DevShells Grid::dev_shells() const {
    DevShells s;
    s.nshell = (int)basis.shells.size();
    s.type = d_sh_type.p;
    s.l = d_sh_l.p;
    s.nprim = d_sh_nprim.p;
    s.prim_off = d_sh_poff.p;
    s.first = d_sh_first.p;
    s.xyz = d_sh_xyz.p;
    s.exps = d_exps.p;
    s.coefs = d_coefs.p;
    return s;
}

void Grid::get_ao(int derivative) {
    NvtxRange nvtx_("xc.getAO");
    CGB_CHECK(derivative >= 0, XC_ERR_ARG, "negative derivative order");
    if (batched) return;  // the mixed path evaluates its own FP32 AO store at the first build
    const int order = type + derivative;
    CGB_CHECK(order <= 2, XC_ERR_UNSUPPORTED, "AO derivative order above 2 is not stored by this build");
    // Hessians (AO2) only when a derivative beyond the functional's own order is asked for (gradients)
    ncomp = (derivative >= 1 && order >= 2) ? 10 : (order >= 1 ? 4 : 1);
    long long off = 0;
    for (auto& bd : blocks) {
        bd.ao_off = off;
        off += (long long)ncomp * bd.nb * bd.ng;
    }
    ao_elements = off / ncomp;
    d_blocks.upload(blocks.data(), blocks.size(), stream);
    d_ao.alloc((size_t)off);
    launch_ao((int)blocks.size(), d_blocks.p, d_shell_lists.p, dev_shells(), d_x.p, d_y.p, d_z.p, ncomp, d_ao.p, stream);
    ao_order = order;
    ao_ff_order = -1;  // the float-float copy is stale
    CGB_CUDA(cudaStreamSynchronize(stream));
}

void Grid::ensure_work() {
    const int nsig = nspin == 1 ? 1 : 3;
    d_rho.alloc(nspin * Gp);
    d_rho1.alloc(3 * nspin * Gp);
    d_tau.alloc(nspin * Gp);
    d_sigma.alloc(nsig * Gp);
    d_eps.alloc(Gp);
    d_vrho.alloc(nspin * Gp);
    d_vsigma.alloc(nsig * Gp);
    d_vtau.alloc(nspin * Gp);
    d_fcoef.alloc(5 * nspin * Gp);
    d_partial.alloc((Gp + 127) / 128 + 1);
    d_scalar.alloc(2);
    d_D.alloc(packed_size());
    d_V.alloc(packed_size());
}

void Grid::mark(int i) {
    if (profiling) CGB_CUDA(cudaEventRecord(ev[i], stream));
}

Grid::~Grid() {
    for (auto& e : ev)
        if (e) cudaEventDestroy(e);
    mx.drop_graph();
    if (capture_stream) cudaStreamDestroy(capture_stream);
}

void Grid::density_device(const double* dD, bool float_float) {
    NvtxRange nvtx_("xc.getDensity");
    CGB_CHECK(!batched, XC_ERR_UNSUPPORTED, "batch grids run mixed-precision builds only");
    CGB_CHECK(ao_order >= type, XC_ERR_STATE, "getAO must run (for the current type) before getDensity");
    ensure_work();
    mark(0);
    if (float_float) {
        if (ao_ff_order != ao_order) {  // split the AO store once per getAO
            d_ao_ff.alloc(d_ao.n);
            launch_split_ff((long)d_ao.n, d_ao.p, d_ao_ff.p, stream);
            ao_ff_order = ao_order;
        }
        const size_t nn = (size_t)nspin * basis.nbasis * basis.nbasis;
        d_D_ff.alloc(nn);
        launch_split_ff((long)nn, dD, d_D_ff.p, stream);
        launch_density_ff((int)blocks.size(), d_blocks.p, d_lists.p, basis.nbasis, nspin, type, d_D_ff.p, d_ao_ff.p,
                          Gp, d_rho.p, d_rho1.p, d_tau.p, stream);
    } else {
        launch_density_fp64((int)blocks.size(), d_blocks.p, d_lists.p, basis.nbasis, nspin, type, dD, d_ao.p, Gp,
                            d_rho.p, d_rho1.p, d_tau.p, stream);
    }
    have_density = true;
    have_potential = false;
    have_fxc = false;
    rt_ready = false;
}

void Grid::evaluate_fxc(const Functional& f) {
    NvtxRange nvtx_("xc.Evaluate.f");
    CGB_CHECK(have_density, XC_ERR_STATE, "Evaluate needs a density (getDensity first)");
    CGB_CHECK(f.nspin == nspin, XC_ERR_ARG, "functional and grid disagree on the number of spins");
    CGB_CHECK(f.family <= 1, XC_ERR_UNSUPPORTED,
              "second derivatives cover LDA and GGA functionals (as the reference's Evaluate(\"f\"))");
    CGB_CHECK(f.family <= type, XC_ERR_STATE, "grid type is below the functional family (setType/getAO)");
    d_f2.alloc((size_t)(nspin == 1 ? 3 : 15) * Gp);
    launch_fxc(f.desc, f.family, nspin, Gp, d_rho.p, d_rho1.p, d_f2.p, stream);
    fxc_family = f.family;
    have_fxc = true;
    rt_ready = false;
}

void Grid::density_u_device(const double* dDU, int nmat) {
    NvtxRange nvtx_("xc.getDensityU");
    CGB_CHECK(!batched, XC_ERR_UNSUPPORTED, "response densities are per molecule");
    CGB_CHECK(ao_order >= type, XC_ERR_STATE, "getAO must run (for the current type) before getDensityU");
    CGB_CHECK(nmat >= 1, XC_ERR_ARG, "at least one response matrix");
    const int n = basis.nbasis;
    const long q = (long)nspin * nmat;
    CGB_CHECK(q <= 65535, XC_ERR_ARG, "at most 65535 (spin, matrix) pairs per call");
    d_DU.alloc((size_t)q * n * n);
    if (resp_precision == XC_PRECISION_MIXED) {
        // the tensor-core path forms each matrix's response density inside getFockU
        // (from the symmetric part of D_U); keep the matrices
        CGB_CUDA(cudaMemcpyAsync(d_DU.p, dDU, (size_t)q * n * n * sizeof(double), cudaMemcpyDeviceToDevice, stream));
        nmat_u = nmat;
        have_density_u = true;
        return;
    }
    d_rhoU.alloc((size_t)q * Gp);
    d_rho1U.alloc((size_t)q * 3 * Gp);
    // the plain density kernel forms 2 sum D(mu, nu) phi_mu grad phi_nu; the transpose gives the
    // reference's 2 sum D(mu, nu) grad phi_mu phi_nu (GridDensity.cpp:67-68) for any D_U
    launch_transpose_batch(n, q, dDU, d_DU.p, stream);
    // (spin, matrix) pairs run as the kernel's spin index; gradients only up to GGA
    launch_density_fp64((int)blocks.size(), d_blocks.p, d_lists.p, n, (int)q, type >= 1 ? 1 : 0, d_DU.p, d_ao.p,
                        Gp, d_rhoU.p, d_rho1U.p, nullptr, stream);
    nmat_u = nmat;
    have_density_u = true;
}

void Grid::fock_u_device(double* dFU) {
    NvtxRange nvtx_("xc.getFockU");
    CGB_CHECK(have_fxc, XC_ERR_STATE, "getFockU needs Evaluate(\"f\") on the current density");
    CGB_CHECK(have_density_u, XC_ERR_STATE, "getFockU needs getDensityU first");
    CGB_CHECK(fxc_family == 0 || (have_potential && eval_family >= 1), XC_ERR_STATE,
              "getFockU of a GGA needs vsigma: Evaluate(\"v\" or \"ev\") on the current density");
    const int n = basis.nbasis;
    const long q = (long)nspin * nmat_u;
    if (resp_precision == XC_PRECISION_MIXED) {
        if (!rt_ready) {
            response_tiles_prepare();
            rt_ready = true;
        }
        response_mixed(d_DU.p, nmat_u, dFU);
        return;
    }
    d_fcoefU.alloc((size_t)q * 5 * Gp);
    launch_response_coef(fxc_family, nspin, Gp, nmat_u, d_w.p, d_rho1.p, d_vsigma.p, d_f2.p, d_rhoU.p, d_rho1U.p,
                         d_fcoefU.p, stream);
    CGB_CUDA(cudaMemsetAsync(dFU, 0, (size_t)q * n * n * sizeof(double), stream));
    launch_fock_fp64((int)blocks.size(), d_blocks.p, d_lists.p, max_nb, n, (int)q, fxc_family, d_ao.p, Gp,
                     d_fcoefU.p, dFU, stream);
}

void Grid::evaluate(const Functional& f, double float_above) {
    NvtxRange nvtx_("xc.Evaluate");
    CGB_CHECK(have_density, XC_ERR_STATE, "Evaluate needs a density (getDensity first)");
    CGB_CHECK(f.nspin == nspin, XC_ERR_ARG, "functional and grid disagree on the number of spins");
    CGB_CHECK(f.family <= type, XC_ERR_STATE, "grid type is below the functional family (setType/getAO)");
    mark(1);
    launch_functional_fp64(f.desc, f.family, nspin, Gp, d_w.p, d_rho.p, d_rho1.p, d_tau.p, d_sigma.p, d_eps.p,
                           d_vrho.p, d_vsigma.p, d_vtau.p, d_fcoef.p, d_partial.p, &n_partial, stream, float_above);
    eval_family = f.family;
    have_potential = true;
}

void Grid::energy_device(double* dE) {
    CGB_CHECK(have_potential, XC_ERR_STATE, "getEnergy needs Evaluate first");
    mark(2);
    launch_reduce_sum(d_partial.p, n_partial, dE, stream);
}

void Grid::fock_device(double* dV, int fam) {
    NvtxRange nvtx_("xc.getFock");
    const size_t nn = (size_t)basis.nbasis * basis.nbasis * nspin;
    mark(3);
    CGB_CUDA(cudaMemsetAsync(dV, 0, nn * sizeof(double), stream));
    launch_fock_fp64((int)blocks.size(), d_blocks.p, d_lists.p, max_nb, basis.nbasis, nspin, fam, d_ao.p, Gp,
                     d_fcoef.p, dV, stream);
    mark(4);
}

// ------------------------------------------------------------ functional
static std::vector<int> functional_ids_by_name(const std::string& name) {
    std::ifstream f(data_path() + "/functionals.txt");
    if (!f.good()) throw Error(XC_ERR_IO, "Density functional file is missing!");
    std::string line;
    while (std::getline(f, line)) {
        if (line.empty() || line[0] == '#') continue;
        std::stringstream ss(line);
        std::string nm;
        ss >> nm;
        if (nm != name) continue;
        std::vector<int> ids;
        int id;
        while (ss >> id) ids.push_back(id);
        return ids;
    }
    throw Error(XC_ERR_IO, "Density functional file is missing! (" + name + ")");
}

void Functional::init(const std::vector<int>& ids_, int ns) {
    CGB_CHECK(ns == 1 || ns == 2, XC_ERR_ARG, "nspin must be 1 or 2");
    CGB_CHECK(!ids_.empty() && ids_.size() <= 4, XC_ERR_ARG, "between 1 and 4 functional ids");
    ids = ids_;
    nspin = ns;
    family = 0;
    exx = 0;
    desc.nids = (int)ids.size();
    for (size_t i = 0; i < ids.size(); i++) {
        const int fam = xcf::family_of_id(ids[i]);
        CGB_CHECK(fam >= 0, XC_ERR_UNSUPPORTED, "functional id " + std::to_string(ids[i]) + " is not implemented");
        family = std::max(family, fam);
        exx = std::max(exx, xcf::exx_of_id(ids[i]));  // ExchangeCorrelation.cpp:63-64
        desc.ids[i] = ids[i];
    }
}

}  // namespace cgb

using namespace cgb;

// ================================================================== C ABI
extern "C" {

int xc_last_error(char* buf, size_t len) {
    if (!buf || len == 0) return XC_ERR_ARG;
    std::strncpy(buf, g_last_error.c_str(), len - 1);
    buf[len - 1] = 0;
    return XC_OK;
}

int xc_set_data_path(const char* path) {
    return guard([&] {
        CGB_CHECK(path, XC_ERR_ARG, "null path");
        set_data_path(path);
    });
}

int xc_basis_create(int natoms, const int* Z, const double* xyz, const char* name, xc_basis** out) {
    return guard([&] {
        CGB_CHECK(natoms > 0 && Z && xyz && name && out, XC_ERR_ARG, "bad basis arguments");
        std::vector<int> z(Z, Z + natoms);
        std::vector<double> c(xyz, xyz + 3 * natoms);
        for (double v : c) CGB_CHECK(std::isfinite(v), XC_ERR_NUMERIC, "non-finite coordinate");
        auto* b = new xc_basis;
        try {
            b->b = load_basis(name, z, c);
        } catch (...) {
            delete b;
            throw;
        }
        *out = b;
    });
}

int xc_basis_create_shells(int natoms, const int* Z, const double* xyz, int nshells, const int* shell_atom,
                           const int* shell_type, const int* nprim, const double* exps, const double* coefs,
                           int normalize, xc_basis** out) {
    return guard([&] {
        CGB_CHECK(natoms > 0 && Z && xyz && nshells > 0 && shell_atom && shell_type && nprim && exps && coefs && out,
                  XC_ERR_ARG, "bad basis arguments");
        CGB_CHECK(normalize == 0 || normalize == 1, XC_ERR_ARG, "normalize must be 0 or 1");
        BasisSet b;
        b.Z.assign(Z, Z + natoms);
        b.xyz.assign(xyz, xyz + 3 * natoms);
        for (double v : b.xyz) CGB_CHECK(std::isfinite(v), XC_ERR_NUMERIC, "non-finite coordinate");
        int first = 0;
        long po = 0;
        for (int i = 0; i < nshells; i++) {
            const int a = shell_atom[i], t = shell_type[i], np = nprim[i];
            CGB_CHECK(a >= 0 && a < natoms, XC_ERR_ARG, "shell atom index out of range");
            CGB_CHECK(np > 0, XC_ERR_ARG, "shell without primitives");
            // Mwfn shell types the reference's AO code evaluates (GridAO.cpp:153-178):
            // 0 s, 1 Cartesian p (x, y, z), -l pure l >= 1 (m = -l..l; pure p is y, z, x)
            CGB_CHECK(t == 0 || t == 1 || (t < 0 && -t <= kMaxL), XC_ERR_UNSUPPORTED,
                      "shell type " + std::to_string(t) + " is not supported (0, 1 or -1..-" +
                          std::to_string(kMaxL) + ")");
            Shell s{};
            s.atom = a;
            s.l = t < 0 ? -t : t;
            s.type = t;
            s.first = first;
            s.nprim = np;
            s.prim_off = (int)po;
            s.x = xyz[3 * a];
            s.y = xyz[3 * a + 1];
            s.z = xyz[3 * a + 2];
            std::vector<double> e(exps + po, exps + po + np), c(coefs + po, coefs + po + np);
            for (int p = 0; p < np; p++)
                CGB_CHECK(std::isfinite(e[p]) && e[p] > 0 && std::isfinite(c[p]), XC_ERR_NUMERIC,
                          "exponents must be positive and finite, coefficients finite");
            if (normalize) c = renorm_contraction(s.l, e, c);
            b.exps.insert(b.exps.end(), e.begin(), e.end());
            b.coefs.insert(b.coefs.end(), c.begin(), c.end());
            first += shell_size(t);
            po += np;
            b.shells.push_back(s);
        }
        b.nbasis = first;
        auto* h = new xc_basis;
        h->b = std::move(b);
        *out = h;
    });
}

int xc_basis_nbasis(const xc_basis* b, int* n) {
    return guard([&] {
        CGB_CHECK(b && n, XC_ERR_ARG, "null argument");
        *n = b->b.nbasis;
    });
}

int xc_basis_nshells(const xc_basis* b, int* n) {
    return guard([&] {
        CGB_CHECK(b && n, XC_ERR_ARG, "null argument");
        *n = (int)b->b.shells.size();
    });
}

int xc_basis_shells(const xc_basis* b, int* atom, int* type, int* first, int* nprim) {
    return guard([&] {
        CGB_CHECK(b, XC_ERR_ARG, "null basis");
        for (size_t i = 0; i < b->b.shells.size(); i++) {
            const Shell& s = b->b.shells[i];
            if (atom) atom[i] = s.atom;
            if (type) type[i] = s.type;
            if (first) first[i] = s.first;
            if (nprim) nprim[i] = s.nprim;
        }
    });
}

int xc_basis_primitives(const xc_basis* b, double* exps, double* coefs) {
    return guard([&] {
        CGB_CHECK(b, XC_ERR_ARG, "null basis");
        if (exps) std::memcpy(exps, b->b.exps.data(), b->b.exps.size() * sizeof(double));
        if (coefs) std::memcpy(coefs, b->b.coefs.data(), b->b.coefs.size() * sizeof(double));
    });
}

int xc_basis_destroy(xc_basis* b) {
    delete b;
    return XC_OK;
}

int xc_grid_create(const xc_basis* b, const char* grid_name, int nspin, double thr, xc_grid** out) {
    return guard([&] {
        CGB_CHECK(b && grid_name && out, XC_ERR_ARG, "bad grid arguments");
        CGB_CHECK(nspin == 1 || nspin == 2, XC_ERR_ARG, "nspin must be 1 or 2");
        CGB_CHECK(thr >= 0 && std::isfinite(thr), XC_ERR_ARG, "screen threshold must be >= 0");
        auto* g = new xc_grid;
        try {
            g->g.build(b->b, grid_name, nspin, thr);
        } catch (...) {
            delete g;
            throw;
        }
        *out = g;
    });
}

int xc_grid_destroy(xc_grid* g) {
    delete g;
    return XC_OK;
}

int xc_grid_set_stream(xc_grid* g, void* stream) {
    return guard([&] {
        CGB_CHECK(g, XC_ERR_ARG, "null grid");
        g->g.stream = (cudaStream_t)stream;
    });
}

int xc_grid_set_type(xc_grid* g, int type) {
    return guard([&] {
        CGB_CHECK(g, XC_ERR_ARG, "null grid");
        CGB_CHECK(type >= 0 && type <= 2, XC_ERR_ARG, "type must be 0, 1 or 2");
        g->g.type = type;
    });
}

int xc_grid_get_ao(xc_grid* g, int derivative) {
    return guard([&] {
        CGB_CHECK(g, XC_ERR_ARG, "null grid");
        g->g.get_ao(derivative);
    });
}

int xc_grid_num_electrons(xc_grid* g, double* n) {
    return guard([&] {
        CGB_CHECK(g && n, XC_ERR_ARG, "null argument");
        Grid& G = g->g;
        CGB_CHECK(G.have_density, XC_ERR_STATE, "getNumElectrons needs a density");
        int np = 0;
        launch_num_electrons(G.Gp, G.nspin, G.d_w.p, G.d_rho.p, G.d_partial.p, &np, G.stream);
        launch_reduce_sum(G.d_partial.p, np, G.d_scalar.p + 1, G.stream);
        CGB_CUDA(cudaMemcpyAsync(n, G.d_scalar.p + 1, sizeof(double), cudaMemcpyDeviceToHost, G.stream));
        CGB_CUDA(cudaStreamSynchronize(G.stream));
        G.have_potential = false;  // partials reused
    });
}

int xc_grid_get_density(xc_grid* g, const double* D, int nspin) {
    return guard([&] {
        CGB_CHECK(g && D, XC_ERR_ARG, "null argument");
        Grid& G = g->g;
        CGB_CHECK(nspin == G.nspin, XC_ERR_ARG, "Wrong number of spin types!");
        G.ensure_work();
        const size_t nn = (size_t)G.basis.nbasis * G.basis.nbasis * nspin;
        CGB_CUDA(cudaMemcpyAsync(G.d_D.p, D, nn * sizeof(double), cudaMemcpyHostToDevice, G.stream));
        G.density_device(G.d_D.p);
        CGB_CUDA(cudaStreamSynchronize(G.stream));
    });
}

int xc_grid_get_energy(xc_grid* g, double* E) {
    return guard([&] {
        CGB_CHECK(g && E, XC_ERR_ARG, "null argument");
        Grid& G = g->g;
        G.energy_device(G.d_scalar.p);
        CGB_CUDA(cudaMemcpyAsync(E, G.d_scalar.p, sizeof(double), cudaMemcpyDeviceToHost, G.stream));
        CGB_CUDA(cudaStreamSynchronize(G.stream));
    });
}

int xc_grid_get_fock(xc_grid* g, double* V) {
    return guard([&] {
        CGB_CHECK(g && V, XC_ERR_ARG, "null argument");
        Grid& G = g->g;
        CGB_CHECK(G.have_potential, XC_ERR_STATE, "getFock needs Evaluate first");
        G.fock_device(G.d_V.p, G.eval_family);
        const size_t nn = (size_t)G.basis.nbasis * G.basis.nbasis * G.nspin;
        CGB_CUDA(cudaMemcpyAsync(V, G.d_V.p, nn * sizeof(double), cudaMemcpyDeviceToHost, G.stream));
        CGB_CUDA(cudaStreamSynchronize(G.stream));
    });
}

int xc_grid_info_get(const xc_grid* g, xc_grid_info* info) {
    return guard([&] {
        CGB_CHECK(g && info, XC_ERR_ARG, "null argument");
        const Grid& G = g->g;
        info->npoints = G.npoints;
        info->npoints_padded = G.Gp;
        info->nblocks = (int)G.blocks.size();
        info->nbasis = G.basis.nbasis;
        info->nspin = G.nspin;
        info->type = G.type;
        info->ao_elements = G.ao_elements;
        info->screened_pairs = G.screened_pairs;
        info->mixed_tiles = G.mx.ready ? G.mx.md.ntiles : 0;
        info->mixed_pairs = G.mx.ready ? G.mx.kept_pairs : 0;
        info->mixed_rows = G.mx.ready ? G.mx.md.rows : 0;
        info->mixed_store_bytes = G.mx.ready ? (long)(G.mx.d_e32.n + G.mx.d_Z.n) * 4 : 0;
        // split_d, density passes, combine, functional, energy, then per spin Z / V partials / reduction
        info->mixed_launches = 1 + G.nspin * (G.type >= 2 ? 4 : 1) + 3 + 3 * G.nspin;
        info->mixed_units_full = G.mx.ready ? G.mx.units_full : 0;
        info->mixed_units_sym = G.mx.ready ? G.mx.units_sym : 0;
        info->mixed_fock_jobs = G.mx.ready ? G.mx.fock_jobs : 0;
        info->mixed_fock_tau_jobs = G.mx.ready ? G.mx.fock_tau_jobs : 0;
        info->mixed_fock_items = G.mx.ready ? G.mx.live_items : 0;
        info->mixed_empty_tiles = G.mx.ready ? G.mx.empty_tiles : 0;
        info->mixed_presplit = G.mx.ready && G.mx.use16 ? 1 : 0;
        info->mixed_presplit_bytes =
            info->mixed_presplit ? (long)((G.mx.d_e16.n + G.mx.d_e16d.n + G.mx.d_R16.n) * sizeof(__nv_bfloat16)) : 0;
    });
}

int xc_grid_points(const xc_grid* g, double* x, double* y, double* z, double* w, int* off, int* ng, int* nreal,
                   int* nb) {
    return guard([&] {
        CGB_CHECK(g, XC_ERR_ARG, "null grid");
        const Grid& G = g->g;
        if (x) std::memcpy(x, G.hx.data(), G.Gp * sizeof(double));
        if (y) std::memcpy(y, G.hy.data(), G.Gp * sizeof(double));
        if (z) std::memcpy(z, G.hz.data(), G.Gp * sizeof(double));
        if (w) {
            CGB_CUDA(cudaMemcpyAsync(w, G.d_w.p, G.Gp * sizeof(double), cudaMemcpyDeviceToHost, G.stream));
            CGB_CUDA(cudaStreamSynchronize(G.stream));
        }
        for (size_t b = 0; b < G.blocks.size(); b++) {
            if (off) off[b] = G.blocks[b].pt_off;
            if (ng) ng[b] = G.blocks[b].ng;
            if (nreal) nreal[b] = G.blocks[b].nreal;
            if (nb) nb[b] = G.blocks[b].nb;
        }
    });
}

static void d2h(void* dst, const void* src, size_t bytes, cudaStream_t s) {
    if (dst && src && bytes) CGB_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s));
}

int xc_grid_density_values(const xc_grid* g, double* rho, double* rho1, double* sigma, double* tau) {
    return guard([&] {
        CGB_CHECK(g, XC_ERR_ARG, "null grid");
        const Grid& G = g->g;
        CGB_CHECK(G.have_density, XC_ERR_STATE, "no density");
        const size_t B = sizeof(double) * G.Gp;
        d2h(rho, G.d_rho.p, B * G.nspin, G.stream);
        if (G.type >= 1) d2h(rho1, G.d_rho1.p, B * 3 * G.nspin, G.stream);
        if (G.type >= 1 && G.have_potential) d2h(sigma, G.d_sigma.p, B * (G.nspin == 1 ? 1 : 3), G.stream);
        if (G.type >= 2) d2h(tau, G.d_tau.p, B * G.nspin, G.stream);
        CGB_CUDA(cudaStreamSynchronize(G.stream));
    });
}

int xc_grid_potential_values(const xc_grid* g, double* eps, double* vrho, double* vsigma, double* vtau) {
    return guard([&] {
        CGB_CHECK(g, XC_ERR_ARG, "null grid");
        const Grid& G = g->g;
        CGB_CHECK(G.have_potential, XC_ERR_STATE, "no potential (Evaluate first)");
        const size_t B = sizeof(double) * G.Gp;
        d2h(eps, G.d_eps.p, B, G.stream);
        d2h(vrho, G.d_vrho.p, B * G.nspin, G.stream);
        if (G.eval_family >= 1) d2h(vsigma, G.d_vsigma.p, B * (G.nspin == 1 ? 1 : 3), G.stream);
        if (G.eval_family >= 2) d2h(vtau, G.d_vtau.p, B * G.nspin, G.stream);
        CGB_CUDA(cudaStreamSynchronize(G.stream));
    });
}

int xc_grid_block_ao(const xc_grid* g, int block, double* ao, double* ao1, int* list) {
    return guard([&] {
        CGB_CHECK(g, XC_ERR_ARG, "null grid");
        const Grid& G = g->g;
        CGB_CHECK(block >= 0 && block < (int)G.blocks.size(), XC_ERR_ARG, "block index out of range");
        CGB_CHECK(G.ao_order >= 0, XC_ERR_STATE, "getAO first");
        const BlockDesc& bd = G.blocks[block];
        const size_t cs = (size_t)bd.nb * bd.ng;
        d2h(ao, G.d_ao.p + bd.ao_off, cs * sizeof(double), G.stream);
        if (G.ncomp == 4) d2h(ao1, G.d_ao.p + bd.ao_off + cs, 3 * cs * sizeof(double), G.stream);
        if (list) std::memcpy(list, G.basis_lists.data() + bd.bas_off, bd.nb * sizeof(int));
        CGB_CUDA(cudaStreamSynchronize(G.stream));
    });
}

int xc_functional_read(const char* name, int nspin, xc_functional** out) {
    return guard([&] {
        CGB_CHECK(name && out, XC_ERR_ARG, "null argument");
        auto ids = functional_ids_by_name(name);
        auto* f = new xc_functional;
        try {
            f->f.init(ids, nspin);
        } catch (...) {
            delete f;
            throw;
        }
        *out = f;
    });
}

int xc_functional_create(const int* ids, int nids, int nspin, xc_functional** out) {
    return guard([&] {
        CGB_CHECK(ids && nids > 0 && out, XC_ERR_ARG, "bad functional arguments");
        auto* f = new xc_functional;
        try {
            f->f.init(std::vector<int>(ids, ids + nids), nspin);
        } catch (...) {
            delete f;
            throw;
        }
        *out = f;
    });
}

int xc_functional_destroy(xc_functional* f) {
    delete f;
    return XC_OK;
}

int xc_functional_exx(const xc_functional* f, double* exx) {
    return guard([&] {
        CGB_CHECK(f && exx, XC_ERR_ARG, "null argument");
        *exx = f->f.exx;
    });
}

int xc_functional_family(const xc_functional* f, int* fam) {
    return guard([&] {
        CGB_CHECK(f && fam, XC_ERR_ARG, "null argument");
        *fam = f->f.family;
    });
}

int xc_evaluate(xc_functional* f, xc_grid* g, const char* order) {
    return guard([&] {
        CGB_CHECK(f && g && order, XC_ERR_ARG, "null argument");
        const std::string o = order;
        CGB_CHECK(o == "e" || o == "v" || o == "ev" || o == "f", XC_ERR_UNSUPPORTED, "order must be e, v, ev or f");
        if (o == "f") g->g.evaluate_fxc(f->f);
        else g->g.evaluate(f->f);
        CGB_CUDA(cudaStreamSynchronize(g->g.stream));
    });
}

int xc_functional_fxc_points(xc_functional* f, long n, const double* rho, const double* sigma, double* v2rho2,
                             double* v2rhosigma, double* v2sigma2) {
    return guard([&] {
        CGB_CHECK(f && rho && v2rho2 && n > 0, XC_ERR_ARG, "bad arguments");
        const Functional& F = f->f;
        CGB_CHECK(F.family <= 1, XC_ERR_UNSUPPORTED,
                  "second derivatives cover LDA and GGA functionals (as the reference's Evaluate(\"f\"))");
        CGB_CHECK(F.family < 1 || (sigma && v2rhosigma && v2sigma2), XC_ERR_ARG, "sigma arrays required for GGA");
        ensure_device();
        const int ns = F.nspin, nsig = ns == 1 ? 1 : 3, nrr = ns == 1 ? 1 : 3, nrs = ns == 1 ? 1 : 6;
        DevBuf<double> dr, ds, d1, d2, d3;
        dr.upload(rho, ns * n);
        ds.alloc(nsig * n);
        if (F.family >= 1) ds.upload(sigma, nsig * n);
        d1.alloc(nrr * n);
        d2.alloc(nrs * n);
        d3.alloc(nrs * n);
        launch_fxc_points(F.desc, F.family, ns, n, dr.p, ds.p, d1.p, d2.p, d3.p, 0);
        CGB_CUDA(cudaMemcpy(v2rho2, d1.p, nrr * n * sizeof(double), cudaMemcpyDeviceToHost));
        if (F.family >= 1) {
            CGB_CUDA(cudaMemcpy(v2rhosigma, d2.p, nrs * n * sizeof(double), cudaMemcpyDeviceToHost));
            CGB_CUDA(cudaMemcpy(v2sigma2, d3.p, nrs * n * sizeof(double), cudaMemcpyDeviceToHost));
        }
    });
}

int xc_grid_get_density_u(xc_grid* g, const double* DU, int nspin, int nmat) {
    return guard([&] {
        CGB_CHECK(g && DU, XC_ERR_ARG, "null argument");
        Grid& G = g->g;
        CGB_CHECK(nspin == G.nspin, XC_ERR_ARG, "Wrong number of spin types!");
        CGB_CHECK(nmat >= 1, XC_ERR_ARG, "at least one response matrix");
        const size_t cnt = (size_t)nspin * nmat * G.basis.nbasis * G.basis.nbasis;
        DevBuf<double> dU;
        dU.upload(DU, cnt);
        G.density_u_device(dU.p, nmat);
        CGB_CUDA(cudaStreamSynchronize(G.stream));
    });
}

int xc_grid_get_fock_u(xc_grid* g, double* FU) {
    return guard([&] {
        CGB_CHECK(g && FU, XC_ERR_ARG, "null argument");
        Grid& G = g->g;
        const size_t cnt = (size_t)G.nspin * G.nmat_u * G.basis.nbasis * G.basis.nbasis;
        DevBuf<double> dF;
        dF.alloc(cnt);
        G.fock_u_device(dF.p);
        CGB_CUDA(cudaMemcpyAsync(FU, dF.p, cnt * sizeof(double), cudaMemcpyDeviceToHost, G.stream));
        CGB_CUDA(cudaStreamSynchronize(G.stream));
        if (G.resp_precision == XC_PRECISION_MIXED && G.mixed_error())
            throw Error(XC_ERR_TIMEOUT, "a bounded wait of the tensor-core pipeline gave up");
    });
}

int xc_grid_set_response_precision(xc_grid* g, int precision) {
    return guard([&] {
        CGB_CHECK(g, XC_ERR_ARG, "null grid");
        CGB_CHECK(precision == XC_PRECISION_FP64 || precision == XC_PRECISION_MIXED, XC_ERR_ARG, "bad precision");
        CGB_CHECK(!g->g.batched, XC_ERR_UNSUPPORTED, "response builds are per molecule");
        if (g->g.resp_precision != precision) g->g.have_density_u = false;
        g->g.resp_precision = precision;
    });
}

int xc_build_response(xc_grid* g, xc_functional* f, const double* D, int nspin, int precision, int nmat,
                      const double* DU, double* FU) {
    return guard([&] {
        CGB_CHECK(g && f && D && DU && FU, XC_ERR_ARG, "null argument");
        Grid& G = g->g;
        CGB_CHECK(!G.batched, XC_ERR_UNSUPPORTED, "response builds are per molecule");
        CGB_CHECK(nspin == G.nspin && f->f.nspin == G.nspin, XC_ERR_ARG, "Wrong number of spin types!");
        CGB_CHECK(precision == XC_PRECISION_FP64 || precision == XC_PRECISION_MIXED, XC_ERR_ARG, "bad precision");
        CGB_CHECK(nmat >= 1, XC_ERR_ARG, "at least one response matrix");
        CGB_CHECK(f->f.family <= 1, XC_ERR_UNSUPPORTED,
                  "response V_xc covers LDA and GGA functionals (as the reference's Evaluate(\"f\"))");
        G.ensure_work();
        const bool mixed = precision == XC_PRECISION_MIXED;
        const int n = G.basis.nbasis;
        const size_t nn = (size_t)n * n;
        CGB_CUDA(cudaMemcpyAsync(G.d_D.p, D, nn * nspin * sizeof(double), cudaMemcpyHostToDevice, G.stream));
        G.density_device(G.d_D.p);
        G.evaluate(f->f);
        G.evaluate_fxc(f->f);
        const int saved = G.resp_precision;
        G.resp_precision = precision;
        struct Restore {
            Grid& g;
            int p;
            ~Restore() { g.resp_precision = p; }
        } restore{G, saved};
        // matrices in chunks that keep the device scratch near 2 GB: per matrix the FP64 path
        // holds rho_U, grad rho_U and 5 coefficient rows per point, both paths D_U and V_U
        const long per_mat = (long)sizeof(double) * nspin * ((mixed ? 0L : 9L * G.Gp) + 2L * (long)nn);
        const int chunk = (int)std::max(1L, std::min<long>(nmat, (2L << 30) / std::max(per_mat, 1L)));
        DevBuf<double> dU, dF;
        dU.alloc((size_t)nspin * chunk * nn);
        dF.alloc((size_t)nspin * chunk * nn);
        for (int m0 = 0; m0 < nmat; m0 += chunk) {
            const int mc = std::min(chunk, nmat - m0);
            // D_U[s][m0 .. m0 + mc) -> device [s][0 .. mc): one contiguous copy per spin
            for (int s = 0; s < nspin; s++)
                CGB_CUDA(cudaMemcpyAsync(dU.p + (size_t)s * mc * nn, DU + ((size_t)s * nmat + m0) * nn,
                                         (size_t)mc * nn * sizeof(double), cudaMemcpyHostToDevice, G.stream));
            G.density_u_device(dU.p, mc);
            G.fock_u_device(dF.p);
            for (int s = 0; s < nspin; s++)
                CGB_CUDA(cudaMemcpyAsync(FU + ((size_t)s * nmat + m0) * nn, dF.p + (size_t)s * mc * nn,
                                         (size_t)mc * nn * sizeof(double), cudaMemcpyDeviceToHost, G.stream));
            CGB_CUDA(cudaStreamSynchronize(G.stream));
        }
        if (mixed && G.mixed_error())
            throw Error(XC_ERR_TIMEOUT, "a bounded wait of the tensor-core pipeline gave up");
    });
}

int xc_functional_eval_points(xc_functional* f, long n, const double* rho, const double* sigma, const double* tau,
                              double* eps, double* vrho, double* vsigma, double* vtau) {
    return guard([&] {
        CGB_CHECK(f && rho && eps && vrho && n > 0, XC_ERR_ARG, "bad arguments");
        ensure_device();
        const Functional& F = f->f;
        const int ns = F.nspin, nsig = ns == 1 ? 1 : 3;
        CGB_CHECK(F.family < 1 || (sigma && vsigma), XC_ERR_ARG, "sigma arrays required for GGA");
        CGB_CHECK(F.family < 2 || (tau && vtau), XC_ERR_ARG, "tau arrays required for meta-GGA");
        DevBuf<double> dr, ds, dt, de, dvr, dvs, dvt;
        dr.upload(rho, ns * n);
        ds.alloc(nsig * n);
        dt.alloc(ns * n);
        if (F.family >= 1) ds.upload(sigma, nsig * n);
        if (F.family >= 2) dt.upload(tau, ns * n);
        de.alloc(n);
        dvr.alloc(ns * n);
        dvs.alloc(nsig * n);
        dvt.alloc(ns * n);
        launch_functional_points(F.desc, F.family, ns, n, dr.p, ds.p, dt.p, de.p, dvr.p, dvs.p, dvt.p, 0);
        CGB_CUDA(cudaMemcpy(eps, de.p, n * sizeof(double), cudaMemcpyDeviceToHost));
        CGB_CUDA(cudaMemcpy(vrho, dvr.p, ns * n * sizeof(double), cudaMemcpyDeviceToHost));
        if (F.family >= 1) CGB_CUDA(cudaMemcpy(vsigma, dvs.p, nsig * n * sizeof(double), cudaMemcpyDeviceToHost));
        if (F.family >= 2) CGB_CUDA(cudaMemcpy(vtau, dvt.p, ns * n * sizeof(double), cudaMemcpyDeviceToHost));
    });
}

static void check_build(Grid& G, const xc_functional* f, int nspin, int precision) {
    CGB_CHECK(nspin == G.nspin, XC_ERR_ARG, "Wrong number of spin types!");
    CGB_CHECK(precision == XC_PRECISION_FP64 || precision == XC_PRECISION_MIXED, XC_ERR_ARG, "bad precision");
    CGB_CHECK(f->f.nspin == G.nspin, XC_ERR_ARG, "functional and grid disagree on the number of spins");
    CGB_CHECK(f->f.family <= G.type, XC_ERR_STATE, "grid type is below the functional family (setType/getAO)");
    CGB_CHECK(precision == XC_PRECISION_MIXED || !G.batched, XC_ERR_UNSUPPORTED,
              "batch grids run mixed-precision builds only");
}

static int num_mols(const Grid& G) { return G.batched ? (int)G.mol_n.size() : 1; }

int xc_build_device(xc_grid* g, xc_functional* f, const double* dD, int nspin, int precision, double* dE, double* dV) {
    return guard([&] {
        CGB_CHECK(g && f && dD && dE && dV, XC_ERR_ARG, "null argument");
        Grid& G = g->g;
        check_build(G, f, nspin, precision);
        if (precision == XC_PRECISION_MIXED) {
            G.ensure_work();
            const size_t nn = (size_t)G.packed_size();
            if (dD != G.d_D.p)
                CGB_CUDA(cudaMemcpyAsync(G.d_D.p, dD, nn * sizeof(double), cudaMemcpyDeviceToDevice, G.stream));
            G.build_mixed_graph(f->f);
            CGB_CUDA(cudaMemcpyAsync(dE, G.d_Emol.p, num_mols(G) * sizeof(double), cudaMemcpyDeviceToDevice,
                                     G.stream));
            if (dV != G.d_V.p)
                CGB_CUDA(cudaMemcpyAsync(dV, G.d_V.p, nn * sizeof(double), cudaMemcpyDeviceToDevice, G.stream));
            return;
        }
        G.density_device(dD);
        G.evaluate(f->f);
        G.energy_device(dE);
        G.fock_device(dV, f->f.family);
    });
}

int xc_grid_energy_grad(xc_grid* g, xc_functional* f, const double* D, int nspin, double* grad) {
    return guard([&] {
        CGB_CHECK(g && f && D && grad, XC_ERR_ARG, "null argument");
        Grid& G = g->g;
        CGB_CHECK(!G.batched, XC_ERR_UNSUPPORTED, "gradients are per molecule");
        CGB_CHECK(nspin == G.nspin && f->f.nspin == G.nspin, XC_ERR_ARG, "Wrong number of spin types!");
        CGB_CHECK(f->f.family <= 1, XC_ERR_UNSUPPORTED,
                  "XC gradients cover LDA and GGA functionals (as the reference's getEnergyGrad)");
        CGB_CHECK(f->f.family <= G.type, XC_ERR_STATE, "grid type is below the functional family (setType/getAO)");
        CGB_CHECK(G.ncomp >= (f->f.family >= 1 ? 10 : 4), XC_ERR_STATE,
                  "the gradient needs AO derivatives one order above the functional's (getAO(1))");
        G.ensure_work();
        const int n = G.basis.nbasis;
        const size_t nn = (size_t)n * n * nspin;
        CGB_CUDA(cudaMemcpyAsync(G.d_D.p, D, nn * sizeof(double), cudaMemcpyHostToDevice, G.stream));
        G.density_device(G.d_D.p);
        G.evaluate(f->f);
        const long nlist = (long)G.basis_lists.size();
        DevBuf<double> part;
        part.alloc((size_t)nspin * nlist * 3);
        NvtxRange nvtx_("xc.getEnergyGrad");
        G.mark(2);  // stage timers: ms[2] = the gradient kernel, ms[3] = 0
        launch_xc_grad((int)G.blocks.size(), G.d_blocks.p, G.d_lists.p, nlist, n, nspin, f->f.family, G.d_D.p,
                       G.d_ao.p, G.Gp, G.d_fcoef.p, part.p, G.stream);
        G.mark(3);
        G.mark(4);
        std::vector<double> h((size_t)nspin * nlist * 3);
        CGB_CUDA(cudaMemcpyAsync(h.data(), part.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost, G.stream));
        CGB_CUDA(cudaStreamSynchronize(G.stream));
        // atom of every basis function, then a fixed-order sum over spins, blocks and functions
        std::vector<int> atom_of(n, 0);
        for (const Shell& sh : G.basis.shells)
            for (int k = 0; k < shell_size(sh.type); k++) atom_of[sh.first + k] = sh.atom;
        const int na = G.basis.natoms();
        std::fill(grad, grad + 3 * na, 0.0);
        for (int sp = 0; sp < nspin; sp++)
            for (long e = 0; e < nlist; e++) {
                const int a = atom_of[G.basis_lists[e]];
                for (int t = 0; t < 3; t++) grad[3 * a + t] += h[((size_t)sp * nlist + e) * 3 + t];
            }
        G.have_potential = false;  // the functional ran on this D
    });
}

int xc_grid_fock_skeleton(xc_grid* g, xc_functional* f, const double* D, int nspin, double* FS, double* FU) {
    return guard([&] {
        CGB_CHECK(g && f && D && FS && FU, XC_ERR_ARG, "null argument");
        Grid& G = g->g;
        CGB_CHECK(!G.batched, XC_ERR_UNSUPPORTED, "skeleton terms are per molecule");
        CGB_CHECK(nspin == G.nspin && f->f.nspin == G.nspin, XC_ERR_ARG, "Wrong number of spin types!");
        CGB_CHECK(f->f.family <= 1, XC_ERR_UNSUPPORTED,
                  "skeleton terms cover LDA and GGA functionals (as the reference's Hessian)");
        CGB_CHECK(f->f.family <= G.type, XC_ERR_STATE, "grid type is below the functional family (setType/getAO)");
        CGB_CHECK(G.ncomp >= (f->f.family >= 1 ? 10 : 4), XC_ERR_STATE,
                  "the skeleton terms need AO derivatives one order above the functional's (getAO(1))");
        NvtxRange nvtx_("xc.getFockSkeleton");
        G.ensure_work();
        const int n = G.basis.nbasis, na = G.basis.natoms();
        const int nmat = 3 * na;
        const long q = (long)nspin * nmat;
        CGB_CHECK(q <= 65535, XC_ERR_ARG, "at most 65535 (spin, atom, direction) matrices");
        const size_t nn = (size_t)n * n;
        CGB_CUDA(cudaMemcpyAsync(G.d_D.p, D, nn * nspin * sizeof(double), cudaMemcpyHostToDevice, G.stream));
        G.density_device(G.d_D.p);
        G.evaluate(f->f);
        G.evaluate_fxc(f->f);
        // the atom of every block list entry
        std::vector<int> atom_of(n, 0);
        for (const Shell& sh : G.basis.shells)
            for (int k = 0; k < shell_size(sh.type); k++) atom_of[sh.first + k] = sh.atom;
        std::vector<int> la(G.basis_lists.size());
        for (size_t e = 0; e < la.size(); e++) la[e] = atom_of[G.basis_lists[e]];
        DevBuf<int> d_la;
        d_la.upload(la.data(), la.size());
        DevBuf<double> rg, r1g, fcU, dFS, dFU;
        rg.alloc((size_t)q * G.Gp);
        r1g.alloc((size_t)q * 3 * G.Gp);
        fcU.alloc((size_t)q * 5 * G.Gp);
        dFS.alloc((size_t)q * nn);
        dFU.alloc((size_t)q * nn);
        CGB_CUDA(cudaMemsetAsync(rg.p, 0, (size_t)q * G.Gp * sizeof(double), G.stream));
        CGB_CUDA(cudaMemsetAsync(r1g.p, 0, (size_t)q * 3 * G.Gp * sizeof(double), G.stream));
        CGB_CUDA(cudaMemsetAsync(dFS.p, 0, (size_t)q * nn * sizeof(double), G.stream));
        CGB_CUDA(cudaMemsetAsync(dFU.p, 0, (size_t)q * nn * sizeof(double), G.stream));
        const int fam = f->f.family;
        const int nbk = (int)G.blocks.size();
        // getDensitySkeleton, then getFockU<s_t> (response of V_xc to the skeleton densities)
        launch_skel_density(nbk, G.d_blocks.p, G.d_lists.p, d_la.p, n, nspin, nmat, fam, G.d_D.p, G.d_ao.p, G.Gp,
                            rg.p, r1g.p, G.stream);
        launch_response_coef(fam, nspin, G.Gp, nmat, G.d_w.p, G.d_rho1.p, G.d_vsigma.p, G.d_f2.p, rg.p, r1g.p, fcU.p,
                             G.stream);
        launch_fock_fp64(nbk, G.d_blocks.p, G.d_lists.p, G.max_nb, n, (int)q, fam, G.d_ao.p, G.Gp, fcU.p, dFU.p,
                         G.stream);
        // getFockSkeleton
        launch_fock_skel(nbk, G.d_blocks.p, G.d_lists.p, d_la.p, G.max_nb, n, nspin, nmat, fam, G.d_ao.p, G.Gp,
                         G.d_fcoef.p, dFS.p, G.stream);
        CGB_CUDA(cudaMemcpyAsync(FS, dFS.p, (size_t)q * nn * sizeof(double), cudaMemcpyDeviceToHost, G.stream));
        CGB_CUDA(cudaMemcpyAsync(FU, dFU.p, (size_t)q * nn * sizeof(double), cudaMemcpyDeviceToHost, G.stream));
        CGB_CUDA(cudaStreamSynchronize(G.stream));
        G.have_density_u = false;  // a new ground state: response densities of an earlier getDensityU belong to the old one
    });
}

int xc_build(xc_grid* g, xc_functional* f, const double* D, int nspin, int precision, double* E, double* V) {
    return guard([&] {
        CGB_CHECK(g && f && D && E && V, XC_ERR_ARG, "null argument");
        Grid& G = g->g;
        check_build(G, f, nspin, precision);
        G.ensure_work();
        const size_t nn = (size_t)G.packed_size();
        CGB_CUDA(cudaMemcpyAsync(G.d_D.p, D, nn * sizeof(double), cudaMemcpyHostToDevice, G.stream));
        if (precision == XC_PRECISION_MIXED) {
            G.build_mixed_graph(f->f);
            CGB_CUDA(cudaMemcpyAsync(E, G.d_Emol.p, num_mols(G) * sizeof(double), cudaMemcpyDeviceToHost, G.stream));
        } else {
            G.density_device(G.d_D.p);
            G.evaluate(f->f);
            G.energy_device(G.d_scalar.p);
            G.fock_device(G.d_V.p, f->f.family);
            CGB_CUDA(cudaMemcpyAsync(E, G.d_scalar.p, sizeof(double), cudaMemcpyDeviceToHost, G.stream));
        }
        CGB_CUDA(cudaMemcpyAsync(V, G.d_V.p, nn * sizeof(double), cudaMemcpyDeviceToHost, G.stream));
        CGB_CUDA(cudaStreamSynchronize(G.stream));
        if (precision == XC_PRECISION_MIXED && G.mixed_error())
            throw Error(XC_ERR_TIMEOUT, "a bounded wait of the tensor-core pipeline gave up");
    });
}

int xc_grid_profile(xc_grid* g, int enable) {
    return guard([&] {
        CGB_CHECK(g, XC_ERR_ARG, "null grid");
        Grid& G = g->g;
        if (enable)
            for (auto& e : G.ev)
                if (!e) CGB_CUDA(cudaEventCreate(&e));
        G.profiling = enable != 0;
    });
}

int xc_grid_stage_ms(xc_grid* g, double* ms) {
    return guard([&] {
        CGB_CHECK(g && ms, XC_ERR_ARG, "null argument");
        Grid& G = g->g;
        CGB_CHECK(G.profiling, XC_ERR_STATE, "profiling is off (xc_grid_profile)");
        CGB_CUDA(cudaEventSynchronize(G.ev[4]));
        for (int i = 0; i < 4; i++) {
            float t = 0;
            CGB_CUDA(cudaEventElapsedTime(&t, G.ev[i], G.ev[i + 1]));
            ms[i] = t;
        }
    });
}

int xc_grid_kernel_ms(xc_grid* g, double* ms) {
    return guard([&] {
        CGB_CHECK(g && ms, XC_ERR_ARG, "null argument");
        Grid& G = g->g;
        CGB_CHECK(G.profiling, XC_ERR_STATE, "profiling is off (xc_grid_profile)");
        CGB_CUDA(cudaEventSynchronize(G.ev[4]));
        const auto span = [&](int a, int b) {
            float t = 0;
            CGB_CUDA(cudaEventElapsedTime(&t, G.ev[a], G.ev[b]));
            return (double)t;
        };
        for (int i = 0; i < 3; i++) ms[i] = span(i, i + 1);
        ms[3] = ms[4] = ms[5] = 0;
        for (int s = 0; s < G.nspin; s++) {  // summed over the spins
            ms[3] += span(s == 0 ? 3 : 4 + 3 * s, 5 + 3 * s);
            ms[4] += span(5 + 3 * s, 6 + 3 * s);
            ms[5] += span(6 + 3 * s, 7 + 3 * s);
        }
    });
}

int xc_build_incremental(xc_grid* g, xc_functional* f, const double* D, int nspin, int anchor, double* E,
                         double* V) {
    return guard([&] {
        CGB_CHECK(g && f && D && E && V, XC_ERR_ARG, "null argument");
        Grid& G = g->g;
        CGB_CHECK(nspin == G.nspin && f->f.nspin == G.nspin, XC_ERR_ARG, "Wrong number of spin types!");
        CGB_CHECK(f->f.family <= G.type, XC_ERR_STATE, "grid type is below the functional family (setType/getAO)");
        CGB_CHECK((anchor & ~(XC_INCREMENTAL_FP32_POTENTIALS | 15)) == 0 && (anchor & 15) <= XC_ANCHOR_MIXED, XC_ERR_ARG,
                  "anchor must be 0..3, optionally with XC_INCREMENTAL_FP32_POTENTIALS");
        G.ensure_work();
        const size_t nn = (size_t)G.basis.nbasis * G.basis.nbasis * nspin;
        CGB_CUDA(cudaMemcpyAsync(G.d_D.p, D, nn * sizeof(double), cudaMemcpyHostToDevice, G.stream));
        G.build_incremental(G.d_D.p, f->f, G.d_scalar.p, G.d_V.p, anchor);
        CGB_CUDA(cudaMemcpyAsync(E, G.d_scalar.p, sizeof(double), cudaMemcpyDeviceToHost, G.stream));
        CGB_CUDA(cudaMemcpyAsync(V, G.d_V.p, nn * sizeof(double), cudaMemcpyDeviceToHost, G.stream));
        CGB_CUDA(cudaStreamSynchronize(G.stream));
        if (G.mixed_error()) throw Error(XC_ERR_TIMEOUT, "a bounded wait of the tensor-core pipeline gave up");
    });
}

int xc_grid_create_batch(int nmol, const xc_basis* const* bases, const char* grid_name, int nspin, xc_grid** out) {
    return guard([&] {
        CGB_CHECK(nmol > 0 && bases && grid_name && out, XC_ERR_ARG, "bad batch arguments");
        CGB_CHECK(nspin == 1 || nspin == 2, XC_ERR_ARG, "nspin must be 1 or 2");
        std::vector<BasisSet> mols;
        for (int i = 0; i < nmol; i++) {
            CGB_CHECK(bases[i], XC_ERR_ARG, "null basis in batch");
            mols.push_back(bases[i]->b);
        }
        auto* g = new xc_grid;
        try {
            g->g.build_batch(mols, grid_name, nspin);
        } catch (...) {
            delete g;
            throw;
        }
        *out = g;
    });
}

int xc_grid_molecules(const xc_grid* g, int* nmol, int* nbasis, long* npoints, long* offset) {
    return guard([&] {
        CGB_CHECK(g, XC_ERR_ARG, "null grid");
        const Grid& G = g->g;
        const int n = num_mols(G);
        if (nmol) *nmol = n;
        long off = 0;
        for (int i = 0; i < n; i++) {
            const int nb = G.batched ? G.mol_n[i] : G.basis.nbasis;
            if (nbasis) nbasis[i] = nb;
            if (npoints) npoints[i] = G.batched ? (long)G.sources[i].x.size() : G.npoints;
            if (offset) offset[i] = off;
            off += (long)G.nspin * nb * nb;
        }
    });
}

int xc_grid_wait_probe(xc_grid* g, double budget_ms) {
    return guard([&] {
        CGB_CHECK(g, XC_ERR_ARG, "null grid");
        CGB_CHECK(budget_ms > 0 && budget_ms <= 1000, XC_ERR_ARG, "budget_ms must be in (0, 1000]");
        Grid& G = g->g;
        CGB_CHECK(G.mx.ready, XC_ERR_STATE, "the wait probe needs the grid's tensor-core state (a mixed build first)");
        launch_wait_probe(budget_ms, G.mx.d_err.p, G.stream);
        if (G.mixed_error()) throw Error(XC_ERR_TIMEOUT, "a bounded wait of the tensor-core pipeline gave up");
    });
}

int xc_grid_set_mixed_config(xc_grid* g, const xc_mixed_config* cfg) {
    return guard([&] {
        CGB_CHECK(g && cfg, XC_ERR_ARG, "null argument");
        CGB_CHECK(cfg->screen >= 0 && std::isfinite(cfg->screen) && cfg->fock_tiles >= 0 &&
                      (cfg->spatial == 0 || cfg->spatial == 1) && cfg->v_operands >= 0 && cfg->v_operands <= 2 &&
                      cfg->func_float_above > 0 &&
                      !std::isnan(cfg->func_float_above),
                  XC_ERR_ARG, "bad mixed configuration");
        Grid& G = g->g;
        MixedConfig c;
        c.screen = cfg->screen;
        c.fock_tiles = cfg->fock_tiles;
        c.spatial = cfg->spatial;
        c.func_float_above = cfg->func_float_above;
        c.v_operands = cfg->v_operands;
        if (!c.same_tiles(G.mx.cfg)) G.mx.ready = false;
        G.mx.cfg = c;
        G.mx.have_ref = false;
        G.mx.drop_graph();
    });
}

int xc_grid_get_mixed_config(const xc_grid* g, xc_mixed_config* cfg) {
    return guard([&] {
        CGB_CHECK(g && cfg, XC_ERR_ARG, "null argument");
        const MixedConfig& c = g->g.mx.cfg;
        cfg->screen = c.screen;
        cfg->fock_tiles = c.fock_tiles;
        cfg->spatial = c.spatial;
        cfg->func_float_above = c.func_float_above;
        cfg->v_operands = c.v_operands;
    });
}

// Autotuner of the mixed path: screening threshold first (accuracy-gated),
// then the V work-item length, then the tile formation, each candidate built
// from scratch (tiles, AO store, work lists) and timed by CUDA events around
// graph replays.
int xc_grid_tune(xc_grid* g, xc_functional* f, const double* D, int nspin, double e_tol, double v_tol, int reps,
                 xc_tune_report* report) {
    return guard([&] {
        CGB_CHECK(g && f && D && e_tol > 0 && v_tol > 0, XC_ERR_ARG, "bad tune arguments");
        Grid& G = g->g;
        check_build(G, f, nspin, XC_PRECISION_MIXED);
        CGB_CHECK(G.batched || G.ao_order >= G.type, XC_ERR_STATE, "getAO must run before tuning");
        reps = std::max(1, std::min(reps, 50));
        G.ensure_work();
        const size_t nn = (size_t)G.packed_size();
        const int nm = num_mols(G);
        CGB_CUDA(cudaMemcpyAsync(G.d_D.p, D, nn * sizeof(double), cudaMemcpyHostToDevice, G.stream));
        const bool prof = G.profiling;
        G.profiling = false;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        CGB_CUDA(cudaEventCreate(&e0));
        CGB_CUDA(cudaEventCreate(&e1));
        struct Run {
            MixedConfig cfg;
            double ms;
            std::vector<double> E, V;
            long pairs;
        };
        auto run = [&](const MixedConfig& c) {
            Run r;
            r.cfg = c;
            G.prepare_mixed(c);
            G.build_mixed_graph(f->f);  // capture + warm-up
            CGB_CUDA(cudaStreamSynchronize(G.stream));
            if (G.mixed_error()) throw Error(XC_ERR_TIMEOUT, "a bounded wait of the tensor-core pipeline gave up");
            std::vector<double> t;
            for (int i = 0; i < reps; i++) {
                CGB_CUDA(cudaEventRecord(e0, G.stream));
                G.build_mixed_graph(f->f);
                CGB_CUDA(cudaEventRecord(e1, G.stream));
                CGB_CUDA(cudaEventSynchronize(e1));
                float ms = 0;
                CGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                t.push_back(ms);
            }
            std::sort(t.begin(), t.end());
            r.ms = t[t.size() / 2];
            r.E.resize(nm);
            r.V.resize(nn);
            CGB_CUDA(cudaMemcpyAsync(r.E.data(), G.d_Emol.p, nm * sizeof(double), cudaMemcpyDeviceToHost, G.stream));
            CGB_CUDA(cudaMemcpyAsync(r.V.data(), G.d_V.p, nn * sizeof(double), cudaMemcpyDeviceToHost, G.stream));
            CGB_CUDA(cudaStreamSynchronize(G.stream));
            r.pairs = G.mx.kept_pairs;
            return r;
        };
        MixedConfig rc;
        rc.screen = 1e-14;
        rc.spatial = 1;
        rc.fock_tiles = 0;
        rc.func_float_above = G.mx.cfg.func_float_above;
        rc.v_operands = G.mx.cfg.v_operands;
        const Run ref = run(rc);
        std::vector<xc_tune_candidate> cands;
        auto assess = [&](const Run& r) {
            xc_tune_candidate c{};
            c.cfg.screen = r.cfg.screen;
            c.cfg.fock_tiles = r.cfg.fock_tiles;
            c.cfg.spatial = r.cfg.spatial;
            c.cfg.func_float_above = r.cfg.func_float_above;
            c.cfg.v_operands = r.cfg.v_operands;
            c.ms = r.ms;
            for (int i = 0; i < nm; i++) c.max_de = std::max(c.max_de, std::fabs(r.E[i] - ref.E[i]));
            for (size_t i = 0; i < nn; i++) c.max_dv = std::max(c.max_dv, std::fabs(r.V[i] - ref.V[i]));
            c.kept_pairs = r.pairs;
            c.accepted = c.max_de <= e_tol && c.max_dv <= v_tol;
            cands.push_back(c);
            return c;
        };
        MixedConfig best = rc;
        double best_ms = ref.ms;
        auto consider = [&](const MixedConfig& c) {
            const xc_tune_candidate k = assess(run(c));
            if (k.accepted && k.ms < best_ms) {
                best = c;
                best_ms = k.ms;
            }
        };
        for (double thr : {1e-8, 1e-9, 1e-10, 1e-11, 1e-12}) {
            MixedConfig c = rc;
            c.screen = thr;
            consider(c);
        }
        // V work-item length around the SM-count default
        {
            long work = 0;
            int nsm = 148, dev = 0;
            CGB_CUDA(cudaGetDevice(&dev));
            CGB_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
            G.prepare_mixed(best);
            for (auto& R : G.mx.mols) work += (long)(R.t1 - R.t0) * R.nblk * R.nblk;
            const long L = std::max(1L, (work + 6L * nsm - 1) / (6L * nsm));
            const MixedConfig base = best;
            for (long Lc : {L / 4, L / 2, 2 * L, 4 * L}) {
                if (Lc < 1) continue;
                MixedConfig c = base;
                c.fock_tiles = (int)Lc;
                consider(c);
            }
        }
        {
            MixedConfig c = best;
            c.spatial = 0;
            consider(c);
        }
        {
            // both operand forms of the tensor-core kernels (pre-split planes /
            // in-kernel split) when the automatic choice finds that the planes fit
            MixedConfig probe = best;
            probe.v_operands = 0;
            G.prepare_mixed(probe);
            if (G.mx.use16) {
                MixedConfig c = best;
                c.v_operands = best.v_operands == 1 ? 2 : 1;
                consider(c);
            }
        }
        CGB_CUDA(cudaEventDestroy(e0));
        CGB_CUDA(cudaEventDestroy(e1));
        G.prepare_mixed(best);
        G.profiling = prof;
        if (report) {
            std::memset(report, 0, sizeof(*report));
            report->best.screen = best.screen;
            report->best.fock_tiles = best.fock_tiles;
            report->best.spatial = best.spatial;
            report->best.func_float_above = best.func_float_above;
            report->best.v_operands = best.v_operands;
            report->ms_best = best_ms;
            report->ms_reference = ref.ms;
            report->ncand = (int)std::min<size_t>(cands.size(), 32);
            for (int i = 0; i < report->ncand; i++) report->cand[i] = cands[i];
        }
    });
}

static void sap_fock(xc_grid* g, double* V, bool tensor_cores) {
    {
        CGB_CHECK(g && V, XC_ERR_ARG, "null argument");
        Grid& G = g->g;
        CGB_CHECK(!G.batched, XC_ERR_UNSUPPORTED, "the SAP guess is per molecule");
        CGB_CHECK(G.ao_order >= 0, XC_ERR_STATE, "getAO must run before the SAP guess");
        G.ensure_work();
        const int natoms = G.basis.natoms();
        std::vector<double> radii, table((size_t)natoms * 751), rv;
        for (int a = 0; a < natoms; a++) {
            sap_table(G.basis.Z[a], radii, rv);
            CGB_CHECK(rv.size() == 751 && radii.size() == 751, XC_ERR_IO, "corrupt SAP table");
            std::memcpy(&table[(size_t)a * 751], rv.data(), 751 * sizeof(double));
        }
        DevBuf<double> d_table, d_radii;
        d_table.upload(table.data(), table.size(), G.stream);
        d_radii.upload(radii.data(), radii.size(), G.stream);
        // GuessSCF.cpp:19-37: pretend LDA, one spin; V = sum_g w v phi phi
        launch_sap_coef(G.Gp, natoms, G.d_atoms.p, d_table.p, d_radii.p, G.d_x.p, G.d_y.p, G.d_z.p, G.d_w.p,
                        G.d_fcoef.p, G.stream);
        const int n = G.basis.nbasis;
        const size_t nn = (size_t)n * n;
        if (tensor_cores) {
            // the same V through the mixed path's tiles: coefficients gathered
            // into tile order, LDA-type Z operand, tensor-core partials, FP64 sum
            G.mixed_ready();
            MixedState& m = G.mx;
            launch_gather(m.d_perm.p, m.md.Gt, G.Gp, 5, G.d_fcoef.p, m.fcoef.p, true, G.stream);
            G.v_prep(m.fcoef.p, 0);
            G.v_partials(1);
            launch_wsum(m.d_wpart.p, m.d_item_live.p, m.d_mols.p, 1, n, 0, 1, G.d_V.p, G.stream);
        } else {
            CGB_CUDA(cudaMemsetAsync(G.d_V.p, 0, nn * sizeof(double), G.stream));
            launch_fock_fp64((int)G.blocks.size(), G.d_blocks.p, G.d_lists.p, G.max_nb, n, 1, 0, G.d_ao.p, G.Gp,
                             G.d_fcoef.p, G.d_V.p, G.stream);
        }
        CGB_CUDA(cudaMemcpyAsync(V, G.d_V.p, nn * sizeof(double), cudaMemcpyDeviceToHost, G.stream));
        CGB_CUDA(cudaStreamSynchronize(G.stream));
        G.have_potential = false;  // fcoef overwritten
        if (tensor_cores && G.mixed_error())
            throw Error(XC_ERR_TIMEOUT, "a bounded wait of the tensor-core pipeline gave up");
    }
}

int xc_sap_fock(xc_grid* g, double* V) {
    return guard([&] { sap_fock(g, V, false); });
}

int xc_sap_fock_tc(xc_grid* g, double* V) {
    return guard([&] { sap_fock(g, V, true); });
}

}  // extern "C"
