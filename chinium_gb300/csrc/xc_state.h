// State behind the opaque C handles: the Grid (SubGrid blocks, AO store and
// per-point work arrays, all resident in HBM) and the functional.
#pragma once

#include <string>
#include <vector>

#include "common.h"
#include "kernels.h"
#include "mixed.h"
#include "model.h"

namespace cgb {

void ensure_device();

// Default AO screening threshold of the mixed-precision tiles (|phi|, |grad phi|).
constexpr double kMixedScreen = 1e-11;
struct Functional {
    std::vector<int> ids;
    int nspin = 1;
    int family = 0;
    double exx = 0;
    xcf::FuncDesc desc{};
    void init(const std::vector<int>& ids, int nspin);
};

// One molecule of the mixed path: its real points (generation order) and its
// place in the combined basis.
struct MolSource {
    int n = 0, f0 = 0, sh0 = 0, sh1 = 0;
    std::vector<double> x, y, z, w;
    std::vector<long> src;  // index of each point in the grid's FP64 arrays (-1: none)
};

struct Grid {
    BasisSet basis;
    int nspin = 1;
    int type = 0;
    double screen_thr = 0;
    cudaStream_t stream = nullptr;

    long npoints = 0, Gp = 0;
    std::vector<BlockDesc> blocks;
    std::vector<int> basis_lists, shell_lists;
    std::vector<double> hx, hy, hz;
    int max_nb = 0;
    long screened_pairs = 0;
    long ao_elements = 0;
    int ncomp = 0;
    int ao_order = -1;
    bool have_density = false, have_potential = false;
    int eval_family = 0;
    int n_partial = 0;

    DevBuf<double> d_x, d_y, d_z, d_w, d_atoms;
    DevBuf<int> d_sh_type, d_sh_l, d_sh_nprim, d_sh_poff, d_sh_first;
    DevBuf<double> d_sh_xyz, d_exps, d_coefs;
    DevBuf<BlockDesc> d_blocks;
    DevBuf<int> d_lists, d_shell_lists;
    DevBuf<double> d_ao;
    DevBuf<float2> d_ao_ff, d_D_ff;  // float-float copies for the reference densities of incremental builds
    int ao_ff_order = -1;            // AO order d_ao_ff was split from (-1: none)
    DevBuf<double> d_rho, d_rho1, d_tau, d_sigma, d_eps, d_vrho, d_vsigma, d_vtau, d_fcoef, d_partial, d_scalar;
    DevBuf<double> d_D, d_V;

    // stage timing: events bracket density, functional, energy, fock
    bool profiling = false;
    // 0-4: build stage bounds; 5 + 3 s, 6 + 3 s, 7 + 3 s: after spin s's Z
    // operand, tensor-core V partials and V reduction (mixed path)
    cudaEvent_t ev[11] = {};
    void mark(int i);
    ~Grid();

    void build(const BasisSet& b, const std::string& grid_name, int nspin, double thr);
    DevShells dev_shells() const;
    void get_ao(int derivative);
    void ensure_work();
    void density_device(const double* dD, bool float_float = false);
    void evaluate(const Functional& f, double float_above = __builtin_huge_val());
    void energy_device(double* dE);
    void fock_device(double* dV, int family);

    // response (coupled-perturbed) V_xc, FP64, LDA / GGA: Evaluate("f"), getDensityU, getFockU<u_t>
    bool have_fxc = false, have_density_u = false;
    int fxc_family = 0;
    int nmat_u = 0;
    DevBuf<double> d_f2, d_DU, d_rhoU, d_rho1U, d_fcoefU;
    void evaluate_fxc(const Functional& f);
    void density_u_device(const double* dDU, int nmat);  // D_U (s, nmat, n, n) on the device
    void fock_u_device(double* dFU);                      // V_U (s, nmat, n, n)
    // the same on the tensor cores (symmetric part of each D_U): ground-state grad rho,
    // vsigma and f_xc gathered into tile order once, then density and V_U per matrix
    DevBuf<double> d_rt_rho1, d_rt_vsig, d_rt_f2, d_rt_fcU, d_rt_D, d_rt_V;
    int resp_precision = 0;  // xc_precision of getDensityU / getFockU
    bool rt_ready = false;   // tile-order ground state matches the current Evaluate("f")
    void response_tiles_prepare();
    void response_mixed(const double* dDU, int nmat, double* dFU);

    // mixed-precision (tensor-core) path; tiles and stores are prepared on first use
    MixedState mx;
    std::vector<MolSource> sources;  // molecules of the mixed path (one unless batched)
    bool batched = false;            // built by build_batch: mixed precision only
    std::vector<int> mol_n;          // basis functions of each molecule
    long packed_size() const;        // doubles of packed per-molecule D / V: sum nspin n^2
    DevBuf<double> d_Emol;           // per-molecule energies of the last mixed build
    cudaStream_t capture_stream = nullptr;
    void build_batch(const std::vector<BasisSet>& mols, const std::string& grid_name, int nspin);
    void collect_sources();
    void prepare_mixed(const MixedConfig& cfg);
    void mixed_ready();
    void density_passes(const __nv_bfloat16* Dp);
    // float_above < 0: the configured FP32-functional bound
    void build_mixed(const double* dD, const Functional& f, double* dE, double* dV, double float_above = -1.0);
    void build_mixed_graph(const Functional& f);  // d_D -> d_Emol, d_V through a CUDA graph
    // anchor: 0 incremental (FP64 anchor on the first call), 1 FP64 anchor, 2 tensor-core anchor
    void build_incremental(const double* dD, const Functional& f, double* dE, double* dV, int anchor);
    void save_refs(const double* dD, const double* dV);
    void v_prep(const double* fcoef_s, int family);
    void v_partials(int ncomp);
    int mixed_error();
};

}  // namespace cgb

struct xc_basis {
    cgb::BasisSet b;
};
struct xc_grid {
    cgb::Grid g;
};
struct xc_functional {
    cgb::Functional f;
};
