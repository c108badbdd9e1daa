/*
 * chinium_xc.h -- C ABI of the GB300 Kohn-Sham exchange-correlation build.
 *
 * Drop-in boundary for Chinium's XC path: the `Grid` class
 * (src/Grid/Grid.h:90-116) and `ExchangeCorrelation` (src/ExchangeCorrelation.h:8-17)
 * that the SCF drivers call once per iteration (src/HartreeFockKohnSham/
 * Restricted/SP.cpp:51-56, Unrestricted/SP.cpp:64-71, Universal.cpp:49-73,
 * GuessSCF.cpp:60).  Each entry point names the member it replaces.
 *
 * Conventions
 *   - Every function returns an int status: XC_OK (0) or a negative XC_ERR_*;
 *     xc_last_error() copies the calling thread's last message.  No exception
 *     crosses the ABI.
 *   - Matrices are n x n FP64 column-major (Eigen's default), one per spin,
 *     spins concatenated: element (mu, nu, s) at D[s*n*n + nu*n + mu].
 *   - Host buffers are caller-owned.  Device buffers are library-owned, except
 *     in the *_device entry points, which take caller-owned device pointers.
 *   - A handle is used by one host thread at a time.  Work is issued on the
 *     handle's CUDA stream (xc_grid_set_stream); host-buffer calls return
 *     after their results are in host memory.
 *   - Coordinates are in bohr.
 */
#ifndef CHINIUM_XC_H
#define CHINIUM_XC_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum xc_status {
    XC_OK = 0,
    XC_ERR_ARG = -1,         /* bad argument (null, size, range) */
    XC_ERR_IO = -2,          /* missing or corrupt data file (grid, basis, .df) */
    XC_ERR_CUDA = -3,        /* CUDA runtime error, or no usable GPU */
    XC_ERR_STATE = -4,       /* call order violated (e.g. energy before density) */
    XC_ERR_NOMEM = -5,       /* host or device allocation failed */
    XC_ERR_UNSUPPORTED = -6, /* functional id / shell type not implemented */
    XC_ERR_NUMERIC = -7,     /* non-finite values detected in inputs or results */
    XC_ERR_TIMEOUT = -8,     /* a bounded device-side wait gave up */
    XC_ERR_INTERNAL = -9
};

enum xc_precision {
    XC_PRECISION_FP64 = 0,  /* plain path: every stage in FP64 */
    XC_PRECISION_MIXED = 1  /* tensor-core split-precision contractions, FP64 accumulation */
};

enum xc_family { XC_FAMILY_LDA = 0, XC_FAMILY_GGA = 1, XC_FAMILY_MGGA = 2 };

typedef struct xc_basis xc_basis;           /* centres + contracted shells (libmwfn Mwfn role) */
typedef struct xc_grid xc_grid;             /* Grid */
typedef struct xc_functional xc_functional; /* ExchangeCorrelation */

/* Copies the calling thread's last error message (NUL-terminated). */
int xc_last_error(char* buf, size_t len);

/* Directory holding lebedev.txt, grids/, basis/, sap.txt (the role of
 * $CHINIUM_PATH in GridGeneration.cpp:234 and ExchangeCorrelation.cpp:21). */
int xc_set_data_path(const char* path);

/* ------------------------------------------------------------------ basis */

/* Centres and shells from a basis-set name (Representation.cpp:30-37 +
 * Normalization.cpp:11-18: libint2-normalised contractions).  P shells are
 * Cartesian (x, y, z); d and higher are pure (m = -l..l). */
int xc_basis_create(int natoms, const int* Z, const double* xyz_bohr, const char* basis_name,
                    xc_basis** out);
/* Centres and shells from the caller's own basis, as Grid::Grid(Mwfn*, ...)
 * reads them (GridGeneration.cpp:232-271 through SubGrid::getAO,
 * GridAO.cpp:14-215: per MwfnShell its centre, Type, Exponents and
 * NormalizedCoefficients).  Shells in basis-function order; per shell its
 * atom (0..natoms-1), type (0 s, 1 Cartesian p in x, y, z order, -l pure
 * l = 1..4 with m = -l..l, pure p being y, z, x) and primitive count;
 * exps/coefs of length sum(nprim), shell by shell.  normalize = 0 takes
 * coefs as normalised by the caller (the Mwfn's NormalizedCoefficients
 * after Normalize(), Normalization.cpp:11-18); normalize = 1 applies that
 * libint2 renormalisation to raw contraction coefficients.  Z gives the
 * Becke partition and the SG-n recipe of each atom. */
int xc_basis_create_shells(int natoms, const int* Z, const double* xyz_bohr, int nshells,
                           const int* shell_atom, const int* shell_type, const int* nprim,
                           const double* exps, const double* coefs, int normalize, xc_basis** out);
int xc_basis_nbasis(const xc_basis* b, int* nbasis);
/* Shell layout: per shell its atom, type (0 S, 1 Cartesian P, -l pure l),
 * first function index and primitive count; arrays of length nshells. */
int xc_basis_nshells(const xc_basis* b, int* nshells);
int xc_basis_shells(const xc_basis* b, int* atom, int* type, int* first, int* nprim);
/* Normalised primitive data; exps/coefs of length sum(nprim). */
int xc_basis_primitives(const xc_basis* b, double* exps, double* coefs);
int xc_basis_destroy(xc_basis* b);

/* ------------------------------------------------------------------- grid */

/* Grid::Grid(Mwfn*, grid, nthreads, output) (GridGeneration.cpp:232-310):
 * SG-n atom grids, Becke partition (FP64, on the GPU), blocks of <= 128
 * points by recursive halving in generation order, padded to a multiple of
 * 8.  nspin is 1 (restricted) or 2 (unrestricted) (SubGrid::Spin).
 * screen_threshold: AO magnitude below which a shell is dropped from a block
 * (0 keeps every shell in every block, as the reference does). */
int xc_grid_create(const xc_basis* b, const char* grid_name, int nspin, double screen_threshold,
                   xc_grid** out);
int xc_grid_destroy(xc_grid* g);
/* Optional CUDA stream (cudaStream_t passed as void*); NULL = legacy default. */
int xc_grid_set_stream(xc_grid* g, void* stream);

/* Grid::setType (Grid.cpp:14-20): 0 LDA, 1 GGA, 2 meta-GGA. */
int xc_grid_set_type(xc_grid* g, int type);

/* Grid::getAO(derivative, output) (Grid.cpp:22-33): evaluates and stores AO
 * values to order type+derivative (<= 1 here) for every block. */
int xc_grid_get_ao(xc_grid* g, int derivative);

/* Grid::getNumElectrons (Grid.cpp:51-61). */
int xc_grid_num_electrons(xc_grid* g, double* n);

/* Grid::getDensity(std::vector<EigenMatrix>) (Grid.cpp:35-49): D is nspin
 * n x n matrices; restricted callers pass the total density 2*C_occ C_occ^T. */
int xc_grid_get_density(xc_grid* g, const double* D, int nspin);

/* Grid::getEnergy (Grid.cpp:112-122): E_xc = sum_g w_g (sum_s rho_gs) eps_g. */
int xc_grid_get_energy(xc_grid* g, double* E);

/* Grid::getFock (Grid.cpp:156-171): V_xc, nspin matrices into V. */
int xc_grid_get_fock(xc_grid* g, double* V);

/* Sizes and per-block layout, for inspection and parity tests. */
typedef struct xc_grid_info {
    long npoints;        /* real points (sum of unpadded block sizes) */
    long npoints_padded; /* sum of padded block sizes */
    int nblocks;
    int nbasis;
    int nspin;
    int type;
    long ao_elements;    /* stored AO values per component */
    long screened_pairs; /* sum over blocks of n_b^2 */
    int mixed_tiles;     /* 128-point tiles of the mixed-precision path (0 before its first build) */
    long mixed_pairs;    /* sum over tiles of (kept functions)^2 */
    long mixed_rows;     /* kept function rows of all tiles (FP32 AO store: rows x 128 x components) */
    long mixed_store_bytes; /* device bytes of the FP32 AO store and the per-build Z operand */
    int mixed_launches;  /* kernels one mixed build launches (for the current type and spins) */
    long mixed_units_full; /* density units (128 x 128 x 64 products) of a full pass (rho + grad rho) */
    long mixed_units_sym;  /* density units of a symmetric pass (rho of LDA, each tau component) */
    long mixed_fock_jobs;  /* V (item, tile) jobs, each 128 x 128 x 128 per component */
    long mixed_fock_tau_jobs; /* jobs that also carry the meta-GGA components (I <= J) */
    long mixed_presplit;      /* 1: the tensor-core kernels read pre-split BF16 planes (v_operands) */
    long mixed_presplit_bytes; /* bytes of those planes (AO store, density A planes, per-build R planes) */
    long mixed_fock_items;    /* V work items with at least one job (one W partial written each) */
    long mixed_empty_tiles;   /* tiles whose points no kept chunk reaches (zero density there) */
} xc_grid_info;
int xc_grid_info_get(const xc_grid* g, xc_grid_info* info);
/* Padded points in block order: x, y, z, w (each npoints_padded) and
 * per-block (offset, padded size, real size, n_b). */
int xc_grid_points(const xc_grid* g, double* x, double* y, double* z, double* w, int* blk_off,
                   int* blk_ng, int* blk_nreal, int* blk_nbasis);
/* Per-point densities in block order: rho (s, G), rho1 (s, 3, G),
 * sigma (ns(ns+1)/2, G), tau (s, G); NULL skips an array. */
int xc_grid_density_values(const xc_grid* g, double* rho, double* rho1, double* sigma,
                           double* tau);
/* Per-point functional outputs: eps (G), vrho (s, G), vsigma (ns(ns+1)/2, G),
 * vtau (s, G); NULL skips an array. */
int xc_grid_potential_values(const xc_grid* g, double* eps, double* vrho, double* vsigma,
                             double* vtau);
/* AO values of one block: ao (n_b, ng) and, if stored, ao1 (3, n_b, ng);
 * basis_list (n_b) gives the global function index of each row. */
int xc_grid_block_ao(const xc_grid* g, int block, double* ao, double* ao1, int* basis_list);

/* ------------------------------------------------------------- functional */

/* ExchangeCorrelation::Read(df, output) (ExchangeCorrelation.cpp:18-84):
 * reads the libxc ids of a named functional (PBE, B3LYP, TPSS, R2SCAN, ...). */
int xc_functional_read(const char* df_name, int nspin, xc_functional** out);
/* Same, from explicit libxc ids. */
int xc_functional_create(const int* ids, int nids, int nspin, xc_functional** out);
int xc_functional_destroy(xc_functional* f);
/* Public fields EXX and Family (ExchangeCorrelation.h:10-12). */
int xc_functional_exx(const xc_functional* f, double* exx);
int xc_functional_family(const xc_functional* f, int* family);

/* ExchangeCorrelation::Evaluate(order, grid) (ExchangeCorrelation.cpp:165-248):
 * order "e", "v" or "ev" on the grid's current density; "f" stores the
 * second derivatives (v2rho2, v2rhosigma, v2sigma2; :101-133, :192-199,
 * :241-244) for xc_grid_get_fock_u, LDA and GGA functionals only (the
 * reference's meta-GGA branch has no "f"; here it fails with
 * XC_ERR_UNSUPPORTED). */
int xc_evaluate(xc_functional* f, xc_grid* g, const char* order);

/* Pointwise evaluation on caller data (host arrays, layout as
 * xc_grid_density_values/xc_grid_potential_values), for parity tests. */
int xc_functional_eval_points(xc_functional* f, long npoints, const double* rho,
                              const double* sigma, const double* tau, double* eps, double* vrho,
                              double* vsigma, double* vtau);

/* Allocation-free functional + E_xc on caller-owned device arrays.  No
 * counterpart in the reference: it serves callers that may not call
 * cudaMalloc / cudaFree (device memory owned by another allocator, or code
 * that must not trigger their device-wide synchronisation).  Inputs rho
 * (s, n), sigma (ns(ns+1)/2, n), tau (s, n) and weights w (n); outputs eps
 * (n), vrho, vsigma, vtau (layouts as the inputs) and *d_E = sum_g w_g
 * rho_g eps_g.  The only scratch (per-CTA energy partials) is a fixed array
 * inside the library, so npoints <= 2 097 152; larger calls fail with
 * XC_ERR_ARG.  The first call on a device looks up that array's device
 * address (with that device current); make that first call before any stream
 * capture.  A lookup that fails returns XC_ERR_CUDA and is not remembered:
 * the next call on that device tries again.  Calls share the array, so calls
 * whose kernels overlap on the GPU race and must be serialised by the
 * caller.  Work is enqueued on `stream`
 * (cudaStream_t as void*, NULL = legacy default) without synchronising. */
int xc_functional_energy_static(const xc_functional* f, long npoints, const double* d_w,
                                const double* d_rho, const double* d_sigma, const double* d_tau,
                                double* d_eps, double* d_vrho, double* d_vsigma, double* d_vtau,
                                double* d_E, void* stream);

/* ------------------------------------------------------------ fused build */

/* getDensity + Evaluate("ev") + getEnergy + getFock in one call
 * (the sequence at Restricted/SP.cpp:52-55).  Host buffers in and out. */
int xc_build(xc_grid* g, xc_functional* f, const double* D, int nspin, int precision, double* E,
             double* V);

/* Same with caller-owned device pointers (d_D in, d_E and d_V out, packed
 * per molecule), issued on the grid's stream; does not synchronise.  Mixed
 * builds replay a CUDA graph of the whole launch sequence (captured at the
 * first build for a functional and grid type). */
int xc_build_device(xc_grid* g, xc_functional* f, const double* d_D, int nspin, int precision,
                    double* d_E, double* d_V);

/* Per-stage device timing of the last build (the reference's __now__ /
 * __duration__ printouts around its stages, src/Macro/Time.h:1-2, as CUDA
 * events on the grid's stream).  enable != 0 records events from the next
 * build on; xc_grid_stage_ms waits for them and returns milliseconds of
 * [density, functional, energy, fock] in ms[0..3]. */
int xc_grid_profile(xc_grid* g, int enable);
int xc_grid_stage_ms(xc_grid* g, double* ms);
/* Finer device timing of the last profiled mixed build: ms[0..5] =
 * [density planes + tensor-core density, functional, per-molecule E_xc,
 * Z operand, tensor-core V partials, FP64 V reduction], the last three summed
 * over the spins.  No reference counterpart. */
int xc_grid_kernel_ms(xc_grid* g, double* ms);

/* Nuclear gradient of E_xc with the grid held fixed (SubGrid::getDensitySkeleton
 * + SubGrid::getEnergyGrad, GridDensity.cpp:79-130, GridEnergy.cpp:15-30,
 * summed over blocks as Grid::getEnergyGrad): grad[3 * atom + t] = dE_xc/dR
 * from the derivatives of the basis functions centred on each atom, FP64.
 * LDA and GGA functionals (the reference's gradient has no meta-GGA terms);
 * needs the AO derivatives one order above the functional's: getAO(1) after
 * setType.  D as for xc_build (column-major, spins concatenated).  With
 * xc_grid_profile on, xc_grid_stage_ms then returns [density, functional,
 * gradient kernel, 0]. */
int xc_grid_energy_grad(xc_grid* g, xc_functional* f, const double* D, int nspin, double* grad);

/* The Hessian's skeleton V_xc derivatives with the grid held fixed, FP64, LDA
 * and GGA (Restricted/Hess.cpp:83-97): FS = getFockSkeleton (GridFock.cpp:52-95)
 * and FU = getFockU<s_t> (GridFock.cpp:97-160) on the skeleton density
 * derivatives of getDensitySkeleton (GridDensity.cpp:79-130), for every atom A
 * and direction t: nspin x 3 natoms column-major n x n matrices, matrix
 * (s * 3 natoms + 3 A + t).  FS + FU is dV_xc / dR_(A,t) at fixed D.  Needs
 * getAO(1) after setType (AO derivatives one order above the functional's).
 * D as for xc_build. */
int xc_grid_fock_skeleton(xc_grid* g, xc_functional* f, const double* D, int nspin, double* FS, double* FU);

/* --------------------------------------------- response (coupled-perturbed)
 * FP64, LDA and GGA.  D_U and V_U hold nspin x nmat column-major n x n
 * matrices, spin-major: matrix m of spin s starts at (s * nmat + m) n^2, as
 * the reference's std::vector<std::vector<EigenMatrix>> D[spin][mat]. */

/* Second derivatives on caller points (host arrays): rho (s, n), sigma
 * (1 or 3, n) -> v2rho2 (1 or 3, n), v2rhosigma (1 or 6, n), v2sigma2 (1 or 6,
 * n) in libxc's layouts (rho_a rho_a, rho_a rho_b, rho_b rho_b; rho_a sigma_aa,
 * rho_a sigma_ab, rho_a sigma_bb, rho_b sigma_aa, ...; the upper triangle of
 * sigma_aa, sigma_ab, sigma_bb).  For parity tests. */
int xc_functional_fxc_points(xc_functional* f, long npoints, const double* rho, const double* sigma,
                             double* v2rho2, double* v2rhosigma, double* v2sigma2);

/* Grid::getDensityU (Grid.cpp:63-77, GridDensity.cpp:47-77): response
 * densities rho_U = sum D_U phi phi and grad rho_U = 2 sum D_U(mu, nu)
 * grad phi_mu phi_nu of every matrix, kept on the grid. */
int xc_grid_get_density_u(xc_grid* g, const double* DU, int nspin, int nmat);

/* Grid::getFockU<u_t> (Grid.cpp:194-218, GridFock.cpp:97-160): V_U of every
 * matrix of the last xc_grid_get_density_u, from the second derivatives of
 * Evaluate("f") and, for GGAs, vsigma and grad rho of the ground-state
 * density (getDensity + Evaluate("v"/"ev") + Evaluate("f") first).  V_U is the
 * derivative of V_xc along D_U.  Restricted grids reproduce the reference's
 * expression; unrestricted grids use the libxc layout of v2rhosigma and the
 * spin-diagonal factor 2 on the output sigma pair, where the reference copies
 * v2rhosigma into a (g, 2, 3) tensor in the other index order
 * (ExchangeCorrelation.cpp:243) and scales the contracted pair
 * (GridFock.cpp:136-138, 145). */
int xc_grid_get_fock_u(xc_grid* g, double* FU);

/* Precision of xc_grid_get_density_u / xc_grid_get_fock_u (no reference
 * counterpart; default XC_PRECISION_FP64).  XC_PRECISION_MIXED keeps the
 * FP64 ground state of Evaluate("ev") / Evaluate("f"), gathered once into the
 * tensor-core tiles, and forms each matrix's response density (symmetric part
 * of D_U) and V_U on the tensor cores inside xc_grid_get_fock_u: the
 * per-iteration work of a CPSCF loop (CoupledPerturbed.cpp:131-134).  With
 * xc_grid_profile on, xc_grid_stage_ms after such a getFockU returns the first
 * matrix's [response density, coefficients + V operand planes, V partials,
 * V sum] of spin 0. */
int xc_grid_set_response_precision(xc_grid* g, int precision);

/* getDensity(D) + Evaluate("ev") + Evaluate("f") + getDensityU(D_U) +
 * getFockU<u_t>, the sequence of CoupledPerturbed.cpp:131-134 and
 * Universal.h:92-118, in one call (matrices processed in chunks that bound
 * the device scratch).  Host buffers.  precision XC_PRECISION_FP64 is the
 * plain path (as xc_grid_get_fock_u); XC_PRECISION_MIXED keeps the ground
 * state (densities, vsigma, second derivatives) in FP64 and forms each
 * matrix's response density and V_U on the tensor cores (split-BF16 products,
 * FP32 accumulation per unit, FP64 sums; ~1e-6 relative), from the symmetric
 * part of D_U -- the response matrices of the reference's callers are
 * symmetric (CoupledPerturbed.cpp:113). */
int xc_build_response(xc_grid* g, xc_functional* f, const double* D, int nspin, int precision, int nmat,
                      const double* DU, double* FU);

/* Incremental mixed-precision build for SCF iterations (the per-iteration
 * sequence at Restricted/SP.cpp:52-55, fused).  Densities are linear in D
 * and V_xc is linear in the per-point potential coefficients, so this call
 * forms rho(D) = rho_ref + rho(D - D_ref) and V = V_ref + V(c - c_ref) with
 * only the differences on the tensor cores (split-BF16, FP32 accumulation);
 * the functional and E_xc are FP64 on the reconstructed densities.  The
 * tensor-core error is relative to the change since the previous call, so it
 * vanishes as an SCF converges.  anchor resets the references: 1 (or the
 * first call on a grid with anchor 0) by a full FP64 build; 2 by densities
 * at FP64 level (float-float arithmetic on the FP32 pipe, ~1e-14 relative),
 * the FP64 functional and E_xc, with V on the tensor cores (a fraction of the
 * cost: an error in V moves a converged SCF energy only at second order,
 * while E_xc takes the density's error at first order); 3 by a full
 * tensor-core build (as xc_build with XC_PRECISION_MIXED: the densities'
 * split-BF16 error then stays in every later E_xc, ~1e-7 relative).  OR-ing
 * XC_INCREMENTAL_FP32_POTENTIALS into anchor runs the functional of the
 * incremental builds as a full mixed build does (FP32 potentials at points
 * whose density is at least the mixed config's func_float_above, FP64 energy
 * density everywhere): E_xc keeps FP64 arithmetic on the reconstructed
 * densities, V_xc takes FP32-level noise.  Host buffers. */
#define XC_ANCHOR_NONE 0
#define XC_ANCHOR_FP64 1
#define XC_ANCHOR_DENSITY 2
#define XC_ANCHOR_MIXED 3
#define XC_INCREMENTAL_FP32_POTENTIALS 16
int xc_build_incremental(xc_grid* g, xc_functional* f, const double* D, int nspin, int anchor,
                         double* E, double* V);

/* SAP potential matrix (GuessSCF.cpp:17-75): V_mu,nu = sum_g w v_SAP(r_g)
 * phi_mu phi_nu with v_SAP the nearest-radius tabulated atomic potentials. */
int xc_sap_fock(xc_grid* g, double* V);
/* The same matrix through the mixed path's tiles (split-BF16 tensor-core
 * partials, FP64 sum; FP32-level accuracy, which a starting guess can take). */
int xc_sap_fock_tc(xc_grid* g, double* V);

/* ------------------------------------------------------- batched molecules
 * No reference counterpart: the reference builds one Grid per molecule
 * (src/Grid/Grid.h:90-116).  A batch grid holds many molecules, each with
 * its own Becke-partitioned grid (the same generation as xc_grid_create with
 * screen threshold 0); the mixed-precision build processes the point tiles
 * of all of them in one persistent launch per stage.  Only
 * XC_PRECISION_MIXED builds are available on a batch grid.
 * Packed per-molecule matrices: molecule m's (nspin, n_m, n_m) column-major
 * block starts at sum_{k<m} nspin n_k^2; E holds one value per molecule.
 * xc_build / xc_build_device on any grid use this layout (one molecule: the
 * usual (nspin, n, n) matrix and a scalar E). */
int xc_grid_create_batch(int nmol, const xc_basis* const* bases, const char* grid_name, int nspin,
                         xc_grid** out);
/* Number of molecules; per molecule (arrays of nmol, each may be NULL):
 * basis functions, real grid points, offset of its block in packed D / V. */
int xc_grid_molecules(const xc_grid* g, int* nmol, int* nbasis, long* npoints, long* offset);

/* Diagnostic of the failure path, no reference counterpart.  Every wait of
 * the tensor-core pipelines is bounded (2 s); one that gives up records
 * XC_ERR_TIMEOUT and its kernel unwinds (TMEM released) instead of hanging,
 * and the build returns XC_ERR_TIMEOUT with the context still usable.  This
 * call runs the same set-up and wait in a one-CTA kernel on a barrier that
 * nothing arrives on, for budget_ms (<= 1000), and returns what a build whose
 * wait gave up returns: XC_ERR_TIMEOUT.  Needs a mixed build on the grid
 * first; later builds on the grid are unaffected. */
int xc_grid_wait_probe(xc_grid* g, double budget_ms);

/* Knobs of the mixed path.  screen: chunk screening threshold on |phi| and
 * |grad phi| (0 keeps every chunk); fock_tiles: point tiles per V work item
 * (0 = from the SM count); spatial: 1 forms tiles from k-d cells of each
 * molecule's points, 0 from 128 consecutive points in generation order.
 * func_float_above: points whose total density is at least this value
 * evaluate the functional in FP32, the rest in FP64 (default 1e-5; +inf or
 * any value above every density keeps the whole functional in FP64).
 * v_operands: operands of the V_xc kernel, 1 split from FP32 inside the
 * kernel, 2 BF16 planes split beforehand in HBM (1.5x the AO store plus the
 * per-build R planes), 0 = 2 when that fits in half of the free memory.
 * Changing screen, fock_tiles, spatial or v_operands discards the prepared
 * tiles (rebuilt at the next build). */
typedef struct xc_mixed_config {
    double screen;
    int fock_tiles;
    int spatial;
    double func_float_above;
    int v_operands;
    int reserved;
} xc_mixed_config;
int xc_grid_set_mixed_config(xc_grid* g, const xc_mixed_config* cfg);
int xc_grid_get_mixed_config(const xc_grid* g, xc_mixed_config* cfg);

/* Autotuner of the mixed path for one functional and a representative
 * density (host D, packed).  Reference: a build with screening 1e-14 and
 * spatial tiles.  Candidates over (screen, spatial, fock_tiles, and the
 * operand form when pre-split planes fit) are built
 * and timed (median of `reps` graph replays); the fastest candidate whose
 * energies (every molecule) are within e_tol and whose V is within v_tol
 * (max abs) of the reference is selected and left set on the grid.
 * report (may be NULL) receives the choice and the candidates tried. */
typedef struct xc_tune_candidate {
    xc_mixed_config cfg;
    double ms;          /* median build time */
    double max_de;      /* max over molecules of |E - E_ref| */
    double max_dv;      /* max |V - V_ref| */
    long kept_pairs;    /* sum over tiles of (kept functions)^2 */
    int accepted;
} xc_tune_candidate;
typedef struct xc_tune_report {
    xc_mixed_config best;
    double ms_best, ms_reference;
    int ncand;
    xc_tune_candidate cand[32];
} xc_tune_report;
int xc_grid_tune(xc_grid* g, xc_functional* f, const double* D, int nspin, double e_tol, double v_tol,
                 int reps, xc_tune_report* report);

#ifdef __cplusplus
}
#endif
#endif
