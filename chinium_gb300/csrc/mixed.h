// Mixed-precision path: point tiles of one or many molecules, chunk
// screening, the FP32 AO store, persistent work lists, and the launch
// wrappers of k_mixed.cu.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>

#include <vector>

#include "common.h"
#include "kernels.h"

namespace cgb {

constexpr int kChunk = 64;     // functions per chunk (MMA K / N granularity)
constexpr int kTilePts = 128;  // points per tile (MMA M)

// Device view of the tile structure (passed by value to kernels).
//   e32 / Z rows: component c, row tile_row[t] + slot*64 + f, 128 points per row.
//   Dp: plane (s*3 + p), row f0(mol) + nu, column mu (local functions).
struct MixedDev {
    int ntiles;
    int nchunk;              // stride of tile_chunks / tile_slot (max chunks of one molecule)
    long Gt;                 // ntiles * 128 points
    long rows;               // kept function rows of all tiles (component stride of e32)
    long drows;              // rows of one density plane (sum of the molecules' padded functions)
    const int* tile_nkept;   // [ntiles]
    const int* tile_chunks;  // [ntiles][nchunk] kept local chunk ids by slot
    const int* tile_slot;    // [ntiles][nchunk] slot of a local chunk, -1 if dropped
    const long* tile_row;    // [ntiles] first row of the tile
    const int* tile_c0;      // [ntiles] first chunk of the tile's molecule in the combined numbering
    const float* e32;        // FP32 AO store [c][rows][128]: phi, d/dx, d/dy, d/dz
};

// One molecule of a (batched) mixed build.
struct MolRange {
    int n = 0;          // basis functions
    int f0 = 0;         // first function in the combined, 64-aligned numbering
    int nchunk = 0;     // 64-function chunks
    int nblk = 0;       // 128-function blocks of V
    int sh0 = 0, sh1 = 0;  // shells of the combined basis
    int t0 = 0, t1 = 0;    // tiles
    long voff = 0;      // offset of the (nspin, n, n) block in packed D / V
    long item0 = 0;     // first V work item
    int nsplit = 0;     // tile splits of each (I, J) block
};

// V work item: W_IJ partial over the wanted tiles of [t0, t1) of one molecule.
struct FockItem {
    int I, J, t0, t1;
};

// One tile of a CTA's density work list.
struct DensJob {
    int t, nk, trow, c0;
};

// One (item, wanted tile) of a CTA's V work list: slots of chunks 2I, 2I+1,
// 2J, 2J+1 (-1 if dropped); flags 1: first tile of the item, 2: last,
// 4: the item carries the meta-GGA components (I <= J), 8: with c2 doubled
// (I < J).
struct FockJob {
    int t, trow, sa0, sa1, sb0, sb1, item, flags;
};

// Tuning knobs of the mixed path (chosen by the autotuner or set directly).
struct MixedConfig {
    double screen = 1e-11;   // chunk screening threshold (|phi|, |grad phi| bound)
    int fock_tiles = 0;      // tiles per V work item (0: from the SM count)
    int spatial = 1;         // 1: tiles from a k-d split of each molecule's points; 0: generation order
    double func_float_above = 1e-5;  // FP32 functional at points with total density >= this
    int v_operands = 0;      // V kernel operands: 0 auto (by free memory), 1 converted in-kernel, 2 pre-split
    bool same_tiles(const MixedConfig& o) const {
        return screen == o.screen && fock_tiles == o.fock_tiles && spatial == o.spatial &&
               v_operands == o.v_operands;
    }
};

struct MixedState {
    bool ready = false;
    MixedConfig cfg;
    MixedDev md{};
    std::vector<MolRange> mols;
    int nspin = 1;
    int dcols = 0;           // columns of a density plane (max padded functions of a molecule)
    int ao_comp = 1;         // components in e32 (1 or 4)
    long real_points = 0;
    std::vector<int> h_nkept, h_chunks, h_slot;
    std::vector<long> h_row;
    long kept_pairs = 0;     // sum over tiles of (64 * nkept)^2
    long units_full = 0, units_sym = 0, fock_jobs = 0, fock_tau_jobs = 0, live_items = 0;
    long empty_tiles = 0;    // tiles that keep no chunk: no density job writes their points
    // work lists (CSR by CTA)
    int dens_ctas = 0, fock_ctas = 0;
    long nitems = 0;
    DevBuf<int> d_nkept, d_chunks, d_slot, d_c0, d_tile_shells, d_tile_shell_off;
    DevBuf<long> d_row;
    DevBuf<int> d_dens_off, d_fock_off, d_item_live;
    DevBuf<DensJob> d_dens_jobs;
    DevBuf<FockJob> d_fock_jobs;
    DevBuf<MolRange> d_mols;
    DevBuf<double> d_shtab;
    DevBuf<double> d_x, d_y, d_z, d_w;   // tile-ordered points (zero weight on padding)
    DevBuf<long> d_perm;                 // FP64-array index of each tile point; -(i+1) on padding
    bool have_perm = false;
    DevBuf<float> d_e32, d_Z, d_c2;
    bool use16 = false;                  // V kernel on pre-split planes
    DevBuf<__nv_bfloat16> d_e16, d_R16;  // AO store planes [c][p][rows][128]; R planes [c][p][rows][128]
    DevBuf<__nv_bfloat16> d_e16d;        // density A planes [c][p][rows][128], fixed point per (point, slot)
    DevBuf<__nv_bfloat16> d_Dp;
    DevBuf<double> d_wpart;
    DevBuf<int> d_err;
    // per-point work arrays of the mixed build (tile order)
    DevBuf<double> rho, rho1, tau, sigma, eps, vrho, vsigma, vtau, fcoef, partial;
    DevBuf<double> rho_b, rho1_b, tau_b;  // column-half-1 partials of the density kernel
    int n_partial = 0;
    // incremental builds: references of the previous build and difference scratch
    bool have_ref = false;
    DevBuf<double> d_Dref, d_rho_ref, d_rho1_ref, d_tau_ref, d_fcoef_ref, d_Vref, d_dD, d_dfcoef;
    CUtensorMap tm_d;                      // density planes, box 64 x 64
    CUtensorMap tm_raw_d;                  // e32, box 128 points x 64 rows (density A tiles)
    CUtensorMap tm_raw_f;                  // e32, box 32 points x 64 rows (V_xc L / R boxes)
    CUtensorMap tm_z;                      // Z, box 32 points x 64 rows
    CUtensorMap tm_e16, tm_r16;            // BF16 planes of e16 / R16, box 64 points x 64 rows
    CUtensorMap tm_e16d;                   // BF16 planes of e16d, box 64 points x 64 rows
    // CUDA graph of one build (replayed while the functional and buffers are unchanged)
    cudaGraphExec_t graph = nullptr;
    std::vector<int> graph_ids;  // functional (libxc ids) and grid type the graph was captured for
    int graph_type = -1;
    ~MixedState();
    void drop_graph();
};

size_t mixed_smem_bytes();
void launch_ao_mixed(const MixedDev& md, DevShells sh, const int* tile_shells, const int* tile_shell_off,
                     const double* x, const double* y, const double* z, const double* shtab, int ao_comp, float* e32,
                     cudaStream_t s);
// Packed per-molecule D (s, n, n) -> three BF16 planes per spin of the density strip.
void launch_split_d(const double* D, const MolRange* mols, int nmol, int nspin, long drows, int dcols, int maxn,
                    __nv_bfloat16* Dp, cudaStream_t s);
// Writes the column-half-0 partials to rho / rho1 / tau and the half-1
// partials to rho_b / rho1_b / tau_b (tau and tau_b accumulate: zero them
// before the first meta-GGA pass); launch_combine adds them.
void launch_density_tc(const CUtensorMap& tm_d, const CUtensorMap& tm_raw, const MixedDev& md, int ctas,
                       const int* job_off, const DensJob* jobs, int epi, int acomp, int spin, double* rho,
                       double* rho1, double* tau, double* rho_b, double* rho1_b, double* tau_b, int* err,
                       cudaStream_t s);
// The same on the pre-split AO planes (tm_e16: A operand MN-major, no conversion).
void launch_density16(const CUtensorMap& tm_d, const CUtensorMap& tm_e16, const MixedDev& md, int ctas,
                      const int* job_off, const DensJob* jobs, int epi, int acomp, int spin, double* rho,
                      double* rho1, double* tau, double* rho_b, double* rho1_b, double* tau_b, int* err,
                      cudaStream_t s);
void launch_combine(long n1, double* rho, const double* rho_b, double* rho1, const double* rho1_b, double* tau,
                    const double* tau_b, int type, cudaStream_t s);
// Z = c0 phi + c1 . grad phi (FP32, e32 row layout) and c2 per point (meta-GGA).
void launch_prep_z(const MixedDev& md, int type, const double* fcoef, float* Z, float* c2, cudaStream_t s);
void launch_fock_tc(const CUtensorMap& tm_e32, const CUtensorMap& tm_z, long rows, int ctas, const int* job_off,
                    const FockJob* jobs, const float* c2, int ncomp, double* wpart, int* err, cudaStream_t s);
// FP32 store (ncomp planes of n) -> BF16 planes e16[(c * 3 + p) * n + i].
void launch_split_store(const float* e32, long n, int ncomp, __nv_bfloat16* e16, cudaStream_t s);
// Components 0..ncomp-1 of the FP32 store (rows x 128 each) -> the density
// kernel's A planes, one fixed-point exponent per (point, 64-row slot).
void launch_split_store_fixed(const float* e32, long rows, int ncomp, __nv_bfloat16* e16d, cudaStream_t s);
// R planes of the pre-split V kernel: Z (component 0) and c2 d_c phi (1-3, meta-GGA).
void launch_prep16(const MixedDev& md, int type, const double* fcoef, __nv_bfloat16* R16, cudaStream_t s);
void launch_fock16(const CUtensorMap& tm_l, const CUtensorMap& tm_r, long rows, int ctas, const int* job_off,
                   const FockJob* jobs, int ncomp, double* wpart, int* err, cudaStream_t s);
// V_m(mu, nu) = sum over splits of W(mu, nu) + W(nu, mu), packed per molecule.
void launch_wsum(const double* wpart, const int* item_live, const MolRange* mols, int nmol, int maxn, int nspin_index,
                 int nspin, double* V, cudaStream_t s);
// E_m = sum of the functional's per-tile partials over the molecule's tiles.
void launch_energy_mols(const double* partial, const MolRange* mols, int nmol, double* E, cudaStream_t s);
void launch_axpby(long n, double a, const double* x, double b, const double* y, double* out, cudaStream_t s);
// dst[p] = src[perm[p]] for every tile point (ncomp planes of Gt / Gp);
// zero_pads: padding points get 0 instead.
void launch_gather(const long* perm, long Gt, long Gp, int ncomp, const double* src, double* dst, bool zero_pads,
                   cudaStream_t s);
void set_mixed_kernel_attributes();
// One CTA that waits on an mbarrier nothing arrives on for budget_ms, then
// records XC_ERR_TIMEOUT in err and unwinds (the pipelines' failure path).
void launch_wait_probe(double budget_ms, int* err, cudaStream_t s);

// 2D bf16 tensor map with 128-byte swizzle over a row-major [rows][cols] array.
void make_tmap_bf16(CUtensorMap* map, const void* base, uint64_t cols, uint64_t rows, uint32_t box_cols,
                    uint32_t box_rows);
// 2D FP32 tensor map without swizzle over a row-major [rows][cols] array.
void make_tmap_f32(CUtensorMap* map, const void* base, uint64_t cols, uint64_t rows, uint32_t box_cols,
                   uint32_t box_rows);

// Tensor-core GEMM of the pair MLP (k_tcgemm.cu).  Operands are BF16 planes,
// K-major, rows padded by tc_pad_rows and K by tc_pad_k; 1 or 3 planes each.
int tc_pad_rows(int n);
int tc_pad_k(int n);
// dst planes (nplanes x pad(rows) x pad(kdim)) of src(r, k) = src[r*ld_r + k*ld_k]; pads are 0.
void tc_to_planes(const float* src, int rows, int kdim, long ld_r, long ld_k, int nplanes, __nv_bfloat16* dst,
                  cudaStream_t s);
// C[m*ldc + n] (+)= sum_k A(m, k) B(n, k) [+ bias[n]] for m < M, n < N; a
// timed-out wait records XC_ERR_TIMEOUT in err.
void tc_gemm(const __nv_bfloat16* A, int npa, const __nv_bfloat16* B, int npb, int M, int N, int K, const float* bias,
             float* C, int ldc, bool accumulate, int* err, cudaStream_t s);

}  // namespace cgb
