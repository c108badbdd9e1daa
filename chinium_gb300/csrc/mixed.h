// Mixed-precision path: point tiles with chunk screening, split-BF16 operand
// stores, TMA tensor maps and the launch wrappers of k_mixed.cu.
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
struct MixedDev {
    int ntiles;
    int nchunk;      // basis chunks of 64 functions
    int kmax;        // max kept functions per tile (multiple of 64)
    int npad;        // nchunk * 64
    long Gt;         // ntiles * 128
    const int* tile_nkept;   // [ntiles]
    const int* tile_chunks;  // [ntiles][nchunk] kept global chunk ids by slot
    const int* tile_slot;    // [ntiles][nchunk] slot of a global chunk, -1 if dropped
    const __nv_bfloat16* pf; // point-major AO planes
    const __nv_bfloat16* fp; // function-major AO planes
    const float* e32;        // function-major FP32 AO values [c][t][kmax][128] (epilogues)
};

struct MixedState {
    bool ready = false;
    double thr = 0;
    MixedDev md{};
    std::vector<int> h_nkept, h_chunks, h_slot;
    long kept_pairs = 0;  // sum over tiles of (64 * nkept)^2
    DevBuf<int> d_nkept, d_chunks, d_slot, d_tile_shells, d_tile_shell_off;
    DevBuf<double> d_shtab;
    DevBuf<__nv_bfloat16> d_pf, d_fp, d_R, d_Dp;
    DevBuf<float> d_e32;
    DevBuf<double> d_wpart;
    DevBuf<int> d_err;
    // incremental builds: references of the previous build and difference scratch
    bool have_ref = false;
    DevBuf<double> d_Dref, d_rho_ref, d_rho1_ref, d_tau_ref, d_fcoef_ref, d_Vref, d_dD, d_dfcoef;
    int r_ncomp = 0;
    int nblk = 0, nsplit = 0;
    CUtensorMap tm_pf, tm_d, tm_fp, tm_r;
};

size_t mixed_smem_bytes();
void launch_ao_mixed(const MixedDev& md, DevShells sh, const int* tile_shells, const int* tile_shell_off,
                     const double* x, const double* y, const double* z, long Gp, const double* shtab,
                     __nv_bfloat16* pf, __nv_bfloat16* fp, float* e32, cudaStream_t s);
void launch_split_d(const double* D, int n, int npad, int nspin, __nv_bfloat16* Dp, cudaStream_t s);
void launch_density_tc(const CUtensorMap& tm_pf, const CUtensorMap& tm_d, const MixedDev& md, int epi, int acomp,
                       int spin, double* rho, double* rho1, double* tau, long Gp, int* err, cudaStream_t s);
void launch_prep_r(const MixedDev& md, int ncomp, int type, const double* fcoef, long Gp, __nv_bfloat16* R,
                   cudaStream_t s);
// r_rows: first of the 64 zero rows of the R store (r_ncomp * 3 * ntiles * kmax).
void launch_fock_tc(const CUtensorMap& tm_fp, const CUtensorMap& tm_r, const MixedDev& md, int ncomp, int r_rows,
                    int nblk, int nsplit, double* wpart, int* err, cudaStream_t s);
void launch_wsum(const double* wpart, int nsplit, int npadw, int n, double* V, cudaStream_t s);
void launch_axpby(long n, double a, const double* x, double b, const double* y, double* out, cudaStream_t s);

// 2D bf16 tensor map with 128-byte swizzle over a row-major [rows][cols] array.
void make_tmap_bf16(CUtensorMap* map, const void* base, uint64_t cols, uint64_t rows, uint32_t box_cols,
                    uint32_t box_rows);

}  // namespace cgb
