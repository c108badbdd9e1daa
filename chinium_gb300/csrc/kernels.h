// Launch wrappers for the XC kernels (implemented in k_*.cu).  All take raw
// device pointers and a stream; none allocates.
#pragma once

#include <cuda_runtime.h>

#include "functional.cuh"
#include "model.h"

namespace cgb {

// Shells on the device (struct of arrays).
struct DevShells {
    int nshell;
    const int* type;
    const int* l;
    const int* nprim;
    const int* prim_off;
    const int* first;
    const double* xyz;  // nshell x 3
    const double* exps;
    const double* coefs;
};

// Upload the solid-harmonic table to constant memory (once per process/device).
void upload_solid_harmonics();

// Becke partition weights (GridGeneration.cpp:134-153), one thread per point.
void launch_becke(int natoms, const double* d_atoms, long npts, const double* x, const double* y,
                  const double* z, const int* owner, const double* w_in, double* w_out, cudaStream_t s);

// AO values (ncomp = 1) or values + gradients (ncomp = 4) for every block.
void launch_ao(int nblocks, const BlockDesc* d_blocks, const int* d_block_shells, DevShells sh,
               const double* x, const double* y, const double* z, int ncomp, double* ao, cudaStream_t s);

// rho (s, G), rho1 (s, 3, G) and tau (s, G) from D (s, n, n) column-major.
void launch_density_fp64(int nblocks, const BlockDesc* d_blocks, const int* d_basis_lists, int nbasis,
                         int nspin, int type, const double* D, const double* ao, long Gp, double* rho,
                         double* rho1, double* tau, cudaStream_t s);
// The same in float-float arithmetic on the FP32 pipe (~1e-14 relative), from
// D and the AO store split into float pairs by launch_split_ff: the
// incremental build's reference densities.
void launch_split_ff(long n, const double* src, float2* dst, cudaStream_t s);
void launch_density_ff(int nblocks, const BlockDesc* d_blocks, const int* d_basis_lists, int nbasis, int nspin,
                       int type, const float2* D, const float2* ao, long Gp, double* rho, double* rho1, double* tau,
                       cudaStream_t s);

// XC nuclear-gradient partials with the grid fixed (LDA / GGA): part[s][list entry][t]
// = -2 sum_g [d_t phi U + sum_r d_t d_r phi f_r T] for the block function at that list entry
// (AO store with Hessians for GGA: 10 components).
void launch_xc_grad(int nblocks, const BlockDesc* d_blocks, const int* d_lists, long nlist, int nbasis, int nspin,
                    int family, const double* D, const double* ao, long Gp, const double* fcoef, double* part,
                    cudaStream_t s);

// Functional on every point: eps, vrho, vsigma, vtau, sigma, the Fock
// coefficients fcoef (s, 5, G) and per-CTA partial energies.  Points whose
// total density is >= float_above are evaluated in FP32 (mixed path); the
// default keeps every point in FP64.
void launch_functional_fp64(const xcf::FuncDesc& f, int family, int nspin, long Gp, const double* w,
                            const double* rho, const double* rho1, const double* tau, double* sigma,
                            double* eps, double* vrho, double* vsigma, double* vtau, double* fcoef,
                            double* e_partial, int* n_partial, cudaStream_t s,
                            double float_above = __builtin_huge_val());

// Deterministic sum of n partials into out[0] (single CTA, fixed order).
void launch_reduce_sum(const double* partial, int n, double* out, cudaStream_t s);

// Number of electrons partials: sum_g w_g sum_s rho_gs.
void launch_num_electrons(long Gp, int nspin, const double* w, const double* rho, double* partial,
                          int* n_partial, cudaStream_t s);

// V (s, n, n) += per-block phi^T A + A^T phi (+ gradient terms), FP64 atomics.
void launch_fock_fp64(int nblocks, const BlockDesc* d_blocks, const int* d_basis_lists, int max_nb,
                      int nbasis, int nspin, int type, const double* ao, long Gp, const double* fcoef,
                      double* V, cudaStream_t s);

// SAP potential times weight into fcoef (s = 1, LDA layout): fcoef[0] = 1/2 w v_SAP.
void launch_sap_coef(long Gp, int natoms, const double* d_atoms, const double* d_table /* natoms x 751 */,
                     const double* d_radii, const double* x, const double* y, const double* z,
                     const double* w, double* fcoef, cudaStream_t s);

// Second derivatives of an LDA / GGA functional at the grid's density (rho, rho1):
// f2 (3 or 15, Gp), rows v2rho2, v2rhosigma, v2sigma2 in libxc's layouts.
void launch_fxc(const xcf::FuncDesc& f, int family, int nspin, long Gp, const double* rho, const double* rho1,
                double* f2, cudaStream_t s);
// The same on caller arrays (parity tests).
void launch_fxc_points(const xcf::FuncDesc& f, int family, int nspin, long n, const double* rho, const double* sigma,
                       double* v2rho2, double* v2rhosigma, double* v2sigma2, cudaStream_t s);
// out[q] = in[q]^T for nmat n x n matrices.
void launch_transpose_batch(int n, long nmat, const double* in, double* out, cudaStream_t s);
// Response V coefficients (layout of fcoef, one 5-row set per (spin, matrix) pair q = s nmat + m)
// from the ground-state gradients and vsigma, f2 and the response densities rhoU (q, Gp), rho1U (q, 3, Gp).
void launch_response_coef(int family, int nspin, long Gp, int nmat, const double* w, const double* rho1,
                          const double* vsigma, const double* f2, const double* rhoU, const double* rho1U,
                          double* fcoefU, cudaStream_t s);

// Hessian skeleton terms (grid fixed, LDA / GGA; AO store with Hessians): the skeleton density
// derivatives rhog (q, Gp) and rho1g (q, 3, Gp), accumulated (zero them first), and the skeleton
// Fock derivatives F (q, n, n), accumulated, for q = s nmat + 3 A + t with the atom of every list
// entry in d_atom_list.
void launch_skel_density(int nblocks, const BlockDesc* d_blocks, const int* d_lists, const int* d_atom_list,
                         int nbasis, int nspin, int nmat, int family, const double* D, const double* ao, long Gp,
                         double* rhog, double* rho1g, cudaStream_t s);
void launch_fock_skel(int nblocks, const BlockDesc* d_blocks, const int* d_lists, const int* d_atom_list,
                      int max_nb, int nbasis, int nspin, int nmat, int family, const double* ao, long Gp,
                      const double* fcoef, double* F, cudaStream_t s);

// Pointwise functional on caller arrays (parity tests).
void launch_functional_points(const xcf::FuncDesc& f, int family, int nspin, long n, const double* rho,
                              const double* sigma, const double* tau, double* eps, double* vrho,
                              double* vsigma, double* vtau, cudaStream_t s);

}  // namespace cgb
