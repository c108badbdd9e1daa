/*
 * chinium_int.h -- Gaussian integrals for the SCF caller of the XC build.
 *
 * The reference's SCF obtains these from libint2 through Int2C1E
 * (src/Integral/Int2C1E.cpp:313, CalculateIntegrals: Overlap, Kinetic,
 * Nuclear) and Int4C2E (src/Integral/Int4C2E.cpp:601-683, in-core repulsion
 * integrals contracted into J and K).  These entry points provide the same
 * matrices over an xc_basis (same functions, order and normalisation as the
 * grid), computed on the host with OpenMP.  Status codes as in chinium_xc.h.
 */
#ifndef CHINIUM_INT_H
#define CHINIUM_INT_H

#include "chinium_xc.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Overlap, kinetic and nuclear-attraction matrices, n x n each (symmetric;
 * the layout is the same in row and column order). */
int xc_int1e(const xc_basis* b, double* S, double* T, double* V);

/* Dipole integrals <mu| r_k - C_k |nu> for k = x, y, z about the origin C
 * (3 doubles, bohr): M holds three symmetric n x n matrices, x first (the
 * position operator itself; the electronic dipole is minus its trace with
 * D).  The reference's counterpart is the dipole part of its libint2
 * multipole call (Int2C1E.cpp:313-324, DipoleX/Y/Z); here they serve the
 * coupled-perturbed electric-field response. */
int xc_dipole(const xc_basis* b, const double* origin, double* M);

/* All electron-repulsion integrals (mu nu | lambda sigma) as an n^4 array,
 * element ((mu*n + nu)*n + lambda)*n + sigma.  Shell quartets whose Schwarz
 * bound is below schwarz_threshold are left zero. */
int xc_eri(const xc_basis* b, double* eri, double schwarz_threshold);

/* --------------------------------------------- Coulomb and exchange (GPU)
 * The reference's Int4C2E (src/Integral/Int4C2E.cpp) on the GPU: Schwarz
 * bounds from the diagonal integrals (getRepulsionDiag, :19-77), the
 * screened list of unique shell quartets (getRepulsionLength /
 * getRepulsionIndices, :79-130), the integrals themselves
 * (CalculateIntegrals, :567-584; McMurchie-Davidson in FP64 here, s to f
 * shells) and their contraction with density matrices every SCF iteration
 * (ContractInts / Gunified, :601-683).  Quartets whose Schwarz product is
 * below `threshold` are dropped (the reference's SCF keeps all of them,
 * threshold -1 at SelfConsistentField.cpp:47; 0 does the same here).  The
 * integrals are computed once and kept in HBM when they take at most
 * max_bytes (0: half of the free device memory); otherwise every build
 * recomputes them in chunks (integral-direct).  Kept integrals of a small
 * molecule also fill a dense Coulomb operator over function pairs when it
 * fits in the same budget and a quarter of the free memory.  In-core builds
 * contract in float-float arithmetic (FP64 integrals and densities held as
 * pairs of floats, 48 significant bits, sums of products on the FP32 pipe;
 * J and K agree with FP64 contractions to ~1e-13 relative) when the shell
 * quartets average at least 24 integrals (basis sets with d and f shells)
 * and one matrix's exchange rows of the largest shell pair fit in shared
 * memory (n up to ~1800 functions with f shells); other builds run in FP64. */
typedef struct xc_jk xc_jk;
int xc_jk_create(const xc_basis* b, double threshold, double max_bytes, xc_jk** out);
int xc_jk_destroy(xc_jk* jk);
/* Quartets and integrals kept, and 1 if the integrals are resident in HBM. */
int xc_jk_info(const xc_jk* jk, long long* nquartets, long long* nints, int* incore);
/* CUDA stream (cudaStream_t as void*) of the builds; NULL = legacy default. */
int xc_jk_set_stream(xc_jk* jk, void* stream);
/* J_m = sum (mu nu|la si) D_m(la, si) and K_m = sum (mu la|nu si) D_m(la, si)
 * for nmat symmetric n x n density matrices (host buffers); J or K may be
 * NULL.  Gunified returns J of the total density and K per spin; a caller
 * forms those from J_m and K_m. */
int xc_jk_build(xc_jk* jk, int nmat, const double* D, double* J, double* K);
/* Same on caller-owned device buffers, issued on the handle's stream
 * without synchronising. */
int xc_jk_build_device(xc_jk* jk, int nmat, const double* d_D, double* d_J, double* d_K);

#ifdef __cplusplus
}
#endif
#endif
