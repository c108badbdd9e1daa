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

#ifdef __cplusplus
}
#endif
#endif
