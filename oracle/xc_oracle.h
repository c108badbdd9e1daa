/*
 * ORACLE -- test infrastructure only.  A CPU FP64 restatement of Chinium's
 * Kohn-Sham XC build (src/Grid + src/ExchangeCorrelation.cpp).  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it; the
 * product never links or calls it.
 *
 * Parity status: the grid, AO, density, energy and Fock stages restate the
 * reference line by line (citations per function).  The functional stage
 * restates libxc's published functionals (libxc is absent; the reference
 * points at the libxc 6.2.2 list, DensityFunctionals/README.md:1): parity
 * with libxc is unpinned.  The reference ships no golden XC vectors.
 *
 * Layouts follow the reference: per block, AO(g, mu) column-major with g
 * fastest, AO1(g, mu, r), Rho(g, s), Rho1(g, r, s), Sigma(g, s(s+1)/2),
 * Tau(g, s); matrices n x n column-major.
 */
#ifndef XC_ORACLE_H
#define XC_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Becke-partitioned weights of raw atom-centred points.
 * GridGeneration.cpp:134-153 with s_p_mu at :50-71.  owner[k] is the atom
 * whose sphere generated point k; w_in is radial*Lebedev*4pi weight. */
void oracle_becke(int natoms, const double* atom_xyz, long npts, const double* px,
                  const double* py, const double* pz, const int* owner, const double* w_in,
                  double* w_out);

/* AO values (deriv=0) or values+gradients (deriv=1) for one block of points.
 * GridAO.cpp:14-215 (radial part, product rule) and AO/{S,CartP,PureP,PureD,
 * PureF,PureG}.hpp (angular part).  Shell arrays: shell_type uses the
 * reference's convention (0 S, 1 Cartesian P, -1 pure P, -l pure l>=2).
 * Output: ao[mu*ng + g]; ao1[(r*nbasis + mu)*ng + g]. */
void oracle_ao(int nshells, const int* shell_type, const int* shell_nprim,
               const int* shell_prim_off, const double* shell_center, const double* exps,
               const double* coefs, int nbasis, int ng, const double* x, const double* y,
               const double* z, int deriv, double* ao, double* ao1);

/* rho, grad rho (x2), sigma, tau (x1/2) for one block.  GridDensity.cpp:12-41
 * with the Rho / Rho1 / Sigma / Tau einsums, loop order kept. D is (n,n,s). */
void oracle_density(int ng, int nbasis, int nspin, int type, const double* D, const double* ao,
                    const double* ao1, double* rho, double* rho1, double* sigma, double* tau);

/* Sum over functional ids of eps, vrho, vsigma, vtau on ng points
 * (ExchangeCorrelation.cpp:165-248, order "ev").  Inputs/outputs use the
 * reference's per-block layout (g fastest).  Returns 0, or -1 on an unknown id. */
int oracle_functional(int nids, const int* ids, int nspin, int ng, const double* rho,
                      const double* sigma, const double* tau, double* eps, double* vrho,
                      double* vsigma, double* vtau);

/* Per-block E_xc contribution, GridEnergy.cpp:11-13 einsum W,Rho,Eps->E. */
double oracle_energy(int ng, int nspin, const double* w, const double* rho, const double* eps);

/* Per-block V_xc accumulated into F (n,n,s) through basis_list.
 * GridFock.cpp:11-49 with the F0 / F1 / F2 einsums; lapl terms are zero for
 * the laplacian-free functionals served here. */
void oracle_fock(int ng, int nbasis_block, int nbasis_total, const int* basis_list, int nspin,
                 int type, const double* w, const double* ao, const double* ao1,
                 const double* rho1, const double* vrho, const double* vsigma,
                 const double* vtau, double* F);

/* SAP potential on points (GuessSCF.cpp:38-57): sum over atoms of the
 * nearest-radius tabulated value divided by r (r += 1e-12). */
void oracle_sap(int natoms, const double* atom_xyz, const double* atom_table /* natoms x 751 */,
                const double* radii, int nradii, long npts, const double* px, const double* py,
                const double* pz, double* v);

/* Whole build over a list of blocks (density -> functional -> energy ->
 * Fock), OpenMP over blocks, mirroring Grid::getDensity / Evaluate /
 * getEnergy / getFock.  Used as the timed CPU baseline.  Blocks are given as
 * offsets into concatenated per-block arrays. */
int oracle_build(int nblocks, const int* blk_ng, const long* blk_pt_off, const long* blk_ao_off,
                 const double* w, const double* ao, const double* ao1, int nbasis, int nspin,
                 int type, const double* D, int nids, const int* ids, int nthreads,
                 double* E_out, double* F_out);

/* Second derivatives of an LDA / GGA functional (order "f",
 * ExchangeCorrelation.cpp:101-133) on ng points: v2rho2 (1 or 3, ng),
 * v2rhosigma (1 or 6, ng), v2sigma2 (1 or 6, ng) in libxc's layouts
 * (rho_a rho_a, rho_a rho_b, rho_b rho_b; rho_w sigma_x at 3 w + x; upper
 * triangle of sigma_aa, sigma_ab, sigma_bb).  Returns -1 for a meta-GGA or an
 * unknown id. */
int oracle_functional_fxc(int nids, const int* ids, int nspin, int ng, const double* rho,
                          const double* sigma, double* v2rho2, double* v2rhosigma, double* v2sigma2);

/* Response densities of one block (GridDensity.cpp:47-77): D_U (n,n,nmat,s)
 * -> RhoU (g,mat,s), Rho1U (g,r,mat,s), SigmaU (g,mat,uv); rho1 is the
 * ground-state Rho1 (g,r,s). */
void oracle_density_u(int ng, int nbasis, int nspin, int nmat, int type, const double* DU,
                      const double* ao, const double* ao1, const double* rho1, double* rhoU,
                      double* rho1U, double* sigmaU);

/* Response V_xc of one block accumulated into F (ntot,ntot,nmat,s) through
 * basis_list (GridFock.cpp:97-160, getFockU<u_t>), from the ground-state Rho1
 * and vsigma, the second derivatives (layouts of oracle_functional_fxc) and
 * the response densities of oracle_density_u. */
void oracle_fock_u(int ng, int nbasis_block, int nbasis_total, const int* basis_list, int nspin,
                   int nmat, int type, const double* w, const double* ao, const double* ao1,
                   const double* rho1, const double* vsigma, const double* v2rho2,
                   const double* v2rhosigma, const double* v2sigma2, const double* rhoU,
                   const double* rho1U, const double* sigmaU, double* F);

/* AO second derivatives of one block: ao2[(c * nbasis + mu) * ng + g] with c = xx, xy, yy, xz,
 * yz, zz (the packing of SubGrid::AO2, GridAO.cpp:254-259). */
void oracle_ao2(int nshells, const int* shell_type, const int* shell_nprim, const int* shell_prim_off,
                const double* shell_center, const double* exps, const double* coefs, int nbasis, int ng,
                const double* x, const double* y, const double* z, double* ao2);

/* Skeleton density derivatives of one block (GridDensity.cpp:79-130): RhoGrad (g,t,A,s),
 * Rho1Grad (g,r,t,A,s), SigmaGrad (g,t,A,uv) for the block functions' atoms atom_of[mu]. */
void oracle_density_skeleton(int ng, int nbasis, int nspin, int natoms, const int* atom_of, int type,
                             const double* D, const double* ao, const double* ao1, const double* ao2,
                             const double* rho1, double* rhog, double* rho1g, double* sigmag);

/* Skeleton Fock derivatives of one block accumulated into F (ntot,ntot,3,natoms,s)
 * (GridFock.cpp:52-95, getFockSkeleton). */
void oracle_fock_skeleton(int ng, int nbasis_block, int nbasis_total, const int* basis_list, int nspin,
                          int natoms, const int* atom_of, int type, const double* w, const double* ao,
                          const double* ao1, const double* ao2, const double* rho1, const double* vrho,
                          const double* vsigma, double* F);

/* AO third derivatives of one block: ao3[(c * nbasis + mu) * ng + g], c the packed sorted triple
 * i0 + i1 (i1 + 1) / 2 + i2 (i2 + 1) (i2 + 2) / 6. */
void oracle_ao3(int nshells, const int* shell_type, const int* shell_nprim, const int* shell_prim_off,
                const double* shell_center, const double* exps, const double* coefs, int nbasis, int ng,
                const double* x, const double* y, const double* z, double* ao3);

/* XC skeleton energy Hessian of one block, restricted (GridDensity.cpp:132-212, GridEnergy.cpp:32-46),
 * added to E (3 natoms x 3 natoms, column-major, index 3 a + t). */
void oracle_energy_hess(int ng, int nbasis, int natoms, const int* atom_of, int type, const double* D,
                        const double* w, const double* ao, const double* ao1, const double* ao2,
                        const double* ao3, const double* rho1, const double* vrho, const double* vsigma,
                        const double* v2rho2, const double* v2rhosigma, const double* v2sigma2,
                        const double* rhog, const double* rho1g, const double* sigmag, double* E);

/* The response V_U of nmat matrices over a list of blocks (layouts as oracle_build; D_U
 * (n,n,nmat,s) column-major), OpenMP over blocks: the timed CPU baseline of the response. */
int oracle_build_response(int nblocks, const int* blk_ng, const long* blk_pt_off, const long* blk_ao_off,
                          const double* w, const double* ao, const double* ao1, int nbasis, int nspin,
                          int type, const double* D, int nmat, const double* DU, int nids, const int* ids,
                          int nthreads, double* F_out);

#ifdef __cplusplus
}
#endif
#endif
