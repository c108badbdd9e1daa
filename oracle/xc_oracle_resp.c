/*
 * ORACLE -- test infrastructure only (see xc_oracle.h).
 *
 * Response (coupled-perturbed) densities and V_xc of one block, restating
 * SubGrid::getDensityU (src/Grid/GridDensity.cpp:47-77) and
 * SubGrid::getFockU<u_t> (src/Grid/GridFock.cpp:97-160) with their einsums,
 * loop order kept.  Layouts follow the reference's tensors (g fastest):
 * D_U (mu, nu, mat, s), RhoU (g, mat, s), Rho1U (g, r, mat, s),
 * SigmaU (g, mat, uv) with uv = u + v (v + 1) / 2 for u <= v.
 */
#include <stdlib.h>
#include <string.h>

#include "xc_oracle.h"

void oracle_density_u(int ng, int nb, int ns, int nmat, int type, const double* DU, const double* ao,
                      const double* ao1, const double* rho1, double* rhoU, double* rho1U, double* sigmaU) {
    double* tmp = (double*)malloc(sizeof(double) * ng);
    const long nn = (long)nb * nb;
    /* D(mu,nu,mat,w) AO(g,mu) AO(g,nu) -> RhoU(g,mat,w) (GridDensity.cpp:61-64) */
    memset(rhoU, 0, sizeof(double) * ng * nmat * ns);
    for (int w = 0; w < ns; w++)
        for (int m = 0; m < nmat; m++) {
            const double* D = DU + ((long)w * nmat + m) * nn;
            double* o = rhoU + ((long)w * nmat + m) * ng;
            for (int nu = 0; nu < nb; nu++) {
                memset(tmp, 0, sizeof(double) * ng);
                for (int mu = 0; mu < nb; mu++) {
                    const double d = D[(long)nu * nb + mu];
                    const double* a = ao + (long)mu * ng;
                    for (int g = 0; g < ng; g++) tmp[g] += d * a[g];
                }
                const double* a = ao + (long)nu * ng;
                for (int g = 0; g < ng; g++) o[g] += tmp[g] * a[g];
            }
        }
    if (type >= 1) {
        /* D(mu,nu,mat,w) AO1(g,mu,r) AO(g,nu) -> Rho1U(g,r,mat,w), x2 (:65-68) */
        memset(rho1U, 0, sizeof(double) * ng * 3 * nmat * ns);
        for (int w = 0; w < ns; w++)
            for (int m = 0; m < nmat; m++) {
                const double* D = DU + ((long)w * nmat + m) * nn;
                for (int r = 0; r < 3; r++) {
                    double* o = rho1U + (((long)w * nmat + m) * 3 + r) * ng;
                    for (int nu = 0; nu < nb; nu++) {
                        memset(tmp, 0, sizeof(double) * ng);
                        for (int mu = 0; mu < nb; mu++) {
                            const double d = D[(long)nu * nb + mu];
                            const double* a = ao1 + ((long)r * nb + mu) * ng;
                            for (int g = 0; g < ng; g++) tmp[g] += d * a[g];
                        }
                        const double* a = ao + (long)nu * ng;
                        for (int g = 0; g < ng; g++) o[g] += tmp[g] * a[g];
                    }
                    for (int g = 0; g < ng; g++) o[g] *= 2;
                }
            }
        /* TMP(g,mat,u,v) = Rho1U(g,r,mat,u) Rho1(g,r,v); TMP += TMP^(u,v);
         * SigmaU(g,mat,uv) = TMP(g,mat,u,v) for u <= v (:69-75) */
        memset(sigmaU, 0, sizeof(double) * ng * nmat * (ns * (ns + 1) / 2));
        for (int v = 0; v < ns; v++)
            for (int u = 0; u <= v; u++) {
                const int uv = u + v * (v + 1) / 2;
                for (int m = 0; m < nmat; m++) {
                    double* o = sigmaU + ((long)uv * nmat + m) * ng;
                    for (int r = 0; r < 3; r++) {
                        const double* aU = rho1U + (((long)u * nmat + m) * 3 + r) * ng;
                        const double* bU = rho1U + (((long)v * nmat + m) * 3 + r) * ng;
                        const double* a = rho1 + ((long)u * 3 + r) * ng;
                        const double* b = rho1 + ((long)v * 3 + r) * ng;
                        for (int g = 0; g < ng; g++) o[g] += aU[g] * b[g] + bU[g] * a[g];
                    }
                }
            }
    }
    free(tmp);
}

/* Second derivatives in libxc's layouts ([k][g]) expanded to the tensors of
 * SubGrid: Eps2Rho2(g,u,v), Eps2RhoSigma(g,w,x), Eps2Sigma2(g,x,y). */
static double f_rr(const double* v2rho2, int ns, int ng, int u, int v, int g) {
    return ns == 1 ? v2rho2[g] : v2rho2[(long)(u + v) * ng + g];
}
static double f_rs(const double* v2rhosigma, int ns, int ng, int w, int x, int g) {
    return ns == 1 ? v2rhosigma[g] : v2rhosigma[(long)(3 * w + x) * ng + g];
}
static double f_ss(const double* v2sigma2, int ns, int ng, int x, int y, int g) {
    if (ns == 1) return v2sigma2[g];
    const int a = x < y ? x : y, b = x < y ? y : x;
    return v2sigma2[(long)(a * 3 - a * (a - 1) / 2 + b - a) * ng + g];
}

void oracle_fock_u(int ng, int nb, int ntot, const int* list, int ns, int nmat, int type, const double* w,
                   const double* ao, const double* ao1, const double* rho1, const double* vsigma,
                   const double* v2rho2, const double* v2rhosigma, const double* v2sigma2, const double* rhoU,
                   const double* rho1U, const double* sigmaU, double* Fout) {
    const int nsig = ns * (ns + 1) / 2;
    const long nn = (long)nb * nb;
    double* F = (double*)calloc((size_t)nn * nmat * ns, sizeof(double));
    double* tmp = (double*)malloc(sizeof(double) * ng);
    double* t1 = (double*)malloc(sizeof(double) * ng);
    /* TMP0(g,mat,u) = Eps2Rho2(g,u,v) RhoU(g,mat,v) + Eps2RhoSigma(g,u,x) SigmaU(g,mat,x);
     * TMP1 = W TMP0; F0 = TMP1 AO AO; F += 0.5 F0 (GridFock.cpp:117-128) */
    for (int u = 0; u < ns; u++)
        for (int m = 0; m < nmat; m++) {
            for (int g = 0; g < ng; g++) {
                double t = 0;
                for (int v = 0; v < ns; v++) t += f_rr(v2rho2, ns, ng, u, v, g) * rhoU[((long)v * nmat + m) * ng + g];
                if (type >= 1)
                    for (int x = 0; x < nsig; x++)
                        t += f_rs(v2rhosigma, ns, ng, u, x, g) * sigmaU[((long)x * nmat + m) * ng + g];
                t1[g] = w[g] * t;
            }
            double* Fm = F + ((long)u * nmat + m) * nn;
            for (int mu = 0; mu < nb; mu++) {
                for (int g = 0; g < ng; g++) tmp[g] = t1[g] * ao[(long)mu * ng + g];
                for (int nu = 0; nu < nb; nu++) {
                    double acc = 0;
                    for (int g = 0; g < ng; g++) acc += tmp[g] * ao[(long)nu * ng + g];
                    Fm[(long)nu * nb + mu] += 0.5 * acc;
                }
            }
        }
    if (type >= 1) {
        /* TMP1(g,mat,uv) = S_uv [Eps2RhoSigma(g,w,uv) RhoU(g,mat,w) + Eps2Sigma2(g,uv,x) SigmaU(g,mat,x)]
         * TMP2(g,r,mat,u) = TMP1(g,mat,u+v) Rho1(g,r,v)
         * TMP3(g,r,mat,u) = S_(u+v) Eps1Sigma(g,u+v) Rho1U(g,r,mat,v)
         * F1(mu,nu,mat,u) = W (TMP2 + TMP3)(g,r,mat,u) AO1(g,mu,r) AO(g,nu) (:129-154).
         * S = 2 on the spin diagonal.  The reference scales the sigma-sigma
         * term on the contracted pair x (:136-138, 145); with one spin both are 2. */
        double* tm1 = (double*)malloc(sizeof(double) * ng * nsig);
        double* t4 = (double*)malloc(sizeof(double) * ng * 3);
        for (int m = 0; m < nmat; m++) {
            for (int uv = 0; uv < nsig; uv++) {
                const double S = (ns == 1 || uv != 1) ? 2.0 : 1.0;
                for (int g = 0; g < ng; g++) {
                    double t = 0;
                    for (int ww = 0; ww < ns; ww++)
                        t += f_rs(v2rhosigma, ns, ng, ww, uv, g) * rhoU[((long)ww * nmat + m) * ng + g];
                    for (int x = 0; x < nsig; x++)
                        t += f_ss(v2sigma2, ns, ng, uv, x, g) * sigmaU[((long)x * nmat + m) * ng + g];
                    tm1[(long)uv * ng + g] = S * t;
                }
            }
            for (int u = 0; u < ns; u++) {
                memset(t4, 0, sizeof(double) * ng * 3);
                for (int v = 0; v < ns; v++) {
                    const int lo = u < v ? u : v, hi = u < v ? v : u;
                    const int uv = lo + hi * (hi + 1) / 2;
                    const double S = (u == v) ? 2.0 : 1.0;
                    for (int r = 0; r < 3; r++)
                        for (int g = 0; g < ng; g++)
                            t4[r * ng + g] += tm1[(long)uv * ng + g] * rho1[((long)v * 3 + r) * ng + g] +
                                              S * vsigma[(long)uv * ng + g] *
                                                  rho1U[(((long)v * nmat + m) * 3 + r) * ng + g];
                }
                double* Fm = F + ((long)u * nmat + m) * nn;
                for (int mu = 0; mu < nb; mu++) {
                    memset(tmp, 0, sizeof(double) * ng);
                    for (int r = 0; r < 3; r++)
                        for (int g = 0; g < ng; g++) tmp[g] += w[g] * t4[r * ng + g] * ao1[((long)r * nb + mu) * ng + g];
                    for (int nu = 0; nu < nb; nu++) {
                        double acc = 0;
                        for (int g = 0; g < ng; g++) acc += tmp[g] * ao[(long)nu * ng + g];
                        Fm[(long)nu * nb + mu] += acc;
                    }
                }
            }
        }
        free(t4);
        free(tm1);
    }
    /* F += F^T (over mu, nu), scatter through BasisList (:155-160) */
    for (int s = 0; s < ns; s++)
        for (int m = 0; m < nmat; m++) {
            const double* Fm = F + ((long)s * nmat + m) * nn;
            double* O = Fout + ((long)s * nmat + m) * ntot * (long)ntot;
            for (int nu = 0; nu < nb; nu++)
                for (int mu = 0; mu < nb; mu++)
                    O[(long)list[nu] * ntot + list[mu]] += Fm[(long)nu * nb + mu] + Fm[(long)mu * nb + nu];
        }
    free(t1);
    free(tmp);
    free(F);
}

/* ----------------------------------------------------- Hessian skeleton terms */

#include <math.h>

/* Angular polynomials (the same restatement as xc_oracle.c's AO/ *.hpp tables)
 * evaluated through oracle_ao on single points: their first derivatives come
 * from the complex step there; here the second derivatives are
 * Richardson-extrapolated central differences of those first derivatives,
 * exact to rounding for polynomials of degree <= 4. */
void oracle_ao(int nshells, const int* shell_type, const int* shell_nprim, const int* shell_prim_off,
               const double* shell_center, const double* exps, const double* coefs, int nbasis, int ng,
               const double* x, const double* y, const double* z, int deriv, double* ao, double* ao1);

/* AO second derivatives ao2[(c * nbasis + mu) * ng + g], c = xx, xy, yy, xz, yz, zz (the packing
 * of SubGrid::AO2, GridAO.cpp:254-259; values as GridAO.cpp:185-196):
 *   d_a d_b phi = A_ab Q + A_a Q_b + A_b Q_a + A Q_ab,
 *   A = sum c e^(-alpha r^2), A_a = -2 x_a sum c alpha e, A_ab = 4 x_a x_b sum c alpha^2 e - 2 delta_ab sum c alpha e
 * (GridAO.cpp:113-135).  Q_a, Q_ab from oracle_ao on a unit radial part: a one-primitive shell with
 * exponent 0 and coefficient 1 gives phi = Q. */
void oracle_ao2(int nshells, const int* shell_type, const int* shell_nprim, const int* shell_prim_off,
                const double* shell_center, const double* exps, const double* coefs, int nbasis, int ng,
                const double* xs, const double* ys, const double* zs, double* ao2) {
    int ibasis = 0;
    const double zero_exp = 0.0, one_coef = 1.0;
    const int one_nprim = 1, zero_off = 0;
    double q[16], q1[48], qp[48], qm[48], qp2[48], qm2[48];
    for (int s = 0; s < nshells; s++) {
        const int type = shell_type[s];
        const double* e = exps + shell_prim_off[s];
        const double* c = coefs + shell_prim_off[s];
        const double* C = shell_center + 3 * s;
        const int size = type == 0 ? 1 : (type == 1 || type == -1) ? 3 : 2 * (-type) + 1;
        for (int k = 0; k < ng; k++) {
            const double r[3] = {xs[k] - C[0], ys[k] - C[1], zs[k] - C[2]};
            const double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
            double t0 = 0, t1 = 0, t2 = 0;
            for (int p = 0; p < shell_nprim[s]; p++) {
                const double t = c[p] * exp(-e[p] * r2);
                t0 += t;
                t1 += t * e[p];
                t2 += t * e[p] * e[p];
            }
            /* Q and grad Q at the point, shell centred at the origin */
            const double org[3] = {0, 0, 0};
            oracle_ao(1, &type, &one_nprim, &zero_off, org, &zero_exp, &one_coef, size, 1, &r[0], &r[1], &r[2], 1,
                      q, q1);
            double Qab[6][16];
            for (int b = 0; b < 3; b++) {
                const double h = 1e-2;
                double rp[3] = {r[0], r[1], r[2]}, rm[3] = {r[0], r[1], r[2]};
                double rp2[3] = {r[0], r[1], r[2]}, rm2[3] = {r[0], r[1], r[2]};
                rp[b] += h;
                rm[b] -= h;
                rp2[b] += 0.5 * h;
                rm2[b] -= 0.5 * h;
                double tq[16];
                oracle_ao(1, &type, &one_nprim, &zero_off, org, &zero_exp, &one_coef, size, 1, &rp[0], &rp[1], &rp[2],
                          1, tq, qp);
                oracle_ao(1, &type, &one_nprim, &zero_off, org, &zero_exp, &one_coef, size, 1, &rm[0], &rm[1], &rm[2],
                          1, tq, qm);
                oracle_ao(1, &type, &one_nprim, &zero_off, org, &zero_exp, &one_coef, size, 1, &rp2[0], &rp2[1],
                          &rp2[2], 1, tq, qp2);
                oracle_ao(1, &type, &one_nprim, &zero_off, org, &zero_exp, &one_coef, size, 1, &rm2[0], &rm2[1],
                          &rm2[2], 1, tq, qm2);
                for (int a = 0; a <= b; a++) {
                    const int pk = a + b * (b + 1) / 2;
                    for (int i = 0; i < size; i++) {
                        const double d1 = (qp[a * size + i] - qm[a * size + i]) / (2 * h);
                        const double d2 = (qp2[a * size + i] - qm2[a * size + i]) / h;
                        Qab[pk][i] = (4 * d2 - d1) / 3;
                    }
                }
            }
            for (int b = 0; b < 3; b++)
                for (int a = 0; a <= b; a++) {
                    const int pk = a + b * (b + 1) / 2;
                    const double Aa = -2 * r[a] * t1, Ab = -2 * r[b] * t1;
                    const double Aab = 4 * r[a] * r[b] * t2 - (a == b ? 2 * t1 : 0.0);
                    for (int i = 0; i < size; i++)
                        ao2[((long)pk * nbasis + ibasis + i) * ng + k] =
                            Aab * q[i] + Aa * q1[b * size + i] + Ab * q1[a * size + i] + t0 * Qab[pk][i];
                }
        }
        ibasis += size;
    }
}

static int pair_pack(int a, int b) {
    const int lo = a < b ? a : b, hi = a < b ? b : a;
    return lo + hi * (hi + 1) / 2;
}

/* SubGrid::getDensitySkeleton (GridDensity.cpp:79-130) for one block: D (n,n,s) column-major,
 * atom_of[mu] the atom of block function mu.  Outputs (g fastest):
 * RhoGrad (g,t,A,s), Rho1Grad (g,r,t,A,s), SigmaGrad (g,t,A,uv). */
void oracle_density_skeleton(int ng, int nb, int ns, int natoms, const int* atom_of, int type, const double* D,
                             const double* ao, const double* ao1, const double* ao2, const double* rho1,
                             double* rhog, double* rho1g, double* sigmag) {
    const long nn = (long)nb * nb;
    memset(rhog, 0, sizeof(double) * ng * 3 * natoms * ns);
    double* T = (double*)malloc(sizeof(double) * ng);
    /* RhoGrada(g,t,w) = -2 sum_(mu in A) sum_nu Da(mu,nu,w) AO1a(g,mu,t) AO(g,nu) (:90-101) */
    for (int w = 0; w < ns; w++)
        for (int mu = 0; mu < nb; mu++) {
            const int A = atom_of[mu];
            memset(T, 0, sizeof(double) * ng);
            for (int nu = 0; nu < nb; nu++) {
                const double d = D[(long)w * nn + (long)nu * nb + mu];
                for (int g = 0; g < ng; g++) T[g] += d * ao[(long)nu * ng + g];
            }
            for (int t = 0; t < 3; t++) {
                double* o = rhog + (((long)w * natoms + A) * 3 + t) * ng;
                const double* a1 = ao1 + ((long)t * nb + mu) * ng;
                for (int g = 0; g < ng; g++) o[g] += -2.0 * a1[g] * T[g];
            }
        }
    if (type >= 1) {
        /* Rho1Grada(g,r,t,w) = -2 sum Da [AO2a(g,mu,r+t) AO(g,nu) + AO1a(g,mu,t) AO1(g,nu,r)] (:103-118) */
        memset(rho1g, 0, sizeof(double) * ng * 9 * natoms * ns);
        double* Tr = (double*)malloc(sizeof(double) * ng * 3);
        for (int w = 0; w < ns; w++)
            for (int mu = 0; mu < nb; mu++) {
                const int A = atom_of[mu];
                memset(T, 0, sizeof(double) * ng);
                memset(Tr, 0, sizeof(double) * ng * 3);
                for (int nu = 0; nu < nb; nu++) {
                    const double d = D[(long)w * nn + (long)nu * nb + mu];
                    for (int g = 0; g < ng; g++) T[g] += d * ao[(long)nu * ng + g];
                    for (int r = 0; r < 3; r++)
                        for (int g = 0; g < ng; g++) Tr[r * ng + g] += d * ao1[((long)r * nb + nu) * ng + g];
                }
                for (int t = 0; t < 3; t++)
                    for (int r = 0; r < 3; r++) {
                        double* o = rho1g + ((((long)w * natoms + A) * 3 + t) * 3 + r) * ng;
                        const double* h2 = ao2 + ((long)pair_pack(r, t) * nb + mu) * ng;
                        const double* a1 = ao1 + ((long)t * nb + mu) * ng;
                        for (int g = 0; g < ng; g++) o[g] += -2.0 * (h2[g] * T[g] + a1[g] * Tr[r * ng + g]);
                    }
            }
        free(Tr);
        /* SigmaGradaFull(g,t,u,v) = Rho1(g,r,u) Rho1Grada(g,r,t,v), symmetrised over (u,v), kept for
         * u <= v (:119-128) */
        const int nsig = ns * (ns + 1) / 2;
        memset(sigmag, 0, sizeof(double) * ng * 3 * natoms * nsig);
        for (int A = 0; A < natoms; A++)
            for (int t = 0; t < 3; t++)
                for (int v = 0; v < ns; v++)
                    for (int u = 0; u <= v; u++) {
                        double* o = sigmag + (((long)pair_pack(u, v) * natoms + A) * 3 + t) * ng;
                        for (int r = 0; r < 3; r++) {
                            const double* ru = rho1 + ((long)u * 3 + r) * ng;
                            const double* rv = rho1 + ((long)v * 3 + r) * ng;
                            const double* gu = rho1g + ((((long)u * natoms + A) * 3 + t) * 3 + r) * ng;
                            const double* gv = rho1g + ((((long)v * natoms + A) * 3 + t) * 3 + r) * ng;
                            for (int g = 0; g < ng; g++) o[g] += ru[g] * gv[g] + rv[g] * gu[g];
                        }
                    }
    }
    free(T);
}

/* SubGrid::getFockSkeleton (GridFock.cpp:52-95) for one block, accumulated into
 * F (ntot,ntot,3,natoms,s) through basis_list:
 *   F0a(mu in A, nu, t, w) = sum_g W Eps1Rho_w AO1a(g,mu,t) AO(g,nu)
 *   Fa1(mu in A, nu, t, u) = sum_g W S_(u+v) Eps1Sigma_(u+v) Rho1(g,r,v)
 *                            [AO2a(g,mu,r+t) AO(g,nu) + AO1a(g,mu,t) AO1(g,nu,r)]
 *   F(:,:,t,A,s) -= F0a + Fa1 (rows of A), then F += F^T over (mu, nu). */
void oracle_fock_skeleton(int ng, int nb, int ntot, const int* list, int ns, int natoms, const int* atom_of,
                          int type, const double* w, const double* ao, const double* ao1, const double* ao2,
                          const double* rho1, const double* vrho, const double* vsigma, double* Fout) {
    const long nn = (long)nb * nb;
    double* F = (double*)calloc((size_t)nn * 3 * natoms * ns, sizeof(double));
    double* L = (double*)malloc(sizeof(double) * ng);
    double* c1 = (double*)malloc(sizeof(double) * ng * 3);
    for (int s = 0; s < ns; s++) {
        /* c1_r(g) = W sum_v S_(s+v) vsigma_(s+v) Rho1(g,r,v) */
        memset(c1, 0, sizeof(double) * ng * 3);
        if (type >= 1)
            for (int v = 0; v < ns; v++) {
                const int uv = pair_pack(s, v);
                const double S = (s == v) ? 2.0 : 1.0;
                for (int r = 0; r < 3; r++)
                    for (int g = 0; g < ng; g++)
                        c1[r * ng + g] += w[g] * S * vsigma[(long)uv * ng + g] * rho1[((long)v * 3 + r) * ng + g];
            }
        for (int mu = 0; mu < nb; mu++) {
            const int A = atom_of[mu];
            for (int t = 0; t < 3; t++) {
                double* Fm = F + (((long)s * natoms + A) * 3 + t) * nn;
                /* L(g) multiplies AO(g,nu): W vrho d_t phi_mu + sum_r c1_r d_r d_t phi_mu */
                const double* a1 = ao1 + ((long)t * nb + mu) * ng;
                for (int g = 0; g < ng; g++) L[g] = w[g] * vrho[(long)s * ng + g] * a1[g];
                if (type >= 1)
                    for (int r = 0; r < 3; r++) {
                        const double* h2 = ao2 + ((long)pair_pack(r, t) * nb + mu) * ng;
                        for (int g = 0; g < ng; g++) L[g] += c1[r * ng + g] * h2[g];
                    }
                for (int nu = 0; nu < nb; nu++) {
                    double acc = 0;
                    for (int g = 0; g < ng; g++) acc += L[g] * ao[(long)nu * ng + g];
                    if (type >= 1)
                        for (int r = 0; r < 3; r++) {
                            const double* b1 = ao1 + ((long)r * nb + nu) * ng;
                            for (int g = 0; g < ng; g++) acc += c1[r * ng + g] * a1[g] * b1[g];
                        }
                    Fm[(long)nu * nb + mu] -= acc;
                }
            }
        }
    }
    for (long m = 0; m < (long)3 * natoms * ns; m++) {
        const double* Fm = F + m * nn;
        double* O = Fout + m * ntot * (long)ntot;
        for (int nu = 0; nu < nb; nu++)
            for (int mu = 0; mu < nb; mu++)
                O[(long)list[nu] * ntot + list[mu]] += Fm[(long)nu * nb + mu] + Fm[(long)mu * nb + nu];
    }
    free(c1);
    free(L);
    free(F);
}

/* ------------------------------------------------ energy Hessian (restricted) */

static int triple_pack(int a, int b, int c) {
    int v[3] = {a, b, c};
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2 - i; j++)
            if (v[j] > v[j + 1]) {
                const int t = v[j];
                v[j] = v[j + 1];
                v[j + 1] = t;
            }
    return v[0] + v[1] * (v[1] + 1) / 2 + v[2] * (v[2] + 1) * (v[2] + 2) / 6;
}

/* AO third derivatives ao3[(c * nbasis + mu) * ng + g], c the packed sorted triple
 * i0 + i1 (i1 + 1) / 2 + i2 (i2 + 1) (i2 + 2) / 6 (xxx, xxy, xyy, yyy, xxz, xyz, yyz, xzz, yzz, zzz):
 *   d_abc phi = A_abc Q + A_ab Q_c + A_ac Q_b + A_bc Q_a + A_a Q_bc + A_b Q_ac + A_c Q_ab + A Q_abc
 * with A_abc = -8 x_a x_b x_c sum c alpha^3 e + 4 (d_ab x_c + d_ac x_b + d_bc x_a) sum c alpha^2 e
 * (GridAO.cpp:134-146, 197-208); Q's derivatives from oracle_ao2 on a unit radial part and central
 * differences of its second derivatives (exact: they are at most quadratic). */
void oracle_ao3(int nshells, const int* shell_type, const int* shell_nprim, const int* shell_prim_off,
                const double* shell_center, const double* exps, const double* coefs, int nbasis, int ng,
                const double* xs, const double* ys, const double* zs, double* ao3) {
    int ibasis = 0;
    const double zero_exp = 0.0, one_coef = 1.0;
    const int one_nprim = 1, zero_off = 0;
    const double org[3] = {0, 0, 0};
    double q[16], q1[48], q2[96], q2p[96], q2m[96];
    for (int s = 0; s < nshells; s++) {
        const int type = shell_type[s];
        const double* e = exps + shell_prim_off[s];
        const double* c = coefs + shell_prim_off[s];
        const double* C = shell_center + 3 * s;
        const int size = type == 0 ? 1 : (type == 1 || type == -1) ? 3 : 2 * (-type) + 1;
        for (int k = 0; k < ng; k++) {
            const double r[3] = {xs[k] - C[0], ys[k] - C[1], zs[k] - C[2]};
            const double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
            double t[4] = {0, 0, 0, 0};
            for (int p = 0; p < shell_nprim[s]; p++) {
                const double v = c[p] * exp(-e[p] * r2);
                t[0] += v;
                t[1] += v * e[p];
                t[2] += v * e[p] * e[p];
                t[3] += v * e[p] * e[p] * e[p];
            }
            oracle_ao(1, &type, &one_nprim, &zero_off, org, &zero_exp, &one_coef, size, 1, &r[0], &r[1], &r[2], 1, q,
                      q1);
            oracle_ao2(1, &type, &one_nprim, &zero_off, org, &zero_exp, &one_coef, size, 1, &r[0], &r[1], &r[2], q2);
            double Q3[10][16];
            for (int cdir = 0; cdir < 3; cdir++) {
                const double h = 1e-2;
                double rp[3] = {r[0], r[1], r[2]}, rm[3] = {r[0], r[1], r[2]};
                rp[cdir] += h;
                rm[cdir] -= h;
                oracle_ao2(1, &type, &one_nprim, &zero_off, org, &zero_exp, &one_coef, size, 1, &rp[0], &rp[1],
                           &rp[2], q2p);
                oracle_ao2(1, &type, &one_nprim, &zero_off, org, &zero_exp, &one_coef, size, 1, &rm[0], &rm[1],
                           &rm[2], q2m);
                for (int b = 0; b < 3; b++)
                    for (int a = 0; a <= b; a++) {
                        if (cdir < b) continue; /* each sorted triple (a <= b <= cdir) once */
                        const int pk2 = a + b * (b + 1) / 2, pk3 = triple_pack(a, b, cdir);
                        for (int i = 0; i < size; i++)
                            Q3[pk3][i] = (q2p[pk2 * size + i] - q2m[pk2 * size + i]) / (2 * h);
                    }
            }
            for (int cc = 0; cc < 3; cc++)
                for (int b = 0; b <= cc; b++)
                    for (int a = 0; a <= b; a++) {
                        const int idx[3] = {a, b, cc};
                        const double x[3] = {r[idx[0]], r[idx[1]], r[idx[2]]};
                        const double dab = a == b, dac = a == cc, dbc = b == cc;
                        const double A1[3] = {-2 * x[0] * t[1], -2 * x[1] * t[1], -2 * x[2] * t[1]};
                        const double Aab = 4 * x[0] * x[1] * t[2] - 2 * dab * t[1];
                        const double Aac = 4 * x[0] * x[2] * t[2] - 2 * dac * t[1];
                        const double Abc = 4 * x[1] * x[2] * t[2] - 2 * dbc * t[1];
                        const double Aabc = -8 * x[0] * x[1] * x[2] * t[3] + 4 * (dab * x[2] + dac * x[1] + dbc * x[0]) * t[2];
                        const int pk3 = triple_pack(a, b, cc);
                        for (int i = 0; i < size; i++) {
                            const double Qa = q1[a * size + i], Qb = q1[b * size + i], Qc = q1[cc * size + i];
                            const double Qbc = q2[pair_pack(b, cc) * size + i], Qac = q2[pair_pack(a, cc) * size + i],
                                         Qab = q2[pair_pack(a, b) * size + i];
                            ao3[((long)pk3 * nbasis + ibasis + i) * ng + k] =
                                Aabc * q[i] + Aab * Qc + Aac * Qb + Abc * Qa + A1[0] * Qbc + A1[1] * Qac + A1[2] * Qab +
                                t[0] * Q3[pk3][i];
                        }
                    }
        }
        ibasis += size;
    }
}

/* SubGrid::getDensitySkeleton2 + SubGrid::getEnergyHess (GridDensity.cpp:132-212,
 * GridEnergy.cpp:32-46) for one block, restricted (the reference marks its sigma Hessian
 * as incorrect for open shells, GridDensity.cpp:210): adds
 *   E(t,a,s,b) += sum_g W [f_rr rho_at rho_bs + v_r rho_at,bs + f_rs (rho_at sigma_bs + sigma_at rho_bs)
 *                          + f_ss sigma_at sigma_bs + v_s sigma_at,bs]
 * to E (3 natoms x 3 natoms, index (3 a + t) + 3 natoms (3 b + s)), with the skeleton first
 * derivatives of oracle_density_skeleton (rhog, rho1g, sigmag) and
 *   rho_at,bs   = 2 [d_ab sum_(mu on a) H_ts,mu T0_mu + sum_(mu on a, nu on b) D d_t phi_mu d_s phi_nu]
 *   (grad_r rho)_at,bs = 2 [d_ab sum_(mu on a) (T3_rts,mu T0_mu + H_ts,mu Tr_mu)
 *                          + sum_(mu on a, nu on b) D (H_rt,mu d_s phi_nu + d_t phi_mu H_rs,nu)]
 *   sigma_at,bs = 2 (grad rho . (grad rho)_at,bs + (grad rho)_at . (grad rho)_bs)
 * where T0_mu = sum_nu D phi_nu, Tr_mu = sum_nu D d_r phi_nu. */
void oracle_energy_hess(int ng, int nb, int natoms, const int* atom_of, int type, const double* D,
                        const double* w, const double* ao, const double* ao1, const double* ao2, const double* ao3,
                        const double* rho1, const double* vrho, const double* vsigma, const double* v2rho2,
                        const double* v2rhosigma, const double* v2sigma2, const double* rhog, const double* rho1g,
                        const double* sigmag, double* E) {
    const int nm = 3 * natoms;
    double* T0 = (double*)calloc((size_t)nb * ng, sizeof(double));
    double* Tr = (double*)calloc((size_t)3 * nb * ng, sizeof(double));
    for (int mu = 0; mu < nb; mu++)
        for (int nu = 0; nu < nb; nu++) {
            const double d = D[(long)nu * nb + mu];
            for (int g = 0; g < ng; g++) {
                T0[(long)mu * ng + g] += d * ao[(long)nu * ng + g];
                if (type >= 1)
                    for (int r = 0; r < 3; r++) Tr[((long)r * nb + mu) * ng + g] += d * ao1[((long)r * nb + nu) * ng + g];
            }
        }
    double* rh = (double*)malloc(sizeof(double) * ng);
    double* r1h = (double*)malloc(sizeof(double) * ng * 3);
    for (int a = 0; a < natoms; a++)
        for (int t = 0; t < 3; t++)
            for (int b = 0; b < natoms; b++)
                for (int s = 0; s < 3; s++) {
                    memset(rh, 0, sizeof(double) * ng);
                    memset(r1h, 0, sizeof(double) * ng * 3);
                    for (int mu = 0; mu < nb; mu++) {
                        if (atom_of[mu] != a) continue;
                        const double* dt = ao1 + ((long)t * nb + mu) * ng;
                        if (a == b) {
                            const double* hts = ao2 + ((long)pair_pack(t, s) * nb + mu) * ng;
                            for (int g = 0; g < ng; g++) rh[g] += hts[g] * T0[(long)mu * ng + g];
                            if (type >= 1)
                                for (int r = 0; r < 3; r++) {
                                    const double* t3 = ao3 + ((long)triple_pack(r, t, s) * nb + mu) * ng;
                                    for (int g = 0; g < ng; g++)
                                        r1h[r * ng + g] += t3[g] * T0[(long)mu * ng + g] + hts[g] * Tr[((long)r * nb + mu) * ng + g];
                                }
                        }
                        for (int nu = 0; nu < nb; nu++) {
                            if (atom_of[nu] != b) continue;
                            const double d = D[(long)nu * nb + mu];
                            if (d == 0) continue;
                            const double* ds = ao1 + ((long)s * nb + nu) * ng;
                            for (int g = 0; g < ng; g++) rh[g] += d * dt[g] * ds[g];
                            if (type >= 1)
                                for (int r = 0; r < 3; r++) {
                                    const double* hrt = ao2 + ((long)pair_pack(r, t) * nb + mu) * ng;
                                    const double* hrs = ao2 + ((long)pair_pack(r, s) * nb + nu) * ng;
                                    for (int g = 0; g < ng; g++) r1h[r * ng + g] += d * (hrt[g] * ds[g] + dt[g] * hrs[g]);
                                }
                        }
                    }
                    const long i = 3 * a + t, j = 3 * b + s;
                    const double* ra = rhog + i * ng;
                    const double* rb = rhog + j * ng;
                    double acc = 0;
                    for (int g = 0; g < ng; g++) {
                        double v = v2rho2[g] * ra[g] * rb[g] + vrho[g] * 2.0 * rh[g];
                        if (type >= 1) {
                            const double sa = sigmag[i * ng + g], sb = sigmag[j * ng + g];
                            double shess = 0;
                            for (int r = 0; r < 3; r++)
                                shess += rho1[r * ng + g] * 2.0 * r1h[r * ng + g] +
                                         rho1g[(i * 3 + r) * ng + g] * rho1g[(j * 3 + r) * ng + g];
                            shess *= 2.0;
                            v += v2rhosigma[g] * (ra[g] * sb + sa * rb[g]) + v2sigma2[g] * sa * sb + vsigma[g] * shess;
                        }
                        acc += w[g] * v;
                    }
                    E[i + nm * j] += acc;
                }
    free(r1h);
    free(rh);
    free(Tr);
    free(T0);
}

/* ------------------------------------------------------ response build (OpenMP) */

#ifdef _OPENMP
#include <omp.h>
#endif

/* The response over a list of blocks (the blocks' AO values concatenated as in oracle_build):
 * per block the ground-state density, vsigma and second derivatives, the response densities
 * of the nmat matrices D_U (n,n,nmat,s) and their V_U accumulated into F (n,n,nmat,s), OpenMP
 * over blocks (the reference's static bins, GridGeneration.cpp:293-300, with per-thread copies
 * of F reduced at the end, as Grid::getFockU does, Grid.cpp:194-218).  Returns 0, or -1 for a
 * meta-GGA or unknown functional id. */
int oracle_build_response(int nblocks, const int* blk_ng, const long* blk_pt_off, const long* blk_ao_off,
                          const double* w, const double* ao, const double* ao1, int nb, int ns, int type,
                          const double* D, int nmat, const double* DU, int nids, const int* ids, int nthreads,
                          double* F_out) {
    if (type > 1) return -1;
    int* list = (int*)malloc(sizeof(int) * nb);
    for (int i = 0; i < nb; i++) list[i] = i;
    const long nf = (long)nb * nb * nmat * ns;
    for (long i = 0; i < nf; i++) F_out[i] = 0;
    int status = 0;
    const int nsig = ns == 1 ? 1 : 3, nrs = ns == 1 ? 1 : 6, nrr = ns == 1 ? 1 : 3;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
    nthreads = 1;
#endif
#pragma omp parallel num_threads(nthreads)
    {
        double* Fp = (double*)calloc(nf, sizeof(double));
        const int cap = 128;
        double* rho = (double*)malloc(sizeof(double) * cap * ns);
        double* rho1 = (double*)malloc(sizeof(double) * cap * 3 * ns);
        double* sigma = (double*)malloc(sizeof(double) * cap * nsig);
        double* tau = (double*)malloc(sizeof(double) * cap * ns);
        double* eps = (double*)malloc(sizeof(double) * cap);
        double* vrho = (double*)malloc(sizeof(double) * cap * ns);
        double* vsigma = (double*)malloc(sizeof(double) * cap * nsig);
        double* vtau = (double*)malloc(sizeof(double) * cap * ns);
        double* f1 = (double*)malloc(sizeof(double) * cap * nrr);
        double* f2 = (double*)malloc(sizeof(double) * cap * nrs);
        double* f3 = (double*)malloc(sizeof(double) * cap * nrs);
        double* rU = (double*)malloc(sizeof(double) * cap * nmat * ns);
        double* r1U = (double*)malloc(sizeof(double) * cap * 3 * nmat * ns);
        double* sU = (double*)malloc(sizeof(double) * cap * nmat * nsig);
#pragma omp for schedule(static)
        for (int b = 0; b < nblocks; b++) {
            const int ng = blk_ng[b];
            if (ng > cap) {
#pragma omp atomic write
                status = -1;
                continue;
            }
            const double* a0 = ao + blk_ao_off[b];
            const double* a1 = type >= 1 ? ao1 + 3 * blk_ao_off[b] : NULL;
            const double* wb = w + blk_pt_off[b];
            oracle_density(ng, nb, ns, type, D, a0, a1, rho, rho1, sigma, tau);
            int st = oracle_functional(nids, ids, ns, ng, rho, sigma, tau, eps, vrho, vsigma, vtau);
            st |= oracle_functional_fxc(nids, ids, ns, ng, rho, sigma, f1, f2, f3);
            if (st) {
#pragma omp atomic write
                status = -1;
            }
            oracle_density_u(ng, nb, ns, nmat, type, DU, a0, a1, rho1, rU, r1U, sU);
            oracle_fock_u(ng, nb, nb, list, ns, nmat, type, wb, a0, a1, rho1, vsigma, f1, f2, f3, rU, r1U, sU, Fp);
        }
#pragma omp critical
        for (long i = 0; i < nf; i++) F_out[i] += Fp[i];
        free(Fp);
        free(rho); free(rho1); free(sigma); free(tau); free(eps); free(vrho); free(vsigma); free(vtau);
        free(f1); free(f2); free(f3); free(rU); free(r1U); free(sU);
    }
    free(list);
    return status;
}
