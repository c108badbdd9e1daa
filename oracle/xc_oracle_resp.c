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
