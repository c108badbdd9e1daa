/*
 * ORACLE -- test infrastructure only (see xc_oracle.h).  CPU FP64
 * restatement of the reference's grid/AO/density/energy/Fock stages.
 * Citations are file:line within the Chinium source tree.
 */
#include "xc_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---------------------------------------------------------------- Becke -- */

/* GridGeneration.cpp:50-71: cell function s(mu) with three smoothing steps,
 * mu = (|r - R_b| - |r - R_c|) / |R_b - R_c|. */
static double s_p_mu(double x0, double y0, double z0, double x1, double y1, double z1, double x2,
                     double y2, double z2) {
    const double x01 = x0 - x1, y01 = y0 - y1, z01 = z0 - z1;
    const double r01 = sqrt(x01 * x01 + y01 * y01 + z01 * z01);
    const double x02 = x0 - x2, y02 = y0 - y2, z02 = z0 - z2;
    const double r02 = sqrt(x02 * x02 + y02 * y02 + z02 * z02);
    const double x12 = x1 - x2, y12 = y1 - y2, z12 = z1 - z2;
    const double r12 = sqrt(x12 * x12 + y12 * y12 + z12 * z12);
    const double mu = (r01 - r02) / r12;
    const double p1 = 1.5 * mu - 0.5 * mu * mu * mu;
    const double p2 = 1.5 * p1 - 0.5 * p1 * p1 * p1;
    const double p3 = 1.5 * p2 - 0.5 * p2 * p2 * p2;
    return 0.5 * (1 - p3);
}

/* GridGeneration.cpp:134-153. */
void oracle_becke(int natoms, const double* a, long npts, const double* px, const double* py,
                  const double* pz, const int* owner, const double* w_in, double* w_out) {
#pragma omp parallel for schedule(static)
    for (long k = 0; k < npts; k++) {
        const double x = px[k], y = py[k], z = pz[k];
        double total = 0, mine = 0;
        for (int b = 0; b < natoms; b++) {
            double pb = 1;
            for (int c = 0; c < natoms; c++) {
                if (b == c) continue;
                pb *= s_p_mu(x, y, z, a[3 * b], a[3 * b + 1], a[3 * b + 2], a[3 * c], a[3 * c + 1],
                             a[3 * c + 2]);
            }
            total += pb;
            if (b == owner[k]) mine = pb;
        }
        w_out[k] = w_in[k] * (mine / total);
    }
}

/* ------------------------------------------------------------------- AO -- */

typedef double complex cplx;

/* Angular parts, restating AO/S.hpp, AO/CartP.hpp, AO/PureP.hpp,
 * AO/PureD.hpp:1-5, AO/PureF.hpp:1-7, AO/PureG.hpp:1-9 (values).  Gradients
 * are taken by complex step on these polynomials, exact to rounding. */
static int angular(int type, cplx x, cplx y, cplx z, cplx* Q) {
    const cplx r2 = x * x + y * y + z * z;
    switch (type) {
        case 0: Q[0] = 1; return 1;
        case 1: Q[0] = x; Q[1] = y; Q[2] = z; return 3;
        case -1: Q[0] = y; Q[1] = z; Q[2] = x; return 3;
        case -2:
            Q[0] = x * y * sqrt(3.);
            Q[1] = y * z * sqrt(3.);
            Q[2] = (3 * z * z - r2) / 2;
            Q[3] = x * z * sqrt(3.);
            Q[4] = (x * x - y * y) * sqrt(3.) / 2;
            return 5;
        case -3:
            Q[0] = y * (3 * x * x - y * y) * sqrt(10.) / 4;
            Q[1] = x * y * z * sqrt(15.);
            Q[2] = y * (5 * z * z - r2) * sqrt(6.) / 4;
            Q[3] = (5 * z * z * z - 3 * z * r2) / 2;
            Q[4] = x * (5 * z * z - r2) * sqrt(6.) / 4;
            Q[5] = (x * x - y * y) * z * sqrt(15.) / 2;
            Q[6] = x * (x * x - 3 * y * y) * sqrt(10.) / 4;
            return 7;
        case -4:
            Q[0] = x * y * (x * x - y * y) * sqrt(35.) / 2;
            Q[1] = y * (3 * x * x - y * y) * z * sqrt(70.) / 4;
            Q[2] = x * y * (7 * z * z - r2) * sqrt(5.) / 2;
            Q[3] = y * (7 * z * z * z - 3 * z * r2) * sqrt(10.) / 4;
            Q[4] = (35 * z * z * z * z - 30 * z * z * r2 + 3 * r2 * r2) / 8;
            Q[5] = x * (7 * z * z * z - 3 * z * r2) * sqrt(10.) / 4;
            Q[6] = (x * x - y * y) * (7 * z * z - r2) * sqrt(5.) / 4;
            Q[7] = x * (x * x - 3 * y * y) * z * sqrt(70.) / 4;
            Q[8] = (x * x * (x * x - 3 * y * y) - y * y * (3 * x * x - y * y)) * sqrt(35.) / 8;
            return 9;
    }
    return -1;
}

/* GridAO.cpp:72-214 restricted to derivative order <= 1. */
void oracle_ao(int nshells, const int* shell_type, const int* shell_nprim,
               const int* shell_prim_off, const double* shell_center, const double* exps,
               const double* coefs, int nbasis, int ng, const double* xs, const double* ys,
               const double* zs, int deriv, double* ao, double* ao1) {
    int ibasis = 0;
    for (int s = 0; s < nshells; s++) {
        const int type = shell_type[s];
        const double* e = exps + shell_prim_off[s];
        const double* c = coefs + shell_prim_off[s];
        const double xo = shell_center[3 * s], yo = shell_center[3 * s + 1],
                     zo = shell_center[3 * s + 2];
        int size = 0;
        for (int k = 0; k < ng; k++) {
            const double x = xs[k] - xo, y = ys[k] - yo, z = zs[k] - zo;
            const double r2 = x * x + y * y + z * z;
            double tmp0 = 0, tmp1 = 0;
            for (int p = 0; p < shell_nprim[s]; p++) { /* GridAO.cpp:113-124 */
                const double t = c[p] * exp(-e[p] * r2);
                tmp0 += t;
                tmp1 += t * e[p];
            }
            const double A = tmp0;
            const double Ax = -2 * x * tmp1, Ay = -2 * y * tmp1, Az = -2 * z * tmp1;
            cplx Q[16] = {0}, Qx[16] = {0}, Qy[16] = {0}, Qz[16] = {0};
            size = angular(type, x, y, z, Q);
            if (deriv) {
                const double h = 1e-30;
                angular(type, x + I * h, y, z, Qx);
                angular(type, x, y + I * h, z, Qy);
                angular(type, x, y, z + I * h, Qz);
                for (int i = 0; i < size; i++) {
                    Qx[i] = cimag(Qx[i]) / h;
                    Qy[i] = cimag(Qy[i]) / h;
                    Qz[i] = cimag(Qz[i]) / h;
                }
            }
            for (int i = 0; i < size; i++) { /* GridAO.cpp:179-184 */
                const double q = creal(Q[i]);
                ao[(long)(ibasis + i) * ng + k] = A * q;
                if (deriv) {
                    ao1[((long)0 * nbasis + ibasis + i) * ng + k] = Ax * q + A * creal(Qx[i]);
                    ao1[((long)1 * nbasis + ibasis + i) * ng + k] = Ay * q + A * creal(Qy[i]);
                    ao1[((long)2 * nbasis + ibasis + i) * ng + k] = Az * q + A * creal(Qz[i]);
                }
            }
        }
        ibasis += size;
    }
}

/* -------------------------------------------------------------- density -- */

void oracle_density(int ng, int nb, int ns, int type, const double* D, const double* ao,
                    const double* ao1, double* rho, double* rho1, double* sigma, double* tau) {
    double* tmp = (double*)malloc(sizeof(double) * ng);
    /* Rho einsum D(mu,nu,w) AO(g,mu) AO(g,nu) -> Rho(g,w): loops w, nu, mu, g */
    for (int i = 0; i < ng * ns; i++) rho[i] = 0;
    for (int w = 0; w < ns; w++)
        for (int nu = 0; nu < nb; nu++) {
            for (int g = 0; g < ng; g++) tmp[g] = 0;
            for (int mu = 0; mu < nb; mu++) {
                const double d = D[(long)w * nb * nb + (long)nu * nb + mu];
                const double* a = ao + (long)mu * ng;
                for (int g = 0; g < ng; g++) tmp[g] += d * a[g];
            }
            const double* a = ao + (long)nu * ng;
            for (int g = 0; g < ng; g++) rho[w * ng + g] += tmp[g] * a[g];
        }
    if (type >= 1) {
        /* Rho1 einsum D(mu,nu,w) AO1(g,mu,r) AO(g,nu) -> Rho1(g,r,w), then x2
         * (GridDensity.cpp:27-29) */
        for (int i = 0; i < ng * 3 * ns; i++) rho1[i] = 0;
        for (int w = 0; w < ns; w++)
            for (int r = 0; r < 3; r++)
                for (int nu = 0; nu < nb; nu++) {
                    for (int g = 0; g < ng; g++) tmp[g] = 0;
                    for (int mu = 0; mu < nb; mu++) {
                        const double d = D[(long)w * nb * nb + (long)nu * nb + mu];
                        const double* a = ao1 + ((long)r * nb + mu) * ng;
                        for (int g = 0; g < ng; g++) tmp[g] += d * a[g];
                    }
                    const double* a = ao + (long)nu * ng;
                    double* o = rho1 + ((long)w * 3 + r) * ng;
                    for (int g = 0; g < ng; g++) o[g] += tmp[g] * a[g];
                }
        for (int i = 0; i < ng * 3 * ns; i++) rho1[i] *= 2;
        /* Sigma einsum (u <= v, index u + v(v+1)/2), GridDensity.cpp:30-31 */
        const int nsig = ns * (ns + 1) / 2;
        for (int i = 0; i < ng * nsig; i++) sigma[i] = 0;
        for (int v = 0; v < ns; v++)
            for (int u = 0; u <= v; u++) {
                const int uv = u + v * (v + 1) / 2;
                for (int r = 0; r < 3; r++)
                    for (int g = 0; g < ng; g++)
                        sigma[uv * ng + g] +=
                            rho1[((long)u * 3 + r) * ng + g] * rho1[((long)v * 3 + r) * ng + g];
            }
    }
    if (type >= 2) {
        /* Tau einsum D(mu,nu,w) AO1(g,mu,r) AO1(g,nu,r) -> Tau(g,w), x1/2
         * (GridDensity.cpp:34-36) */
        for (int i = 0; i < ng * ns; i++) tau[i] = 0;
        for (int w = 0; w < ns; w++)
            for (int r = 0; r < 3; r++)
                for (int nu = 0; nu < nb; nu++) {
                    for (int g = 0; g < ng; g++) tmp[g] = 0;
                    for (int mu = 0; mu < nb; mu++) {
                        const double d = D[(long)w * nb * nb + (long)nu * nb + mu];
                        const double* a = ao1 + ((long)r * nb + mu) * ng;
                        for (int g = 0; g < ng; g++) tmp[g] += d * a[g];
                    }
                    const double* a = ao1 + ((long)r * nb + nu) * ng;
                    for (int g = 0; g < ng; g++) tau[w * ng + g] += tmp[g] * a[g];
                }
        for (int i = 0; i < ng * ns; i++) tau[i] *= 0.5;
    }
    free(tmp);
}

/* --------------------------------------------------------------- energy -- */

/* EnergyEinSum/W_g...Rho_g,w...Eps_g---E_.hpp:32-44 */
double oracle_energy(int ng, int ns, const double* w, const double* rho, const double* eps) {
    double E = 0;
    for (int g = 0; g < ng; g++) {
        double wr = 0;
        for (int s = 0; s < ns; s++) wr += w[g] * rho[s * ng + g];
        E += wr * eps[g];
    }
    return E;
}

/* ----------------------------------------------------------------- Fock -- */

void oracle_fock(int ng, int nb, int ntot, const int* list, int ns, int type, const double* w,
                 const double* ao, const double* ao1, const double* rho1, const double* vrho,
                 const double* vsigma, const double* vtau, double* Fout) {
    double* F = (double*)calloc((size_t)nb * nb * ns, sizeof(double));
    double* tmp = (double*)malloc(sizeof(double) * ng);
    /* F0 = W vrho AO AO, added as 0.5*F0 (GridFock.cpp:16-20) */
    for (int s = 0; s < ns; s++)
        for (int mu = 0; mu < nb; mu++) {
            for (int g = 0; g < ng; g++) tmp[g] = w[g] * vrho[s * ng + g] * ao[(long)mu * ng + g];
            for (int nu = 0; nu < nb; nu++) {
                double acc = 0;
                for (int g = 0; g < ng; g++) acc += tmp[g] * ao[(long)nu * ng + g];
                F[(long)s * nb * nb + (long)nu * nb + mu] += 0.5 * acc;
            }
        }
    if (type >= 1) {
        /* F1 = W S(uv) vsigma(u+v) Rho1(g,r,v) AO1(g,mu,r) AO(g,nu)
         * with S = 2 on the spin diagonal (GridFock.cpp:21-31) */
        double* wsr = (double*)malloc(sizeof(double) * ng * 3);
        for (int u = 0; u < ns; u++) {
            for (int i = 0; i < ng * 3; i++) wsr[i] = 0;
            for (int v = 0; v < ns; v++) {
                const int lo = u < v ? u : v, hi = u < v ? v : u;
                const int uv = lo + hi * (hi + 1) / 2;
                const double S = (u == v) ? 2.0 : 1.0;
                for (int r = 0; r < 3; r++)
                    for (int g = 0; g < ng; g++)
                        wsr[r * ng + g] +=
                            w[g] * S * vsigma[uv * ng + g] * rho1[((long)v * 3 + r) * ng + g];
            }
            for (int mu = 0; mu < nb; mu++) {
                for (int g = 0; g < ng; g++) tmp[g] = 0;
                for (int r = 0; r < 3; r++)
                    for (int g = 0; g < ng; g++)
                        tmp[g] += wsr[r * ng + g] * ao1[((long)r * nb + mu) * ng + g];
                for (int nu = 0; nu < nb; nu++) {
                    double acc = 0;
                    for (int g = 0; g < ng; g++) acc += tmp[g] * ao[(long)nu * ng + g];
                    F[(long)u * nb * nb + (long)nu * nb + mu] += acc;
                }
            }
        }
        free(wsr);
    }
    if (type >= 2) {
        /* 0.5 * W (vtau/2 + 2 vlapl) AO1 . AO1 with vlapl = 0 (GridFock.cpp:32-36) */
        for (int s = 0; s < ns; s++)
            for (int mu = 0; mu < nb; mu++)
                for (int nu = 0; nu < nb; nu++) {
                    double acc = 0;
                    for (int r = 0; r < 3; r++)
                        for (int g = 0; g < ng; g++)
                            acc += w[g] * 0.5 * vtau[s * ng + g] * ao1[((long)r * nb + mu) * ng + g] *
                                   ao1[((long)r * nb + nu) * ng + g];
                    F[(long)s * nb * nb + (long)nu * nb + mu] += 0.5 * acc;
                }
    }
    /* F += F^T, scatter through BasisList (GridFock.cpp:41-48) */
    for (int s = 0; s < ns; s++)
        for (int nu = 0; nu < nb; nu++)
            for (int mu = 0; mu < nb; mu++) {
                const double* Fs = F + (long)s * nb * nb;
                const double v = Fs[(long)nu * nb + mu] + Fs[(long)mu * nb + nu];
                Fout[(long)s * ntot * ntot + (long)list[nu] * ntot + list[mu]] += v;
            }
    free(tmp);
    free(F);
}

/* ------------------------------------------------------------------ SAP -- */

void oracle_sap(int natoms, const double* a, const double* table, const double* radii, int nradii,
                long npts, const double* px, const double* py, const double* pz, double* v) {
#pragma omp parallel for schedule(static)
    for (long k = 0; k < npts; k++) {
        double acc = 0;
        for (int at = 0; at < natoms; at++) {
            const double x = px[k] - a[3 * at], y = py[k] - a[3 * at + 1], z = pz[k] - a[3 * at + 2];
            const double r = sqrt(x * x + y * y + z * z) + 1.e-12;
            double bestdiff = 114514, bestvap = 114514;
            for (int i = 0; i < nradii; i++) {
                if (bestdiff > fabs(radii[i] - r)) {
                    bestdiff = fabs(radii[i] - r);
                    bestvap = table[(long)at * nradii + i] / r;
                }
            }
            acc += bestvap;
        }
        v[k] = acc;
    }
}

/* ---------------------------------------------------------- whole build -- */

int oracle_build(int nblocks, const int* blk_ng, const long* blk_pt_off, const long* blk_ao_off,
                 const double* w, const double* ao, const double* ao1, int nb, int ns, int type,
                 const double* D, int nids, const int* ids, int nthreads, double* E_out,
                 double* F_out) {
    int* list = (int*)malloc(sizeof(int) * nb);
    for (int i = 0; i < nb; i++) list[i] = i;
    const long nn = (long)nb * nb * ns;
    for (long i = 0; i < nn; i++) F_out[i] = 0;
    double E = 0;
    int status = 0;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
    nthreads = 1;
#endif
#pragma omp parallel num_threads(nthreads) reduction(+ : E)
    {
        double* Fp = (double*)calloc(nn, sizeof(double));
        double *rho = NULL, *rho1 = NULL, *sigma = NULL, *tau = NULL, *eps = NULL, *vrho = NULL,
               *vsigma = NULL, *vtau = NULL;
        int cap = 0;
#pragma omp for schedule(static)
        for (int b = 0; b < nblocks; b++) {
            const int ng = blk_ng[b];
            if (ng > cap) {
                cap = ng;
                rho = (double*)realloc(rho, sizeof(double) * ng * ns);
                rho1 = (double*)realloc(rho1, sizeof(double) * ng * 3 * ns);
                sigma = (double*)realloc(sigma, sizeof(double) * ng * 3);
                tau = (double*)realloc(tau, sizeof(double) * ng * ns);
                eps = (double*)realloc(eps, sizeof(double) * ng);
                vrho = (double*)realloc(vrho, sizeof(double) * ng * ns);
                vsigma = (double*)realloc(vsigma, sizeof(double) * ng * 3);
                vtau = (double*)realloc(vtau, sizeof(double) * ng * ns);
            }
            const double* a0 = ao + blk_ao_off[b];
            const double* a1 = type >= 1 ? ao1 + 3 * blk_ao_off[b] : NULL;
            const double* wb = w + blk_pt_off[b];
            oracle_density(ng, nb, ns, type, D, a0, a1, rho, rho1, sigma, tau);
            if (oracle_functional(nids, ids, ns, ng, rho, sigma, tau, eps, vrho, vsigma, vtau))
                status = -1;
            E += oracle_energy(ng, ns, wb, rho, eps);
            oracle_fock(ng, nb, nb, list, ns, type, wb, a0, a1, rho1, vrho, vsigma, vtau, Fp);
        }
#pragma omp critical
        for (long i = 0; i < nn; i++) F_out[i] += Fp[i];
        free(Fp);
        free(rho); free(rho1); free(sigma); free(tau);
        free(eps); free(vrho); free(vsigma); free(vtau);
    }
    free(list);
    *E_out = E;
    return status;
}
