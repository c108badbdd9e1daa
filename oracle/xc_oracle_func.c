/*
 * ORACLE -- test infrastructure only (see xc_oracle.h).
 *
 * Exchange-correlation functionals restated from their published papers, as
 * libxc implements them behind the ids in the DensityFunctionals .df files (called at
 * src/ExchangeCorrelation.cpp:86-163, :202-217).  libxc is absent, so parity
 * with it is unpinned.  Each functional is written once as an energy density
 * per volume e(rho_a, rho_b, sigma_aa, sigma_ab, sigma_bb, tau_a, tau_b) in
 * complex arithmetic; potentials are exact complex-step derivatives
 * Im e(x + ih) / h, so no hand-derived derivative enters the oracle.
 *
 * Input thresholds follow libxc's documented conventions (a density
 * threshold below which the point is skipped, sigma >= threshold^(8/3),
 * tau >= 1e-20, sigma <= 8 rho tau for meta-GGAs, |zeta| clamped away from 1).
 */
#include <complex.h>
#include <math.h>
#include <string.h>

#include "xc_oracle.h"

typedef double complex cplx;

#define DENS_THR 1e-15
#define TAU_THR 1e-20
#define ZETA_THR 2.220446049250313e-16

static const double PI = 3.14159265358979323846;

typedef struct {
    cplx ra, rb, saa, sab, sbb, ta, tb;
} xin;

static cplx cpw(cplx z, double p) { return cpow(z, p); }
static cplx cmaxr(cplx a, cplx b) { return creal(a) >= creal(b) ? a : b; }
static cplx cminr(cplx a, cplx b) { return creal(a) <= creal(b) ? a : b; }

/* 1 +/- zeta clamped away from zero. */
static cplx opz_clamp(cplx v) { return creal(v) < ZETA_THR ? (cplx)ZETA_THR : v; }

/* ------------------------------------------------------------------ LDA -- */

/* Slater exchange for one spin channel by spin scaling:
 * e = 1/2 e_unif(2 rho_s), e_unif(n) = -(3/4)(3/pi)^(1/3) n^(4/3). */
static cplx ex_unif_half(cplx rs_) {
    const double Cx = 0.75 * pow(3.0 / PI, 1.0 / 3.0);
    return -0.5 * Cx * cpw(2.0 * rs_, 4.0 / 3.0);
}

static cplx e_lda_x(const xin* v) { return ex_unif_half(v->ra) + ex_unif_half(v->rb); }

/* VWN interpolation formula (Vosko, Wilk, Nusair 1980), x = sqrt(rs). */
static cplx vwn_f(cplx x, double A, double b, double c, double x0) {
    const double Q = sqrt(4 * c - b * b);
    const cplx X = x * x + b * x + c;
    const double X0 = x0 * x0 + b * x0 + c;
    const cplx at = catan(Q / (2 * x + b));
    return A * (clog(x * x / X) + 2 * b / Q * at -
                b * x0 / X0 * (clog((x - x0) * (x - x0) / X) + 2 * (b + 2 * x0) / Q * at));
}

static cplx fzeta(cplx opz, cplx omz) {
    return (cpw(opz, 4.0 / 3.0) + cpw(omz, 4.0 / 3.0) - 2) / (pow(2.0, 4.0 / 3.0) - 2);
}

/* rs, zeta and clamped 1 +/- zeta from spin densities. */
static void rs_zeta(const xin* v, cplx* rho, cplx* rs, cplx* z, cplx* opz, cplx* omz) {
    *rho = v->ra + v->rb;
    *rs = cpw(3.0 / (4 * PI * *rho), 1.0 / 3.0);
    *z = (v->ra - v->rb) / *rho;
    *opz = opz_clamp(1 + *z);
    *omz = opz_clamp(1 - *z);
}

/* id 7 (VWN5) and id 8 (VWN_RPA, simple f(zeta) interpolation). */
static cplx e_vwn(const xin* v, int rpa) {
    cplx rho, rs, z, opz, omz;
    rs_zeta(v, &rho, &rs, &z, &opz, &omz);
    const cplx x = csqrt(rs);
    const cplx f = fzeta(opz, omz);
    if (rpa) {
        const cplx ep = vwn_f(x, 0.0310907, 13.0720, 42.7198, -0.409286);
        const cplx ef = vwn_f(x, 0.01554535, 20.1231, 101.578, -0.743294);
        return rho * (ep + (ef - ep) * f);
    }
    const cplx ep = vwn_f(x, 0.0310907, 3.72744, 12.9352, -0.10498);
    const cplx ef = vwn_f(x, 0.01554535, 7.06042, 18.0578, -0.32500);
    const cplx ac = vwn_f(x, -1.0 / (6 * PI * PI), 1.13107, 13.0045, -0.0047584);
    const double fpp0 = 4.0 / (9.0 * (pow(2.0, 1.0 / 3.0) - 1));
    const cplx z4 = z * z * z * z;
    return rho * (ep + ac * f / fpp0 * (1 - z4) + (ef - ep) * f * z4);
}

/* PW92 G(rs) (Perdew, Wang 1992, eq. 10) and its rs derivative. */
typedef struct {
    double A, a1, b1, b2, b3, b4;
} pwpar;
static const pwpar PW_E0 = {0.0310907, 0.21370, 7.5957, 3.5876, 1.6382, 0.49294};
static const pwpar PW_E1 = {0.01554535, 0.20548, 14.1189, 6.1977, 3.3662, 0.62517};
static const pwpar PW_AC = {0.0168869, 0.11125, 10.357, 3.6231, 0.88026, 0.49671};
static const double PW_FPP = 1.709920934161365617563962776245;

static cplx pw_G(cplx rs, pwpar p) {
    const cplx srs = csqrt(rs);
    const cplx q1 = 2 * p.A * (p.b1 * srs + p.b2 * rs + p.b3 * rs * srs + p.b4 * rs * rs);
    return -2 * p.A * (1 + p.a1 * rs) * clog(1 + 1 / q1);
}
static cplx pw_dG(cplx rs, pwpar p) {
    const cplx srs = csqrt(rs);
    const cplx q1 = 2 * p.A * (p.b1 * srs + p.b2 * rs + p.b3 * rs * srs + p.b4 * rs * rs);
    const cplx dq1 = 2 * p.A * (p.b1 / (2 * srs) + p.b2 + 1.5 * p.b3 * srs + 2 * p.b4 * rs);
    return -2 * p.A * p.a1 * clog(1 + 1 / q1) + 2 * p.A * (1 + p.a1 * rs) * dq1 / (q1 * q1 + q1);
}

/* eps_c^PW92(rs, zeta) (modified parameter set) and d eps / d rs. */
static cplx pw_eps(cplx rs, cplx z, cplx opz, cplx omz, cplx* deps_drs) {
    const cplx f = fzeta(opz, omz);
    const cplx z4 = z * z * z * z;
    const cplx e0 = pw_G(rs, PW_E0), e1 = pw_G(rs, PW_E1), mac = pw_G(rs, PW_AC);
    if (deps_drs) {
        const cplx d0 = pw_dG(rs, PW_E0), d1 = pw_dG(rs, PW_E1), dmac = pw_dG(rs, PW_AC);
        *deps_drs = d0 - dmac * f * (1 - z4) / PW_FPP + (d1 - d0) * f * z4;
    }
    return e0 - mac * f * (1 - z4) / PW_FPP + (e1 - e0) * f * z4;
}

/* ------------------------------------------------------------------ GGA -- */

/* Spin-scaled exchange: sum_s 1/2 e_unif(n) F(p, alpha) with n = 2 rho_s,
 * sigma_n = 4 sigma_ss, tau_n = 2 tau_s.  p = s^2. */
typedef cplx (*fx_t)(cplx n, cplx sig, cplx tau, const double* par);

static cplx spin_exchange(const xin* v, fx_t F, const double* par) {
    cplx out = 0;
    const cplx rr[2] = {v->ra, v->rb}, ss[2] = {v->saa, v->sbb}, tt[2] = {v->ta, v->tb};
    for (int s = 0; s < 2; s++) {
        if (creal(rr[s]) <= DENS_THR * 0.5) continue;
        const cplx n = 2 * rr[s];
        out += ex_unif_half(rr[s]) * F(n, 4 * ss[s], 2 * tt[s], par);
    }
    return out;
}

static cplx p_red(cplx n, cplx sig) {
    return sig / (4 * pow(3 * PI * PI, 2.0 / 3.0) * cpw(n, 8.0 / 3.0));
}

/* PBE exchange enhancement (Perdew, Burke, Ernzerhof 1996): par = {kappa, mu}. */
static cplx fx_pbe(cplx n, cplx sig, cplx tau, const double* par) {
    (void)tau;
    const double kappa = par[0], mu = par[1];
    const cplx p = p_red(n, sig);
    return 1 + kappa - kappa / (1 + mu * p / kappa);
}

/* Becke 88 (Becke 1988) written per spin channel. */
static cplx e_b88(const xin* v) {
    const double beta = 0.0042;
    cplx out = 0;
    const cplx rr[2] = {v->ra, v->rb}, ss[2] = {v->saa, v->sbb};
    for (int s = 0; s < 2; s++) {
        if (creal(rr[s]) <= DENS_THR * 0.5) continue;
        const cplx r43 = cpw(rr[s], 4.0 / 3.0);
        const cplx x = csqrt(ss[s]) / r43;
        out += -1.5 * pow(3.0 / (4 * PI), 1.0 / 3.0) * r43 -
               beta * r43 * x * x / (1 + 6 * beta * x * casinh(x));
    }
    return out;
}

/* Lee-Yang-Parr correlation in the form of Miehlich, Savin, Stoll, Preuss 1989. */
static cplx e_lyp(const xin* v) {
    const double a = 0.04918, b = 0.132, c = 0.2533, d = 0.349;
    const double CF = 0.3 * pow(3 * PI * PI, 2.0 / 3.0);
    const cplx ra = v->ra, rb = v->rb, rho = ra + rb;
    const cplx saa = v->saa, sbb = v->sbb, sig = v->saa + 2 * v->sab + v->sbb;
    const cplx rm13 = cpw(rho, -1.0 / 3.0);
    const cplx den = 1 + d * rm13;
    const cplx omega = cexp(-c * rm13) / den * cpw(rho, -11.0 / 3.0);
    const cplx delta = c * rm13 + d * rm13 / den;
    const cplx t1 = -a * 4 / den * ra * rb / rho;
    const cplx inner = ra * rb * (pow(2.0, 11.0 / 3.0) * CF * (cpw(ra, 8.0 / 3.0) + cpw(rb, 8.0 / 3.0)) +
                                  (47.0 / 18 - 7 * delta / 18) * sig - (2.5 - delta / 18) * (saa + sbb) -
                                  (delta - 11) / 9 * (ra / rho * saa + rb / rho * sbb)) -
                       2.0 / 3 * rho * rho * sig + (2.0 / 3 * rho * rho - ra * ra) * sbb +
                       (2.0 / 3 * rho * rho - rb * rb) * saa;
    return t1 - a * b * omega * inner;
}

/* PBE correlation energy per particle for total density rho, zeta, total
 * sigma (Perdew, Burke, Ernzerhof 1996), beta given. */
static cplx pbe_c_eps(cplx rho, cplx z, cplx opz, cplx omz, cplx sig, double beta) {
    const double gamma = (1 - log(2.0)) / (PI * PI);
    const cplx rs = cpw(3.0 / (4 * PI * rho), 1.0 / 3.0);
    const cplx ec = pw_eps(rs, z, opz, omz, NULL);
    const cplx phi = (cpw(opz, 2.0 / 3.0) + cpw(omz, 2.0 / 3.0)) / 2;
    const cplx phi3 = phi * phi * phi;
    const cplx kf = cpw(3 * PI * PI * rho, 1.0 / 3.0);
    const cplx t2 = sig * PI / (16 * phi * phi * kf * rho * rho);
    const cplx A = beta / gamma / (cexp(-ec / (gamma * phi3)) - 1);
    const cplx At2 = A * t2;
    const cplx H = gamma * phi3 * clog(1 + beta / gamma * t2 * (1 + At2) / (1 + At2 + At2 * At2));
    return ec + H;
}

static cplx e_pbe_c(const xin* v, double beta) {
    cplx rho, rs, z, opz, omz;
    rs_zeta(v, &rho, &rs, &z, &opz, &omz);
    const cplx sig = v->saa + 2 * v->sab + v->sbb;
    return rho * pbe_c_eps(rho, z, opz, omz, sig, beta);
}

/* ----------------------------------------------------------------- mGGA -- */

/* TPSS exchange enhancement (Tao, Perdew, Staroverov, Scuseria 2003, eqs. 4-10). */
static cplx fx_tpss(cplx n, cplx sig, cplx tau, const double* par) {
    (void)par;
    const double b = 0.40, c = 1.59096, e = 1.537, kappa = 0.804, mu = 0.21951;
    const cplx p = p_red(n, sig);
    const cplx tauw = sig / (8 * n);
    const cplx z = tauw / tau;
    const cplx tunif = 0.3 * pow(3 * PI * PI, 2.0 / 3.0) * cpw(n, 5.0 / 3.0);
    const cplx alpha = (tau - tauw) / tunif;
    const cplx qb = 0.45 * (alpha - 1) / csqrt(1 + b * alpha * (alpha - 1)) + 2 * p / 3;
    const cplx z2 = z * z;
    const double se = sqrt(e);
    const cplx num = (10.0 / 81 + c * z2 / ((1 + z2) * (1 + z2))) * p + 146.0 / 2025 * qb * qb -
                     73.0 / 405 * qb * csqrt(0.5 * (0.6 * z) * (0.6 * z) + 0.5 * p * p) +
                     (1 / kappa) * (10.0 / 81) * (10.0 / 81) * p * p +
                     2 * se * 10.0 / 81 * (0.6 * z) * (0.6 * z) + e * mu * p * p * p;
    const cplx x = num / ((1 + se * p) * (1 + se * p));
    return 1 + kappa - kappa / (1 + x / kappa);
}

/* TPSS correlation (same paper, eqs. 11-14) on top of PBE correlation. */
static cplx e_tpss_c(const xin* v) {
    const double beta = 0.06672455060314922, d = 2.8;
    cplx rho, rs, z, opz, omz;
    rs_zeta(v, &rho, &rs, &z, &opz, &omz);
    const cplx sig = v->saa + 2 * v->sab + v->sbb;
    const cplx tau = v->ta + v->tb;
    const cplx epbe = pbe_c_eps(rho, z, opz, omz, sig, beta);
    /* xi^2 = |grad zeta|^2 / (4 (3 pi^2 rho)^(2/3)),
     * |grad zeta|^2 = 4 (rb^2 saa - 2 ra rb sab + ra^2 sbb) / rho^4 */
    const cplx gz2 = 4 * (v->rb * v->rb * v->saa - 2 * v->ra * v->rb * v->sab + v->ra * v->ra * v->sbb) /
                     (rho * rho * rho * rho);
    const cplx xi2 = gz2 / (4 * cpw(3 * PI * PI * rho, 2.0 / 3.0));
    const cplx z2_ = z * z;
    const cplx C0 = 0.53 + 0.87 * z2_ + 0.50 * z2_ * z2_ + 2.26 * z2_ * z2_ * z2_;
    const cplx den = 1 + xi2 * (cpw(opz, -4.0 / 3.0) + cpw(omz, -4.0 / 3.0)) / 2;
    const cplx C = C0 / (den * den * den * den);
    /* single-spin PBE correlation, fully polarized */
    const cplx rr[2] = {v->ra, v->rb}, ss[2] = {v->saa, v->sbb};
    cplx sum = 0;
    for (int s = 0; s < 2; s++) {
        if (creal(rr[s]) <= DENS_THR * 0.5) continue;
        const cplx es = pbe_c_eps(rr[s], 1.0, 2.0, ZETA_THR, ss[s], beta);
        sum += rr[s] / rho * cmaxr(es, epbe);
    }
    const cplx tauw = sig / (8 * rho);
    const cplx zz = tauw / tau;
    const cplx zz2 = zz * zz;
    const cplx erev = epbe * (1 + C * zz2) - (1 + C) * zz2 * sum;
    return rho * erev * (1 + d * erev * zz2 * zz);
}

/* r2SCAN (Furness, Kaplan, Ning, Perdew, Sun 2020). */
static const double R2_CX[8] = {1.0, -0.667, -0.4445555, -0.663086601049, 1.451297044490,
                                -0.887998041597, 0.234528941479, -0.023185843322};
static const double R2_CC[8] = {1.0, -0.64, -0.4352, -1.535685604549, 3.061560252175,
                                -1.915710236206, 0.516884468372, -0.051848879792};
static const double R2_ETA = 0.001, R2_DP2 = 0.361;

static cplx r2_interp(cplx a, const double* cc, double d, double c2) {
    if (creal(a) <= 2.5) {
        cplx s = 0, ap = 1;
        for (int i = 0; i < 8; i++) {
            s += cc[i] * ap;
            ap *= a;
        }
        return s;
    }
    return -d * cexp(c2 / (1 - a));
}

static double r2_dfsum(const double* cc) {
    double s = 0;
    for (int i = 1; i < 8; i++) s += i * cc[i];
    return s;
}

static cplx fx_r2scan(cplx n, cplx sig, cplx tau, const double* par) {
    (void)par;
    const double k1 = 0.065, hx0 = 1.174, a1 = 4.9479, dx = 1.24, c2x = 0.8;
    const double mu_ak = 10.0 / 81;
    const double Ceta = 20.0 / 27 + R2_ETA * 5.0 / 3;
    const double C2 = -r2_dfsum(R2_CX) * (1 - hx0);
    const cplx p = p_red(n, sig);
    const cplx tauw = sig / (8 * n);
    const cplx tunif = 0.3 * pow(3 * PI * PI, 2.0 / 3.0) * cpw(n, 5.0 / 3.0);
    const cplx ab = (tau - tauw) / (tunif + R2_ETA * tauw);
    const double dp24 = R2_DP2 * R2_DP2 * R2_DP2 * R2_DP2;
    const cplx x = (Ceta * C2 * cexp(-p * p / dp24) + mu_ak) * p;
    const cplx hx1 = 1 + k1 - k1 / (1 + x / k1);
    const cplx fx = r2_interp(ab, R2_CX, dx, c2x);
    const cplx gx = 1 - cexp(-a1 / cpw(p, 0.25));
    return (hx1 + fx * (hx0 - hx1)) * gx;
}

static cplx e_r2scan_c(const xin* v) {
    const double b1c = 0.0285764, b2c = 0.0889, b3c = 0.125541, chi = 0.128026;
    const double dc = 0.7, c2c = 1.5;
    const double gamma = (1 - log(2.0)) / (PI * PI);
    cplx rho, rs, z, opz, omz;
    rs_zeta(v, &rho, &rs, &z, &opz, &omz);
    const cplx sig = v->saa + 2 * v->sab + v->sbb;
    const cplx tau = v->ta + v->tb;
    const cplx phi = (cpw(opz, 2.0 / 3.0) + cpw(omz, 2.0 / 3.0)) / 2;
    const cplx phi3 = phi * phi * phi;
    const cplx ds = (cpw(opz, 5.0 / 3.0) + cpw(omz, 5.0 / 3.0)) / 2;
    const cplx dxz = (cpw(opz, 4.0 / 3.0) + cpw(omz, 4.0 / 3.0)) / 2;
    const cplx p = sig / (4 * pow(3 * PI * PI, 2.0 / 3.0) * cpw(rho, 8.0 / 3.0));
    const cplx kf = cpw(3 * PI * PI * rho, 1.0 / 3.0);
    const cplx t2 = sig * PI / (16 * phi * phi * kf * rho * rho);
    /* eps_c^1 (alpha = 1 limit) */
    cplx de1;
    const cplx e1 = pw_eps(rs, z, opz, omz, &de1);
    const cplx w1 = cexp(-e1 / (gamma * phi3)) - 1;
    const cplx betars = 0.066725 * (1 + 0.1 * rs) / (1 + 0.1778 * rs);
    const cplx y = betars / (gamma * w1) * t2;
    /* eps_c^0 (alpha = 0 limit) */
    const cplx srs = csqrt(rs);
    const cplx dd = 1 + b2c * srs + b3c * rs;
    const cplx elda0 = -b1c / dd;
    const cplx delda0 = b1c * (b2c / (2 * srs) + b3c) / (dd * dd);
    const cplx z2 = z * z, z4 = z2 * z2;
    const cplx z12 = z4 * z4 * z4;
    const cplx Gc = (1 - 2.3631 * (dxz - 1)) * (1 - z12);
    const cplx w0 = cexp(-elda0 / b1c) - 1;
    const cplx ginf = cpw(1 + 4 * chi * p, -0.25);
    const cplx H0 = b1c * clog(1 + w0 * (1 - ginf));
    const cplx e0 = (elda0 + H0) * Gc;
    /* gradient-expansion restoring shift of y */
    const double dfc2 = r2_dfsum(R2_CC);
    const double dp24 = R2_DP2 * R2_DP2 * R2_DP2 * R2_DP2;
    const cplx dy = dfc2 / (27 * gamma * ds * phi3 * w1) *
                    (20 * rs * (delda0 * Gc - de1) - 45 * R2_ETA * (elda0 * Gc - e1)) * p *
                    cexp(-p * p / dp24);
    const cplx g = cpw(1 + 4 * (y - dy), -0.25);
    const cplx H1 = gamma * phi3 * clog(1 + w1 * (1 - g));
    const cplx ec1 = e1 + H1;
    /* interpolation in alpha-bar */
    const cplx tauw = sig / (8 * rho);
    const cplx tunif = 0.3 * pow(3 * PI * PI, 2.0 / 3.0) * cpw(rho, 5.0 / 3.0) * ds;
    const cplx ab = (tau - tauw) / (tunif + R2_ETA * tauw);
    const cplx fc = r2_interp(ab, R2_CC, dc, c2c);
    return rho * (ec1 + fc * (e0 - ec1));
}

/* ----------------------------------------------------------- registry -- */

static const double PBE_PAR[2] = {0.8040, 0.2195149727645171};
static const double PBE_G_PAR[2] = {0.804, 0.2195164512208958};

/* Energy density of one libxc id; *family is 0 LDA, 1 GGA, 2 mGGA. */
static int e_id(int id, const xin* v, cplx* e, int* family) {
    switch (id) {
        case 1: *family = 0; *e = e_lda_x(v); return 0;
        case 7: *family = 0; *e = e_vwn(v, 0); return 0;
        case 8: *family = 0; *e = e_vwn(v, 1); return 0;
        case 101: *family = 1; *e = spin_exchange(v, fx_pbe, PBE_PAR); return 0;
        case 130: *family = 1; *e = e_pbe_c(v, 0.06672455060314922); return 0;
        case 321: *family = 1; *e = spin_exchange(v, fx_pbe, PBE_G_PAR); return 0;
        case 322: *family = 1; *e = e_pbe_c(v, 0.066725); return 0;
        case 106: *family = 1; *e = e_b88(v); return 0;
        case 131: *family = 1; *e = e_lyp(v); return 0;
        case 402: /* B3LYP: 0.08 Slater + 0.72 B88 + 0.19 VWN_RPA + 0.81 LYP */
            *family = 1;
            *e = 0.08 * e_lda_x(v) + 0.72 * e_b88(v) + 0.19 * e_vwn(v, 1) + 0.81 * e_lyp(v);
            return 0;
        case 406: /* PBE0 */
            *family = 1;
            *e = 0.75 * spin_exchange(v, fx_pbe, PBE_PAR) + e_pbe_c(v, 0.06672455060314922);
            return 0;
        case 436: /* BHandHLYP */
            *family = 1;
            *e = 0.5 * e_b88(v) + e_lyp(v);
            return 0;
        case 202: *family = 2; *e = spin_exchange(v, fx_tpss, NULL); return 0;
        case 231: *family = 2; *e = e_tpss_c(v); return 0;
        case 457: /* TPSSh */
            *family = 2;
            *e = 0.9 * spin_exchange(v, fx_tpss, NULL) + e_tpss_c(v);
            return 0;
        case 497: *family = 2; *e = spin_exchange(v, fx_r2scan, NULL); return 0;
        case 498: *family = 2; *e = e_r2scan_c(v); return 0;
    }
    return -1;
}

/* Threshold-conditioned polarized inputs (on real parts; a clamped input
 * becomes a constant and loses its derivative, as in libxc). */
static xin condition_pol(xin v, int mgga) {
    v.ra = cmaxr(v.ra, DENS_THR);
    v.rb = cmaxr(v.rb, DENS_THR);
    const double sthr = pow(DENS_THR, 8.0 / 3.0);
    v.saa = cmaxr(v.saa, sthr);
    v.sbb = cmaxr(v.sbb, sthr);
    if (mgga) {
        v.ta = cmaxr(v.ta, TAU_THR);
        v.tb = cmaxr(v.tb, TAU_THR);
        v.saa = cminr(v.saa, 8 * v.ra * v.ta);
        v.sbb = cminr(v.sbb, 8 * v.rb * v.tb);
    }
    const cplx half = (v.saa + v.sbb) / 2;
    v.sab = cmaxr(cminr(v.sab, half), -half);
    return v;
}

/* Unpolarized inputs (total rho, sigma, tau) mapped onto equal spin halves. */
static xin from_unpol(cplx rho, cplx sig, cplx tau, int mgga) {
    sig = cmaxr(sig, pow(DENS_THR, 8.0 / 3.0));
    if (mgga) {
        tau = cmaxr(tau, TAU_THR);
        sig = cminr(sig, 8 * rho * tau);
    }
    xin v = {rho / 2, rho / 2, sig / 4, sig / 4, sig / 4, tau / 2, tau / 2};
    return v;
}

static cplx e_sum(int nids, const int* ids, const xin* v, int* bad) {
    cplx e = 0;
    for (int i = 0; i < nids; i++) {
        cplx ei;
        int fam;
        if (e_id(ids[i], v, &ei, &fam)) *bad = 1;
        else e += ei;
    }
    return e;
}

static int family_of(int nids, const int* ids) {
    int fam = 0;
    xin v = {0.1, 0.1, 0.01, 0.01, 0.01, 0.1, 0.1};
    for (int i = 0; i < nids; i++) {
        cplx e;
        int f = 0;
        if (e_id(ids[i], &v, &e, &f)) return -1;
        if (f > fam) fam = f;
    }
    return fam;
}

static double step(cplx x) {
    const double a = fabs(creal(x));
    return a > 1e-200 ? 1e-20 * a : 1e-220;
}

int oracle_functional(int nids, const int* ids, int ns, int ng, const double* rho,
                      const double* sigma, const double* tau, double* eps, double* vrho,
                      double* vsigma, double* vtau) {
    const int fam = family_of(nids, ids);
    if (fam < 0) return -1;
    const int mgga = fam >= 2;
    int bad = 0;
    for (int g = 0; g < ng; g++) {
        if (ns == 1) {
            const double r = rho[g];
            const double s = fam >= 1 ? sigma[g] : 0;
            const double t = mgga ? tau[g] : 0;
            eps[g] = 0;
            vrho[g] = 0;
            if (fam >= 1) vsigma[g] = 0;
            if (mgga) vtau[g] = 0;
            if (r < DENS_THR) continue;
            const double x[3] = {r, s, t};
            const int nin = mgga ? 3 : (fam >= 1 ? 2 : 1);
            xin v = from_unpol(x[0], x[1], x[2], mgga);
            const double e0 = creal(e_sum(nids, ids, &v, &bad));
            eps[g] = e0 / r;
            double d[3] = {0, 0, 0};
            for (int k = 0; k < nin; k++) {
                cplx xc[3] = {x[0], x[1], x[2]};
                const double h = step(x[k]);
                xc[k] += I * h;
                xin vk = from_unpol(xc[0], xc[1], xc[2], mgga);
                d[k] = cimag(e_sum(nids, ids, &vk, &bad)) / h;
            }
            vrho[g] = d[0];
            if (fam >= 1) vsigma[g] = d[1];
            if (mgga) vtau[g] = d[2];
        } else {
            const double x[7] = {rho[g], rho[ng + g], fam >= 1 ? sigma[g] : 0,
                                 fam >= 1 ? sigma[ng + g] : 0, fam >= 1 ? sigma[2 * ng + g] : 0,
                                 mgga ? tau[g] : 0, mgga ? tau[ng + g] : 0};
            eps[g] = 0;
            vrho[g] = vrho[ng + g] = 0;
            if (fam >= 1) vsigma[g] = vsigma[ng + g] = vsigma[2 * ng + g] = 0;
            if (mgga) vtau[g] = vtau[ng + g] = 0;
            const double rt = x[0] + x[1];
            if (rt < DENS_THR) continue;
            xin v0 = {x[0], x[1], x[2], x[3], x[4], x[5], x[6]};
            xin vc = condition_pol(v0, mgga);
            eps[g] = creal(e_sum(nids, ids, &vc, &bad)) / rt;
            const int idx[7] = {0, 1, 2, 3, 4, 5, 6};
            const int nin = mgga ? 7 : (fam >= 1 ? 5 : 2);
            double d[7] = {0};
            for (int k = 0; k < nin; k++) {
                cplx xc[7];
                for (int j = 0; j < 7; j++) xc[j] = x[j];
                const double h = step(x[idx[k]]);
                xc[idx[k]] += I * h;
                xin vk = {xc[0], xc[1], xc[2], xc[3], xc[4], xc[5], xc[6]};
                vk = condition_pol(vk, mgga);
                d[k] = cimag(e_sum(nids, ids, &vk, &bad)) / h;
            }
            vrho[g] = d[0];
            vrho[ng + g] = d[1];
            if (fam >= 1) {
                vsigma[g] = d[2];
                vsigma[ng + g] = d[3];
                vsigma[2 * ng + g] = d[4];
            }
            if (mgga) {
                vtau[g] = d[5];
                vtau[ng + g] = d[6];
            }
        }
    }
    return bad ? -1 : 0;
}

/* Single-point evaluation used by tests: returns e (energy per volume). */
double oracle_functional_point(int nids, const int* ids, int ns, const double* in) {
    const int fam = family_of(nids, ids);
    int bad = 0;
    if (ns == 1) {
        xin v = from_unpol(in[0], in[1], in[2], fam >= 2);
        return creal(e_sum(nids, ids, &v, &bad));
    }
    xin v = {in[0], in[1], in[2], in[3], in[4], in[5], in[6]};
    v = condition_pol(v, fam >= 2);
    return creal(e_sum(nids, ids, &v, &bad));
}

/* Second derivatives (order "f", ExchangeCorrelation.cpp:101-133): the
 * complex-step first derivative g_i = Im e(x + i h e_i) / h, differentiated
 * in x_j by differences combined by Richardson extrapolation.  A mixed entry
 * comes from the better-conditioned of d g_i / d x_j and d g_j / d x_i: the
 * step along the input with the larger |x g| (a step of 1e-3 sigma at a tiny
 * sigma moves v_rho by less than its rounding, while the step along rho moves
 * v_sigma well).  Central steps d, d/2, d/4 (d = 1e-2 |x_j|, error O(d^6)), except
 * for a sigma input of a polarized point whose step could cross the clamp
 * |sigma_ab| <= (sigma_aa + sigma_bb) / 2 (gradients of the two spins nearly
 * parallel and equal, as near a nucleus): there one-sided steps s, s/2, s/4
 * away from the clamp (s = 1e-4 |x_j|, error O(s^3)).  Outputs in libxc's
 * layouts, component-major [k][g] (see xc_oracle.h). */
static void grad_cs(int nids, const int* ids, int ns, const double* x, int nin, double* gout, int* bad) {
    for (int k = 0; k < nin; k++) {
        cplx xc[7];
        for (int j = 0; j < 7; j++) xc[j] = x[j];
        const double h = step(x[k]);
        xc[k] += I * h;
        xin v;
        if (ns == 1) v = from_unpol(xc[0], xc[1], xc[2], 0);
        else {
            xin v0 = {xc[0], xc[1], xc[2], xc[3], xc[4], xc[5], xc[6]};
            v = condition_pol(v0, 0);
        }
        gout[k] = cimag(e_sum(nids, ids, &v, bad)) / h;
    }
}

/* column j of the Hessian: d g / d x_j; dir 0 central, +-1 one-sided */
static void hess_col(int nids, const int* ids, int ns, const double* x, int nin, int j, int dir, double* col,
                     int* bad) {
    double xs[7], a[5], b[5], c[5], e[5];
    /* sigma_ab enters through sigma_aa + 2 sigma_ab + sigma_bb and is smooth
     * through zero: its step follows the larger of |sigma_ab| and a tenth of
     * (sigma_aa + sigma_bb) / 2 */
    const double scale = (ns == 2 && j == 3) ? fmax(fabs(x[3]), 0.05 * (x[2] + x[4])) : fabs(x[j]);
    if (dir == 0) {
        /* central differences with steps d, d/2, d/4 and two Richardson levels (error O(d^6)) */
        const double d = scale > 0 ? 1e-2 * scale : 1e-30;
        double cd[3][5];
        for (int l = 0; l < 3; l++) {
            const double h = d / (double)(1 << l);
            memcpy(xs, x, sizeof(xs));
            xs[j] += h;
            grad_cs(nids, ids, ns, xs, nin, a, bad);
            memcpy(xs, x, sizeof(xs));
            xs[j] -= h;
            grad_cs(nids, ids, ns, xs, nin, b, bad);
            for (int i = 0; i < nin; i++) cd[l][i] = (a[i] - b[i]) / (2 * h);
        }
        for (int i = 0; i < nin; i++) {
            const double r1 = (4 * cd[1][i] - cd[0][i]) / 3, r2 = (4 * cd[2][i] - cd[1][i]) / 3;
            col[i] = (16 * r2 - r1) / 15;
        }
        return;
    }
    const double s = dir * (scale > 0 ? 1e-4 * scale : 1e-30);
    const double st[3] = {s, 0.5 * s, 0.25 * s};
    double* out[3] = {a, b, c};
    grad_cs(nids, ids, ns, x, nin, e, bad);
    for (int k = 0; k < 3; k++) {
        memcpy(xs, x, sizeof(xs));
        xs[j] += st[k];
        grad_cs(nids, ids, ns, xs, nin, out[k], bad);
    }
    for (int i = 0; i < nin; i++) {
        const double D1 = (a[i] - e[i]) / s, D2 = (b[i] - e[i]) / (0.5 * s), D4 = (c[i] - e[i]) / (0.25 * s);
        const double R1 = 2 * D2 - D1, R2 = 2 * D4 - D2;
        col[i] = (4 * R2 - R1) / 3;
    }
}

int oracle_functional_fxc(int nids, const int* ids, int ns, int ng, const double* rho, const double* sigma,
                          double* v2rho2, double* v2rhosigma, double* v2sigma2) {
    const int fam = family_of(nids, ids);
    if (fam < 0 || fam > 1) return -1;
    const int nrr = ns == 1 ? 1 : 3, nrs = ns == 1 ? 1 : 6;
    for (long i = 0; i < (long)nrr * ng; i++) v2rho2[i] = 0;
    if (fam >= 1)
        for (long i = 0; i < (long)nrs * ng; i++) v2rhosigma[i] = v2sigma2[i] = 0;
    int bad = 0;
    for (int g = 0; g < ng; g++) {
        double x[7] = {0, 0, 0, 0, 0, 0, 0};
        int nin;
        if (ns == 1) {
            x[0] = rho[g];
            x[1] = fam >= 1 ? sigma[g] : 0;
            nin = fam >= 1 ? 2 : 1;
            if (x[0] < DENS_THR) continue;
        } else {
            x[0] = rho[g];
            x[1] = rho[ng + g];
            if (fam >= 1) {
                x[2] = sigma[g];
                x[3] = sigma[ng + g];
                x[4] = sigma[2 * ng + g];
            }
            nin = fam >= 1 ? 5 : 2;
            if (x[0] + x[1] < DENS_THR) continue;
        }
        double H[5][5];
        const double gap = 0.5 * (x[2] + x[4]) - fabs(x[3]);
        for (int j = 0; j < nin; j++) {
            int dir = 0;
            const double sc = j == 3 ? fmax(fabs(x[3]), 0.05 * (x[2] + x[4])) : fabs(x[j]);
            if (ns == 2 && j >= 2 && gap < 2e-2 * (sc + fabs(x[3]))) {
                if (j == 3) dir = x[3] >= 0 ? -1 : 1;  /* shrink |sigma_ab| */
                else dir = 1;                           /* grow sigma_aa / sigma_bb */
            }
            double col[5];
            hess_col(nids, ids, ns, x, nin, j, dir, col, &bad);
            for (int i = 0; i < nin; i++) H[i][j] = col[i];
        }
        double g0[5], S[5][5];
        grad_cs(nids, ids, ns, x, nin, g0, &bad);
        for (int i = 0; i < nin; i++)
            for (int j = 0; j < nin; j++)
                S[i][j] = fabs(x[j] * g0[j]) >= fabs(x[i] * g0[i]) ? H[i][j] : H[j][i];
        if (ns == 1) {
            v2rho2[g] = S[0][0];
            if (fam >= 1) {
                v2rhosigma[g] = S[0][1];
                v2sigma2[g] = S[1][1];
            }
        } else {
            v2rho2[g] = S[0][0];
            v2rho2[ng + g] = S[0][1];
            v2rho2[2 * ng + g] = S[1][1];
            if (fam >= 1) {
                for (int a = 0; a < 2; a++)
                    for (int xx = 0; xx < 3; xx++) v2rhosigma[(long)(3 * a + xx) * ng + g] = S[a][2 + xx];
                int k = 0;
                for (int p = 2; p < 5; p++)
                    for (int q = p; q < 5; q++) v2sigma2[(long)(k++) * ng + g] = S[p][q];
            }
        }
    }
    return bad ? -1 : 0;
}
