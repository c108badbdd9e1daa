// One- and two-electron Gaussian integrals for the SCF caller of the XC
// build (the role of the reference's libint2 layer, src/Integral/Int2C1E.cpp
// and Int4C2E.cpp): overlap, kinetic, nuclear attraction and electron
// repulsion over the same contracted shells the grid evaluates (libint2
// contraction normalisation, real solid harmonics, Cartesian P shells).
//
// Method: McMurchie-Davidson.  Products of Cartesian Gaussians are expanded
// in Hermite Gaussians (E coefficients, by the two-term recursion); Coulomb
// integrals use the Hermite integrals R_tuv built from the Boys function.
// Cartesian results are transformed to the pure functions with the solid
// harmonic table.  Host code, OpenMP over shell pairs / quartets.
#include <cmath>
#include <cstring>
#include <vector>

#include "common.h"
#include "model.h"
#include "xc_state.h"
#include "eri.h"

namespace cgb {
namespace {

constexpr int kMaxLInt = 4;
constexpr int kMaxHerm = 4 * kMaxLInt + 1;

struct CShell {
    int l, nfunc, ncart, first;
    double A[3];
    std::vector<double> exps, coefs;
    std::vector<int> ca, cb, cc;    // Cartesian exponents, canonical order
    std::vector<double> T;          // nfunc x ncart pure transform
};

std::vector<CShell> make_shells(const BasisSet& b) {
    static double table[kMaxL + 1][2 * kMaxL + 1][(kMaxL + 1) * (kMaxL + 2) / 2];
    static bool init = false;
    if (!init) {
        solid_harmonic_table(table);
        init = true;
    }
    std::vector<CShell> out;
    for (const Shell& s : b.shells) {
        CShell c;
        c.l = s.l;
        c.first = s.first;
        c.nfunc = shell_size(s.type);
        c.ncart = (s.l + 1) * (s.l + 2) / 2;
        c.A[0] = s.x;
        c.A[1] = s.y;
        c.A[2] = s.z;
        c.exps.assign(b.exps.begin() + s.prim_off, b.exps.begin() + s.prim_off + s.nprim);
        c.coefs.assign(b.coefs.begin() + s.prim_off, b.coefs.begin() + s.prim_off + s.nprim);
        for (int a = s.l; a >= 0; a--)
            for (int bb = s.l - a; bb >= 0; bb--) {
                c.ca.push_back(a);
                c.cb.push_back(bb);
                c.cc.push_back(s.l - a - bb);
            }
        c.T.assign((size_t)c.nfunc * c.ncart, 0.0);
        for (int f = 0; f < c.nfunc; f++) {
            const int row = (s.type == 1) ? (f == 0 ? 2 : f - 1) : f;  // Cartesian P: x, y, z
            for (int k = 0; k < c.ncart; k++) c.T[(size_t)f * c.ncart + k] = table[s.l][row][k];
        }
        out.push_back(std::move(c));
    }
    return out;
}

// Boys function F_n(T), n = 0..nmax.
void boys(int nmax, double T, double* F) {
    if (T < 1e-15) {
        for (int n = 0; n <= nmax; n++) F[n] = 1.0 / (2 * n + 1);
        return;
    }
    if (T > 36.0) {
        F[0] = 0.5 * std::sqrt(M_PI / T);
        for (int n = 1; n <= nmax; n++) F[n] = F[n - 1] * (2 * n - 1) / (2 * T);
        return;
    }
    double term = 1.0 / (2 * nmax + 1), sum = term;
    for (int i = 1; i < 400; i++) {
        term *= 2 * T / (2 * nmax + 2 * i + 1);
        sum += term;
        if (term < 1e-17 * sum) break;
    }
    const double et = std::exp(-T);
    F[nmax] = et * sum;
    for (int n = nmax; n > 0; n--) F[n - 1] = (2 * T * F[n] + et) / (2 * n - 1);
}

// Hermite expansion coefficients of one Cartesian direction:
// E[i][j][t], i <= la, j <= lb, t <= i + j.
struct Herm1 {
    double E[kMaxLInt + 3][kMaxLInt + 3][2 * kMaxLInt + 5];
};

void hermite_e(int la, int lb, double a, double b, double Ax, double Bx, Herm1& h) {
    const double p = a + b, mu = a * b / p, X = Ax - Bx;
    const double Px = (a * Ax + b * Bx) / p, XPA = Px - Ax, XPB = Px - Bx, i2p = 0.5 / p;
    for (int i = 0; i <= la; i++)
        for (int j = 0; j <= lb; j++)
            for (int t = 0; t <= la + lb + 1; t++) h.E[i][j][t] = 0;
    h.E[0][0][0] = std::exp(-mu * X * X);
    for (int i = 0; i <= la; i++)
        for (int j = 0; j <= lb; j++) {
            if (i == 0 && j == 0) continue;
            for (int t = 0; t <= i + j; t++) {
                double v;
                if (i > 0) {
                    v = XPA * h.E[i - 1][j][t];
                    if (t > 0) v += i2p * h.E[i - 1][j][t - 1];
                    if (t + 1 <= i - 1 + j) v += (t + 1) * h.E[i - 1][j][t + 1];
                } else {
                    v = XPB * h.E[i][j - 1][t];
                    if (t > 0) v += i2p * h.E[i][j - 1][t - 1];
                    if (t + 1 <= i + j - 1) v += (t + 1) * h.E[i][j - 1][t + 1];
                }
                h.E[i][j][t] = v;
            }
        }
}

// Hermite Coulomb integrals R_{tuv} (n = 0) for t + u + v <= L.
struct HermR {
    double R[kMaxHerm + 1][kMaxHerm + 1][kMaxHerm + 1];
};

void hermite_r(int L, double alpha, double X, double Y, double Z, HermR& out) {
    static thread_local double R[kMaxHerm + 1][kMaxHerm + 1][kMaxHerm + 1][kMaxHerm + 1];  // [n][t][u][v]
    double F[kMaxHerm + 2];
    boys(L, alpha * (X * X + Y * Y + Z * Z), F);
    double m2a = 1.0;
    for (int n = 0; n <= L; n++) {
        R[n][0][0][0] = m2a * F[n];
        m2a *= -2 * alpha;
    }
    for (int n = L - 1; n >= 0; n--) {
        const int top = L - n;
        for (int t = 0; t <= top; t++)
            for (int u = 0; u + t <= top; u++)
                for (int v = 0; v + u + t <= top; v++) {
                    if (t + u + v == 0) continue;
                    double val;
                    if (t > 0) {
                        val = X * R[n + 1][t - 1][u][v];
                        if (t > 1) val += (t - 1) * R[n + 1][t - 2][u][v];
                    } else if (u > 0) {
                        val = Y * R[n + 1][t][u - 1][v];
                        if (u > 1) val += (u - 1) * R[n + 1][t][u - 2][v];
                    } else {
                        val = Z * R[n + 1][t][u][v - 1];
                        if (v > 1) val += (v - 1) * R[n + 1][t][u][v - 2];
                    }
                    R[n][t][u][v] = val;
                }
    }
    for (int t = 0; t <= L; t++)
        for (int u = 0; u + t <= L; u++)
            for (int v = 0; v + u + t <= L; v++) out.R[t][u][v] = R[0][t][u][v];
}

// Cartesian block -> pure block: out(f1, f2) = sum T1(f1,k1) T2(f2,k2) in(k1,k2).
void to_pure2(const CShell& s1, const CShell& s2, const double* cart, double* pure) {
    for (int f1 = 0; f1 < s1.nfunc; f1++)
        for (int f2 = 0; f2 < s2.nfunc; f2++) {
            double acc = 0;
            for (int k1 = 0; k1 < s1.ncart; k1++) {
                const double t1 = s1.T[(size_t)f1 * s1.ncart + k1];
                if (t1 == 0) continue;
                for (int k2 = 0; k2 < s2.ncart; k2++) acc += t1 * s2.T[(size_t)f2 * s2.ncart + k2] * cart[k1 * s2.ncart + k2];
            }
            pure[f1 * s2.nfunc + f2] = acc;
        }
}

// S, T, V(nuc) Cartesian blocks of a shell pair.
void one_e_pair(const CShell& a, const CShell& b, const BasisSet& bs, double* S, double* Tk, double* V) {
    const int na = a.ncart, nb = b.ncart;
    std::fill(S, S + na * nb, 0.0);
    std::fill(Tk, Tk + na * nb, 0.0);
    std::fill(V, V + na * nb, 0.0);
    Herm1 hx, hy, hz;
    HermR hr;
    for (size_t pa = 0; pa < a.exps.size(); pa++)
        for (size_t pb = 0; pb < b.exps.size(); pb++) {
            const double ea = a.exps[pa], eb = b.exps[pb], p = ea + eb;
            const double cab = a.coefs[pa] * b.coefs[pb];
            // b shell raised by 2 for the kinetic term
            hermite_e(a.l, b.l + 2, ea, eb, a.A[0], b.A[0], hx);
            hermite_e(a.l, b.l + 2, ea, eb, a.A[1], b.A[1], hy);
            hermite_e(a.l, b.l + 2, ea, eb, a.A[2], b.A[2], hz);
            const double sp = std::sqrt(M_PI / p);
            auto s1 = [&](const Herm1& h, int i, int j) { return j < 0 ? 0.0 : h.E[i][j][0] * sp; };
            auto t1 = [&](const Herm1& h, int i, int j) {
                // <i| d2/dx2 |j> = j(j-1) S(i,j-2) - 2b(2j+1) S(i,j) + 4b^2 S(i,j+2)
                return j * (j - 1) * s1(h, i, j - 2) - 2 * eb * (2 * j + 1) * s1(h, i, j) + 4 * eb * eb * s1(h, i, j + 2);
            };
            const double P[3] = {(ea * a.A[0] + eb * b.A[0]) / p, (ea * a.A[1] + eb * b.A[1]) / p,
                                 (ea * a.A[2] + eb * b.A[2]) / p};
            for (int ka = 0; ka < na; ka++)
                for (int kb = 0; kb < nb; kb++) {
                    const int ia = a.ca[ka], ja = a.cb[ka], la = a.cc[ka];
                    const int ib = b.ca[kb], jb = b.cb[kb], lb = b.cc[kb];
                    const double sx = s1(hx, ia, ib), sy = s1(hy, ja, jb), sz = s1(hz, la, lb);
                    S[ka * nb + kb] += cab * sx * sy * sz;
                    Tk[ka * nb + kb] += cab * -0.5 * (t1(hx, ia, ib) * sy * sz + sx * t1(hy, ja, jb) * sz + sx * sy * t1(hz, la, lb));
                }
            const int L = a.l + b.l;
            for (int at = 0; at < bs.natoms(); at++) {
                const double Zc = bs.Z[at];
                hermite_r(L, p, P[0] - bs.xyz[3 * at], P[1] - bs.xyz[3 * at + 1], P[2] - bs.xyz[3 * at + 2], hr);
                const double pre = -Zc * 2 * M_PI / p * cab;
                for (int ka = 0; ka < na; ka++)
                    for (int kb = 0; kb < nb; kb++) {
                        const int ia = a.ca[ka], ja = a.cb[ka], la = a.cc[ka];
                        const int ib = b.ca[kb], jb = b.cb[kb], lb = b.cc[kb];
                        double acc = 0;
                        for (int t = 0; t <= ia + ib; t++)
                            for (int u = 0; u <= ja + jb; u++)
                                for (int v = 0; v <= la + lb; v++)
                                    acc += hx.E[ia][ib][t] * hy.E[ja][jb][u] * hz.E[la][lb][v] * hr.R[t][u][v];
                        V[ka * nb + kb] += pre * acc;
                    }
            }
        }
}

// Dipole blocks <a| r_k - C_k |b> (k = x, y, z) of a shell pair, Cartesian:
// per direction M1(i, j) = sqrt(pi / p) (E_1^{ij} + (P_k - C_k) E_0^{ij}).
void dipole_pair(const CShell& a, const CShell& b, const double* C, double* M /* 3 x na x nb */) {
    const int na = a.ncart, nb = b.ncart;
    std::fill(M, M + 3 * na * nb, 0.0);
    Herm1 h[3];
    for (size_t pa = 0; pa < a.exps.size(); pa++)
        for (size_t pb = 0; pb < b.exps.size(); pb++) {
            const double ea = a.exps[pa], eb = b.exps[pb], p = ea + eb;
            const double cab = a.coefs[pa] * b.coefs[pb];
            for (int k = 0; k < 3; k++) hermite_e(a.l, b.l, ea, eb, a.A[k], b.A[k], h[k]);
            const double sp = std::sqrt(M_PI / p);
            double PC[3];
            for (int k = 0; k < 3; k++) PC[k] = (ea * a.A[k] + eb * b.A[k]) / p - C[k];
            for (int ka = 0; ka < na; ka++)
                for (int kb = 0; kb < nb; kb++) {
                    const int ix[3] = {a.ca[ka], a.cb[ka], a.cc[ka]}, jx[3] = {b.ca[kb], b.cb[kb], b.cc[kb]};
                    double s0[3], m1[3];
                    for (int k = 0; k < 3; k++) {
                        const double e0 = h[k].E[ix[k]][jx[k]][0];
                        const double e1 = ix[k] + jx[k] >= 1 ? h[k].E[ix[k]][jx[k]][1] : 0.0;
                        s0[k] = e0 * sp;
                        m1[k] = (e1 + PC[k] * e0) * sp;
                    }
                    M[(0 * na + ka) * nb + kb] += cab * m1[0] * s0[1] * s0[2];
                    M[(1 * na + ka) * nb + kb] += cab * s0[0] * m1[1] * s0[2];
                    M[(2 * na + ka) * nb + kb] += cab * s0[0] * s0[1] * m1[2];
                }
        }
}

// Primitive-pair Hermite data for the ERI.
struct PairData {
    double p, P[3], K;  // K = c_a c_b (E00 factors folded in E)
    // Etuv for every Cartesian component pair: [ka*nb+kb][t][u][v] flattened
    std::vector<double> E;
    int la_lb;
};

void eri_quartet(const CShell& a, const CShell& b, const CShell& c, const CShell& d, double* out /* cart a,b,c,d */) {
    const int na = a.ncart, nb = b.ncart, nc = c.ncart, nd = d.ncart;
    const int Lab = a.l + b.l, Lcd = c.l + d.l, L = Lab + Lcd;
    const int Hab = (Lab + 1), Hcd = (Lcd + 1);
    std::fill(out, out + (size_t)na * nb * nc * nd, 0.0);
    Herm1 ax, ay, az, cx, cy, cz;
    HermR hr;
    std::vector<double> X((size_t)nc * nd * Hab * Hab * Hab);
    for (size_t pa = 0; pa < a.exps.size(); pa++)
        for (size_t pb = 0; pb < b.exps.size(); pb++) {
            const double ea = a.exps[pa], eb = b.exps[pb], p = ea + eb;
            hermite_e(a.l, b.l, ea, eb, a.A[0], b.A[0], ax);
            hermite_e(a.l, b.l, ea, eb, a.A[1], b.A[1], ay);
            hermite_e(a.l, b.l, ea, eb, a.A[2], b.A[2], az);
            const double P[3] = {(ea * a.A[0] + eb * b.A[0]) / p, (ea * a.A[1] + eb * b.A[1]) / p,
                                 (ea * a.A[2] + eb * b.A[2]) / p};
            const double cab = a.coefs[pa] * b.coefs[pb];
            for (size_t pc = 0; pc < c.exps.size(); pc++)
                for (size_t pd = 0; pd < d.exps.size(); pd++) {
                    const double ec = c.exps[pc], ed = d.exps[pd], q = ec + ed;
                    hermite_e(c.l, d.l, ec, ed, c.A[0], d.A[0], cx);
                    hermite_e(c.l, d.l, ec, ed, c.A[1], d.A[1], cy);
                    hermite_e(c.l, d.l, ec, ed, c.A[2], d.A[2], cz);
                    const double Q[3] = {(ec * c.A[0] + ed * d.A[0]) / q, (ec * c.A[1] + ed * d.A[1]) / q,
                                         (ec * c.A[2] + ed * d.A[2]) / q};
                    const double alpha = p * q / (p + q);
                    hermite_r(L, alpha, P[0] - Q[0], P[1] - Q[1], P[2] - Q[2], hr);
                    const double pre = 2 * std::pow(M_PI, 2.5) / (p * q * std::sqrt(p + q)) * cab * c.coefs[pc] * d.coefs[pd];
                    // X[cd][t][u][v] = sum_{tau nu phi} (-1)^{tau+nu+phi} E^cd R_{t+tau, u+nu, v+phi}
                    for (int kc = 0; kc < nc; kc++)
                        for (int kd = 0; kd < nd; kd++) {
                            const int ic = c.ca[kc], jc = c.cb[kc], lc = c.cc[kc];
                            const int id = d.ca[kd], jd = d.cb[kd], ld = d.cc[kd];
                            double* x = &X[((size_t)kc * nd + kd) * Hab * Hab * Hab];
                            for (int t = 0; t <= Lab; t++)
                                for (int u = 0; u + t <= Lab; u++)
                                    for (int v = 0; v + u + t <= Lab; v++) {
                                        double acc = 0;
                                        for (int ta = 0; ta <= ic + id; ta++) {
                                            const double e1 = cx.E[ic][id][ta];
                                            if (e1 == 0) continue;
                                            for (int nu = 0; nu <= jc + jd; nu++) {
                                                const double e2 = e1 * cy.E[jc][jd][nu];
                                                if (e2 == 0) continue;
                                                for (int ph = 0; ph <= lc + ld; ph++) {
                                                    const double e3 = e2 * cz.E[lc][ld][ph];
                                                    const double sg = ((ta + nu + ph) & 1) ? -1.0 : 1.0;
                                                    acc += sg * e3 * hr.R[t + ta][u + nu][v + ph];
                                                }
                                            }
                                        }
                                        x[(t * Hab + u) * Hab + v] = acc;
                                    }
                        }
                    for (int ka = 0; ka < na; ka++)
                        for (int kb = 0; kb < nb; kb++) {
                            const int ia = a.ca[ka], ja = a.cb[ka], la = a.cc[ka];
                            const int ib = b.ca[kb], jb = b.cb[kb], lb = b.cc[kb];
                            for (int kc = 0; kc < nc; kc++)
                                for (int kd = 0; kd < nd; kd++) {
                                    const double* x = &X[((size_t)kc * nd + kd) * Hab * Hab * Hab];
                                    double acc = 0;
                                    for (int t = 0; t <= ia + ib; t++) {
                                        const double e1 = ax.E[ia][ib][t];
                                        if (e1 == 0) continue;
                                        for (int u = 0; u <= ja + jb; u++) {
                                            const double e2 = e1 * ay.E[ja][jb][u];
                                            if (e2 == 0) continue;
                                            for (int v = 0; v <= la + lb; v++)
                                                acc += e2 * az.E[la][lb][v] * x[(t * Hab + u) * Hab + v];
                                        }
                                    }
                                    out[(((size_t)ka * nb + kb) * nc + kc) * nd + kd] += pre * acc;
                                }
                        }
                }
        }
    (void)Hcd;
}

// pure transform of a Cartesian quartet block into the full n^4 tensor
void scatter_quartet(const CShell& a, const CShell& b, const CShell& c, const CShell& d, const double* cart, int n,
                     double* eri) {
    const int na = a.ncart, nb = b.ncart, nc = c.ncart, nd = d.ncart;
    std::vector<double> t1((size_t)a.nfunc * nb * nc * nd, 0.0);
    for (int f = 0; f < a.nfunc; f++)
        for (int k = 0; k < na; k++) {
            const double tv = a.T[(size_t)f * na + k];
            if (tv == 0) continue;
            for (size_t r = 0; r < (size_t)nb * nc * nd; r++) t1[(size_t)f * nb * nc * nd + r] += tv * cart[(size_t)k * nb * nc * nd + r];
        }
    std::vector<double> t2((size_t)a.nfunc * b.nfunc * nc * nd, 0.0);
    for (int fa = 0; fa < a.nfunc; fa++)
        for (int f = 0; f < b.nfunc; f++)
            for (int k = 0; k < nb; k++) {
                const double tv = b.T[(size_t)f * nb + k];
                if (tv == 0) continue;
                for (size_t r = 0; r < (size_t)nc * nd; r++)
                    t2[((size_t)fa * b.nfunc + f) * nc * nd + r] += tv * t1[((size_t)fa * nb + k) * nc * nd + r];
            }
    std::vector<double> t3((size_t)a.nfunc * b.nfunc * c.nfunc * nd, 0.0);
    for (int fab = 0; fab < a.nfunc * b.nfunc; fab++)
        for (int f = 0; f < c.nfunc; f++)
            for (int k = 0; k < nc; k++) {
                const double tv = c.T[(size_t)f * nc + k];
                if (tv == 0) continue;
                for (int r = 0; r < nd; r++) t3[((size_t)fab * c.nfunc + f) * nd + r] += tv * t2[((size_t)fab * nc + k) * nd + r];
            }
    for (int fa = 0; fa < a.nfunc; fa++)
        for (int fb = 0; fb < b.nfunc; fb++)
            for (int fc = 0; fc < c.nfunc; fc++)
                for (int fd = 0; fd < d.nfunc; fd++) {
                    double acc = 0;
                    for (int k = 0; k < nd; k++)
                        acc += d.T[(size_t)fd * nd + k] * t3[(((size_t)fa * b.nfunc + fb) * c.nfunc + fc) * nd + k];
                    const size_t i = a.first + fa, j = b.first + fb, k = c.first + fc, l = d.first + fd;
                    // 8-fold permutational symmetry
                    const size_t nn = n;
                    eri[((i * nn + j) * nn + k) * nn + l] = acc;
                    eri[((j * nn + i) * nn + k) * nn + l] = acc;
                    eri[((i * nn + j) * nn + l) * nn + k] = acc;
                    eri[((j * nn + i) * nn + l) * nn + k] = acc;
                    eri[((k * nn + l) * nn + i) * nn + j] = acc;
                    eri[((l * nn + k) * nn + i) * nn + j] = acc;
                    eri[((k * nn + l) * nn + j) * nn + i] = acc;
                    eri[((l * nn + k) * nn + j) * nn + i] = acc;
                }
}

}  // namespace

// Hermite data of the pure function products of shell pairs for the GPU
// integral engine (eri.h): per primitive pair kept (overlap charge
// |c_i c_j| exp(-mu R^2) (pi / p)^(3/2) >= prim_cut) its exponent sum, product
// centre and Ep[fa * nb + fb][h(t, u, v)] with the coefficients folded in.
// OpenMP over the pairs.
void eri_pairs_hermite(const BasisSet& b, const std::vector<std::pair<int, int>>& pairs, double prim_cut,
                       std::vector<PairHermite>& out) {
    const std::vector<CShell> sh = make_shells(b);
    out.assign(pairs.size(), PairHermite{});
#pragma omp parallel for schedule(dynamic)
    for (long ip = 0; ip < (long)pairs.size(); ip++) {
        const CShell &a = sh[pairs[ip].first], &c = sh[pairs[ip].second];
        PairHermite& o = out[ip];
        const int L = a.l + c.l, H = (L + 1) * (L + 2) * (L + 3) / 6;
        const int nab = a.nfunc * c.nfunc;
        Herm1 hx, hy, hz;
        std::vector<double> cartE((size_t)a.ncart * c.ncart * H);
        double R2 = 0;
        for (int k = 0; k < 3; k++) R2 += (a.A[k] - c.A[k]) * (a.A[k] - c.A[k]);
        for (size_t i = 0; i < a.exps.size(); i++)
            for (size_t j = 0; j < c.exps.size(); j++) {
                const double ea = a.exps[i], eb = c.exps[j], p = ea + eb;
                const double cc = a.coefs[i] * c.coefs[j];
                if (std::fabs(cc) * std::exp(-ea * eb / p * R2) * std::pow(M_PI / p, 1.5) < prim_cut) continue;
                hermite_e(a.l, c.l, ea, eb, a.A[0], c.A[0], hx);
                hermite_e(a.l, c.l, ea, eb, a.A[1], c.A[1], hy);
                hermite_e(a.l, c.l, ea, eb, a.A[2], c.A[2], hz);
                std::fill(cartE.begin(), cartE.end(), 0.0);
                for (int ka = 0; ka < a.ncart; ka++)
                    for (int kb = 0; kb < c.ncart; kb++) {
                        const int ix = a.ca[ka], iy = a.cb[ka], iz = a.cc[ka];
                        const int jx = c.ca[kb], jy = c.cb[kb], jz = c.cc[kb];
                        double* dst = &cartE[((size_t)ka * c.ncart + kb) * H];
                        for (int t = 0; t <= ix + jx; t++)
                            for (int u = 0; u <= iy + jy; u++)
                                for (int v = 0; v <= iz + jz; v++) {
                                    const int N = t + u + v, m = N - t;
                                    dst[N * (N + 1) * (N + 2) / 6 + m * (m + 1) / 2 + (m - u)] =
                                        cc * hx.E[ix][jx][t] * hy.E[iy][jy][u] * hz.E[iz][jz][v];
                                }
                    }
                o.p.push_back(p);
                for (int k = 0; k < 3; k++) o.P.push_back((ea * a.A[k] + eb * c.A[k]) / p);
                const size_t off = o.ep.size();
                o.ep.resize(off + (size_t)nab * H, 0.0);
                for (int fa = 0; fa < a.nfunc; fa++)
                    for (int fb = 0; fb < c.nfunc; fb++) {
                        double* dst = &o.ep[off + ((size_t)fa * c.nfunc + fb) * H];
                        for (int ka = 0; ka < a.ncart; ka++) {
                            const double ta = a.T[(size_t)fa * a.ncart + ka];
                            if (ta == 0) continue;
                            for (int kb = 0; kb < c.ncart; kb++) {
                                const double tb = c.T[(size_t)fb * c.ncart + kb];
                                if (tb == 0) continue;
                                const double* src = &cartE[((size_t)ka * c.ncart + kb) * H];
                                for (int h = 0; h < H; h++) dst[h] += ta * tb * src[h];
                            }
                        }
                    }
            }
    }
}

// Boys function table F_n(i * step), n < cols, i < rows (series and downward
// recursion of boys(), ~1e-16 relative).
void boys_table(int rows, int cols, double step, double* out) {
#pragma omp parallel for
    for (int i = 0; i < rows; i++) boys(cols - 1, i * step, out + (size_t)i * cols);
}

}  // namespace cgb

using namespace cgb;

extern "C" int xc_int1e(const xc_basis* bh, double* S, double* T, double* V) {
    return guard([&] {
        CGB_CHECK(bh && S && T && V, XC_ERR_ARG, "null argument");
        const BasisSet& b = bh->b;
        for (const Shell& s : b.shells) CGB_CHECK(s.l <= kMaxLInt, XC_ERR_UNSUPPORTED, "integrals support l <= 4");
        auto sh = make_shells(b);
        const int n = b.nbasis, ns = (int)sh.size();
#pragma omp parallel for schedule(dynamic)
        for (int ij = 0; ij < ns * ns; ij++) {
            const int i = ij / ns, j = ij % ns;
            if (j > i) continue;
            const CShell &a = sh[i], &c = sh[j];
            std::vector<double> cs(a.ncart * c.ncart), ct(cs.size()), cv(cs.size());
            std::vector<double> ps(a.nfunc * c.nfunc), pt(ps.size()), pv(ps.size());
            one_e_pair(a, c, b, cs.data(), ct.data(), cv.data());
            to_pure2(a, c, cs.data(), ps.data());
            to_pure2(a, c, ct.data(), pt.data());
            to_pure2(a, c, cv.data(), pv.data());
            for (int fa = 0; fa < a.nfunc; fa++)
                for (int fc = 0; fc < c.nfunc; fc++) {
                    const size_t mu = a.first + fa, nu = c.first + fc;
                    const int k = fa * c.nfunc + fc;
                    S[mu * n + nu] = S[nu * n + mu] = ps[k];
                    T[mu * n + nu] = T[nu * n + mu] = pt[k];
                    V[mu * n + nu] = V[nu * n + mu] = pv[k];
                }
        }
    });
}

extern "C" int xc_dipole(const xc_basis* bh, const double* origin, double* M) {
    return guard([&] {
        CGB_CHECK(bh && origin && M, XC_ERR_ARG, "null argument");
        const BasisSet& b = bh->b;
        for (const Shell& s : b.shells) CGB_CHECK(s.l <= kMaxLInt, XC_ERR_UNSUPPORTED, "integrals support l <= 4");
        auto sh = make_shells(b);
        const int n = b.nbasis, ns = (int)sh.size();
        const size_t nn = (size_t)n * n;
#pragma omp parallel for schedule(dynamic)
        for (int ij = 0; ij < ns * ns; ij++) {
            const int i = ij / ns, j = ij % ns;
            if (j > i) continue;
            const CShell &a = sh[i], &c = sh[j];
            const size_t blk = (size_t)a.ncart * c.ncart;
            std::vector<double> cm(3 * blk), pm((size_t)a.nfunc * c.nfunc);
            dipole_pair(a, c, origin, cm.data());
            for (int k = 0; k < 3; k++) {
                to_pure2(a, c, cm.data() + k * blk, pm.data());
                for (int fa = 0; fa < a.nfunc; fa++)
                    for (int fc = 0; fc < c.nfunc; fc++) {
                        const size_t mu = a.first + fa, nu = c.first + fc;
                        const double v = pm[fa * c.nfunc + fc];
                        M[k * nn + mu * n + nu] = M[k * nn + nu * n + mu] = v;
                    }
            }
        }
    });
}

extern "C" int xc_eri(const xc_basis* bh, double* eri, double schwarz_threshold) {
    return guard([&] {
        CGB_CHECK(bh && eri, XC_ERR_ARG, "null argument");
        const BasisSet& b = bh->b;
        for (const Shell& s : b.shells) CGB_CHECK(s.l <= kMaxLInt, XC_ERR_UNSUPPORTED, "integrals support l <= 4");
        auto sh = make_shells(b);
        const int n = b.nbasis, ns = (int)sh.size();
        std::memset(eri, 0, sizeof(double) * (size_t)n * n * n * n);
        // Schwarz bounds Q_ij = sqrt(max |(ij|ij)|)
        std::vector<double> Q((size_t)ns * ns, 0.0);
#pragma omp parallel for schedule(dynamic)
        for (int ij = 0; ij < ns * ns; ij++) {
            const int i = ij / ns, j = ij % ns;
            const CShell &a = sh[i], &c = sh[j];
            std::vector<double> buf((size_t)a.ncart * c.ncart * a.ncart * c.ncart);
            eri_quartet(a, c, a, c, buf.data());
            double m = 0;
            for (int x = 0; x < a.ncart * c.ncart; x++)
                m = std::max(m, std::fabs(buf[(size_t)x * a.ncart * c.ncart + x]));
            Q[ij] = std::sqrt(m) * 4.0;  // pure transform can mix Cartesian magnitudes
        }
        std::vector<std::pair<int, int>> pairs;
        for (int i = 0; i < ns; i++)
            for (int j = 0; j <= i; j++) pairs.emplace_back(i, j);
        const long np = (long)pairs.size();
#pragma omp parallel for schedule(dynamic)
        for (long pq = 0; pq < np * np; pq++) {
            const long p1 = pq / np, p2 = pq % np;
            if (p2 > p1) continue;
            const auto [i, j] = pairs[p1];
            const auto [k, l] = pairs[p2];
            if (Q[(size_t)i * ns + j] * Q[(size_t)k * ns + l] < schwarz_threshold) continue;
            const CShell &a = sh[i], &bb = sh[j], &c = sh[k], &d = sh[l];
            std::vector<double> cart((size_t)a.ncart * bb.ncart * c.ncart * d.ncart);
            eri_quartet(a, bb, c, d, cart.data());
            scatter_quartet(a, bb, c, d, cart.data(), n, eri);
        }
    });
}
