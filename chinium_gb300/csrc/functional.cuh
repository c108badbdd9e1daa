// Exchange-correlation functionals on the device.
//
// Each functional is an energy density per volume e(rho_a, rho_b, sigma_aa,
// sigma_ab, sigma_bb, tau_a, tau_b) written once as a template over a scalar
// type.  Potentials come from forward-mode automatic differentiation with
// Dual<R, N> (N seeded inputs), so vrho/vsigma/vtau are exact derivatives of
// the same expression that gives eps.  R = double is the plain path; the
// mixed path evaluates in float above the low-density threshold.
//
// The formulas are the published ones behind the libxc ids that the
// reference's DensityFunctionals/*.df files list (ExchangeCorrelation.cpp:
// 86-163): Slater; VWN5 and VWN-RPA (Vosko, Wilk, Nusair 1980); PW92 with
// libxc's modified parameters (Perdew, Wang 1992); PBE x/c (Perdew, Burke,
// Ernzerhof 1996) incl. the parameter set of ids 321/322; Becke 88; LYP
// (Miehlich et al. 1989 form); TPSS x/c (Tao et al. 2003); r2SCAN x/c
// (Furness et al. 2020); hybrids B3LYP (402), PBE0 (406), BHandHLYP (436),
// TPSSh (457).
#pragma once

#include <cuda_runtime.h>
#include <math.h>

namespace cgb {
namespace xcf {

#ifndef CGB_HD
#define CGB_HD __host__ __device__ __forceinline__
#endif
// Large functional bodies are compiled once per scalar type and called, not
// inlined into every kernel (keeps register pressure and build time bounded).
#ifndef CGB_HDN
#define CGB_HDN __host__ __device__ __noinline__
#endif

// ------------------------------------------------------------ float-float
// ff: a value held as hi + lo, two floats with |lo| <= ulp(hi) / 2 (48-bit
// significand), so FP64-level arithmetic runs on the FP32 pipe (64x GB300's
// FP64 rate).  The error-free transformations are Knuth's TwoSum, Dekker's
// Fast2Sum and the FMA product, combined as in the QD library (Hida, Li and
// Bailey 2001): accurate addition, multiplication, long division.  Used for
// the mixed path's FP64-level energy density.
struct ff {
    float hi, lo;
    CGB_HD ff() : hi(0.f), lo(0.f) {}
    CGB_HD ff(float h, float l) : hi(h), lo(l) {}
    CGB_HD ff(double x) : hi((float)x), lo((float)(x - (double)(float)x)) {}
    CGB_HD ff(int x) : ff((double)x) {}
};
CGB_HD void ff_two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}
CGB_HD void ff_fast_two_sum(float a, float b, float& s, float& e) {  // |a| >= |b|
    s = a + b;
    e = b - (s - a);
}
CGB_HD ff operator+(ff a, ff b) {
    float s, e, t, f;
    ff_two_sum(a.hi, b.hi, s, e);
    ff_two_sum(a.lo, b.lo, t, f);
    e += t;
    ff_fast_two_sum(s, e, s, e);
    e += f;
    ff_fast_two_sum(s, e, s, e);
    return ff(s, e);
}
CGB_HD ff operator-(ff a) { return ff(-a.hi, -a.lo); }
CGB_HD ff operator-(ff a, ff b) { return a + (-b); }
CGB_HD ff operator*(ff a, ff b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);  // the product's rounding error, exactly
    e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
    float s;
    ff_fast_two_sum(p, e, s, e);
    return ff(s, e);
}
CGB_HD ff operator/(ff a, ff b) {
    const float q1 = a.hi / b.hi;
    ff r = a - b * ff(q1, 0.f);
    const float q2 = r.hi / b.hi;
    r = r - b * ff(q2, 0.f);
    const float q3 = r.hi / b.hi;
    float s, e;
    ff_fast_two_sum(q1, q2, s, e);
    return ff(s, e) + ff(q3, 0.f);
}
CGB_HD ff& operator+=(ff& a, ff b) { return a = a + b; }
CGB_HD ff& operator-=(ff& a, ff b) { return a = a - b; }
CGB_HD ff& operator*=(ff& a, ff b) { return a = a * b; }
CGB_HD ff& operator/=(ff& a, ff b) { return a = a / b; }
CGB_HD bool operator<(ff a, ff b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
CGB_HD bool operator>(ff a, ff b) { return b < a; }
CGB_HD bool operator<=(ff a, ff b) { return !(b < a); }
CGB_HD bool operator>=(ff a, ff b) { return !(a < b); }
CGB_HD double ff_value(ff a) { return (double)a.hi + (double)a.lo; }
// x 2^k, exact (both parts scaled).
CGB_HD ff ff_ldexp(ff a, int k) { return ff(ldexpf(a.hi, k), ldexpf(a.lo, k)); }

template <class R, int N>
struct Dual {
    R v;
    R d[N > 0 ? N : 1];  // N = 0: value only (the slot is never read)
    CGB_HD Dual() {}
    CGB_HD Dual(R x) : v(x) {
#pragma unroll
        for (int i = 0; i < N; i++) d[i] = R(0);
    }
};

template <class R>
struct Scal {
    static CGB_HD R exp_(R x) { return ::exp(x); }
    static CGB_HD R log_(R x) { return ::log(x); }
    static CGB_HD R sqrt_(R x) { return ::sqrt(x); }
    static CGB_HD R pow_(R x, R p) { return ::pow(x, p); }
    static CGB_HD R cbrt_(R x) { return ::cbrt(x); }
    static CGB_HD R atan_(R x) { return ::atan(x); }
    static CGB_HD R asinh_(R x) { return ::asinh(x); }
};
template <>
struct Scal<float> {
    static CGB_HD float exp_(float x) { return ::expf(x); }
    static CGB_HD float log_(float x) { return ::logf(x); }
    static CGB_HD float sqrt_(float x) { return ::sqrtf(x); }
    static CGB_HD float pow_(float x, float p) { return ::powf(x, p); }
    static CGB_HD float cbrt_(float x) { return ::cbrtf(x); }
    static CGB_HD float atan_(float x) { return ::atanf(x); }
    static CGB_HD float asinh_(float x) { return ::asinhf(x); }
};

// Elementary functions in float-float, each from the FP32 function's value by
// one Newton step (quadratic: 2^-23 -> ~2^-46; log after reducing its
// argument to [1/sqrt 2, sqrt 2)) or, for exp, by argument reduction:
// exp(a) = 2^k (1 + s)^(2^9) with r = a - k ln2, s = expm1(r / 512) from its
// Taylor series, then s <- s (s + 2) nine times (the QD library's method;
// squaring 1 + s in that form keeps the small part's relative accuracy).
// atan and asinh (VWN's and Becke 88's) go through FP64.  Accuracy ~1e-14
// relative while results stay well inside FP32's range (lo is a normal float
// down to |hi| ~ 1e-31: exp arguments above about -70).
template <>
struct Scal<ff> {
    static CGB_HD ff exp_(ff a) {
        if (a.hi > 88.f) return ff(INFINITY, 0.f);
        if (a.hi < -87.f) return ff(0.f, 0.f);
        // r = a - k ln2 with ln2 = c1 + c2 (Cody and Waite): c1 has 16 significant
        // bits, so k c1 (|k| <= 127) is exact in one float; c2 is the rest in ff
        const float k = rintf(a.hi * 1.44269504f);
        const float c1 = 0.693145751953125f;
        const ff c2(1.4286068203094172321214581765680755e-06);
        const ff r = ff_ldexp((a - ff(k * c1, 0.f)) - ff(k, 0.f) * c2, -9);
        // expm1(r) for |r| <= ln2 / 1024: r + r^2/2 + ... + r^6/720 (next term < 2^-80)
        ff s = r * (ff(1.0) + r * (ff(0.5) + r * (ff(1.0 / 6.0) + r * (ff(1.0 / 24.0) +
                     r * (ff(1.0 / 120.0) + r * ff(1.0 / 720.0))))));
        for (int i = 0; i < 9; i++) s = s * (s + ff(2.0));
        return ff_ldexp(ff(1.0) + s, (int)k);
    }
    static CGB_HD ff log_(ff a) {
        // a = m 2^e with m in [1/sqrt 2, sqrt 2): log a = e ln2 + log m, and log m
        // by one Newton step on exp from logf(m) (error ~ (2^-24 |log m|)^2 / 2)
        int e;
        const float f = frexpf(a.hi, &e);  // a.hi = f 2^e, f in [1/2, 1)
        if (f < 0.70710678f) e -= 1;
        const ff m = ff_ldexp(a, -e);
        const float x0 = logf(m.hi);
        const ff lm = ff(x0, 0.f) + m * exp_(ff(-x0, 0.f)) - ff(1.0);
        const float c1 = 0.693145751953125f;  // ln2 = c1 + c2 as in exp_ (e c1 exact)
        const ff c2(1.4286068203094172321214581765680755e-06);
        return (ff((float)e * c1, 0.f) + ff((float)e, 0.f) * c2) + lm;
    }
    static CGB_HD ff sqrt_(ff a) {
        if (!(a.hi > 0.f)) return ff(0.f, 0.f);
        const float x = sqrtf(a.hi);
        const ff X(x, 0.f);
        const ff r = a - X * X;
        return X + ff(r.hi * (0.5f / x), 0.f);
    }
    static CGB_HD ff cbrt_(ff a) {
        if (a.hi == 0.f) return ff(0.f, 0.f);
        const float x = cbrtf(a.hi);
        const ff X(x, 0.f);
        const ff r = a - X * X * X;
        return X + ff(r.hi / (3.f * x * x), 0.f);
    }
    static CGB_HD ff atan_(ff a) { return ff(::atan(ff_value(a))); }
    static CGB_HD ff asinh_(ff a) { return ff(::asinh(ff_value(a))); }
    static CGB_HD ff pow_(ff a, ff p) { return ff(::pow(ff_value(a), ff_value(p))); }
};

// value / derivative-propagation primitives
template <class R, int N>
CGB_HD Dual<R, N> chain(const Dual<R, N>& a, R f, R df) {
    Dual<R, N> r;
    r.v = f;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = df * a.d[i];
    return r;
}

template <class R, int N>
CGB_HD Dual<R, N> operator+(const Dual<R, N>& a, const Dual<R, N>& b) {
    Dual<R, N> r;
    r.v = a.v + b.v;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = a.d[i] + b.d[i];
    return r;
}
template <class R, int N>
CGB_HD Dual<R, N> operator-(const Dual<R, N>& a, const Dual<R, N>& b) {
    Dual<R, N> r;
    r.v = a.v - b.v;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = a.d[i] - b.d[i];
    return r;
}
template <class R, int N>
CGB_HD Dual<R, N> operator-(const Dual<R, N>& a) {
    Dual<R, N> r;
    r.v = -a.v;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = -a.d[i];
    return r;
}
template <class R, int N>
CGB_HD Dual<R, N> operator*(const Dual<R, N>& a, const Dual<R, N>& b) {
    Dual<R, N> r;
    r.v = a.v * b.v;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
    return r;
}
template <class R, int N>
CGB_HD Dual<R, N> operator/(const Dual<R, N>& a, const Dual<R, N>& b) {
    Dual<R, N> r;
    const R ib = R(1) / b.v;
    r.v = a.v * ib;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
    return r;
}
// mixed scalar forms
template <class R, int N>
CGB_HD Dual<R, N> operator+(const Dual<R, N>& a, R b) {
    Dual<R, N> r = a;
    r.v += b;
    return r;
}
template <class R, int N>
CGB_HD Dual<R, N> operator+(R b, const Dual<R, N>& a) { return a + b; }
template <class R, int N>
CGB_HD Dual<R, N> operator-(const Dual<R, N>& a, R b) {
    Dual<R, N> r = a;
    r.v -= b;
    return r;
}
template <class R, int N>
CGB_HD Dual<R, N> operator-(R b, const Dual<R, N>& a) {
    Dual<R, N> r = -a;
    r.v += b;
    return r;
}
template <class R, int N>
CGB_HD Dual<R, N> operator*(const Dual<R, N>& a, R b) {
    Dual<R, N> r;
    r.v = a.v * b;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = a.d[i] * b;
    return r;
}
template <class R, int N>
CGB_HD Dual<R, N> operator*(R b, const Dual<R, N>& a) { return a * b; }
template <class R, int N>
CGB_HD Dual<R, N> operator/(const Dual<R, N>& a, R b) { return a * (R(1) / b); }
template <class R, int N>
CGB_HD Dual<R, N> operator/(R a, const Dual<R, N>& b) {
    Dual<R, N> r;
    const R ib = R(1) / b.v;
    r.v = a * ib;
    const R f = -r.v * ib;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = f * b.d[i];
    return r;
}

template <class R, int N>
CGB_HD Dual<R, N> exp(const Dual<R, N>& a) {
    const R e = Scal<R>::exp_(a.v);
    return chain(a, e, e);
}
template <class R, int N>
CGB_HD Dual<R, N> log(const Dual<R, N>& a) { return chain(a, Scal<R>::log_(a.v), R(1) / a.v); }
template <class R, int N>
CGB_HD Dual<R, N> sqrt(const Dual<R, N>& a) {
    const R s = Scal<R>::sqrt_(a.v);
    return chain(a, s, R(0.5) / s);
}
template <class R, int N>
CGB_HD Dual<R, N> pow(const Dual<R, N>& a, R p) {
    const R f = Scal<R>::pow_(a.v, p);
    return chain(a, f, p * f / a.v);
}
// x^(k/3) for an integer k: cbrt and binary powering (FP64 pow is several
// times the cost of cbrt; the functionals' exponents are all thirds).
template <class R>
CGB_HD R pow_third(R x, int k) {
    const R c = Scal<R>::cbrt_(x);
    R b = k < 0 ? R(1) / c : c, r = R(1);
    for (int m = k < 0 ? -k : k; m; m >>= 1) {
        if (m & 1) r *= b;
        b *= b;
    }
    return r;
}
template <class R, int N>
CGB_HD Dual<R, N> pow3(const Dual<R, N>& a, int k) {
    const R f = pow_third(a.v, k);
    return chain(a, f, R(k) / R(3) * f / a.v);
}
template <class R>
CGB_HD R pow3(R a, int k) { return pow_third(a, k); }
template <class R, int N>
CGB_HD Dual<R, N> atan(const Dual<R, N>& a) { return chain(a, Scal<R>::atan_(a.v), R(1) / (R(1) + a.v * a.v)); }
template <class R, int N>
CGB_HD Dual<R, N> asinh(const Dual<R, N>& a) {
    return chain(a, Scal<R>::asinh_(a.v), R(1) / Scal<R>::sqrt_(R(1) + a.v * a.v));
}
template <class R, int N>
CGB_HD R val(const Dual<R, N>& a) { return a.v; }

template <class T>
CGB_HD T tmax(const T& a, const T& b) { return val(a) >= val(b) ? a : b; }
template <class T>
CGB_HD T tmin(const T& a, const T& b) { return val(a) <= val(b) ? a : b; }

constexpr double kDensThr = 1e-15;
constexpr double kTauThr = 1e-20;
constexpr double kZetaThr = 2.220446049250313e-16;
constexpr double kPi = 3.14159265358979323846;

template <class T>
struct XIn {
    T ra, rb, saa, sab, sbb, ta, tb;
};

template <class T, class R>
CGB_HD T clamp_opz(const T& v) { return val(v) < R(kZetaThr) ? T(R(kZetaThr)) : v; }

// ------------------------------------------------------------------- LDA
template <class T, class R>
CGB_HD T ex_unif_half(const T& rs) {
    const R Cx = R(0.75 * 0.98474502184269654);  // 0.75 (3/pi)^(1/3)
    return R(-0.5) * Cx * pow3(R(2) * rs, 4);
}

template <class T, class R>
CGB_HD T fzeta(const T& opz, const T& omz) {
    return (pow3(opz, 4) + pow3(omz, 4) - R(2)) * R(1.0 / 0.51984209978974632953);
}

template <class T, class R>
CGB_HD T vwn_f(const T& x, R A, R b, R c, R x0) {
    const R Q = Scal<R>::sqrt_(R(4) * c - b * b);
    const T X = x * x + b * x + c;
    const R X0 = x0 * x0 + b * x0 + c;
    const T at = atan(Q / (R(2) * x + b));
    return A * (log(x * x / X) + R(2) * b / Q * at -
                b * x0 / X0 * (log((x - x0) * (x - x0) / X) + R(2) * (b + R(2) * x0) / Q * at));
}

template <class T, class R>
CGB_HD void rs_zeta(const XIn<T>& v, T& rho, T& rs, T& z, T& opz, T& omz) {
    rho = v.ra + v.rb;
    rs = pow3(R(3.0 / (4.0 * kPi)) / rho, 1);
    z = (v.ra - v.rb) / rho;
    opz = clamp_opz<T, R>(R(1) + z);
    omz = clamp_opz<T, R>(R(1) - z);
}

template <class T, class R>
CGB_HD T e_lda_x(const XIn<T>& v) { return ex_unif_half<T, R>(v.ra) + ex_unif_half<T, R>(v.rb); }

template <class T, class R>
CGB_HDN T e_vwn(const XIn<T>& v, bool rpa) {
    T rho, rs, z, opz, omz;
    rs_zeta<T, R>(v, rho, rs, z, opz, omz);
    const T x = sqrt(rs);
    const T f = fzeta<T, R>(opz, omz);
    if (rpa) {
        const T ep = vwn_f<T, R>(x, R(0.0310907), R(13.0720), R(42.7198), R(-0.409286));
        const T ef = vwn_f<T, R>(x, R(0.01554535), R(20.1231), R(101.578), R(-0.743294));
        return rho * (ep + (ef - ep) * f);
    }
    const T ep = vwn_f<T, R>(x, R(0.0310907), R(3.72744), R(12.9352), R(-0.10498));
    const T ef = vwn_f<T, R>(x, R(0.01554535), R(7.06042), R(18.0578), R(-0.32500));
    const T ac = vwn_f<T, R>(x, R(-1.0 / (6.0 * kPi * kPi)), R(1.13107), R(13.0045), R(-0.0047584));
    const R fpp0 = R(4.0 / (9.0 * 0.25992104989487316477));  // 4 / (9 (2^(1/3) - 1))
    const T z2 = z * z, z4 = z2 * z2;
    return rho * (ep + ac * f / fpp0 * (R(1) - z4) + (ef - ep) * f * z4);
}

// PW92 G(rs) and dG/drs
struct PwPar {
    double A, a1, b1, b2, b3, b4;
};
template <class T, class R>
CGB_HD T pw_G(const T& rs, const PwPar& p) {
    const T srs = sqrt(rs);
    const T q1 = R(2 * p.A) * (R(p.b1) * srs + R(p.b2) * rs + R(p.b3) * rs * srs + R(p.b4) * rs * rs);
    return R(-2 * p.A) * (R(1) + R(p.a1) * rs) * log(R(1) + R(1) / q1);
}
template <class T, class R>
CGB_HD T pw_dG(const T& rs, const PwPar& p) {
    const T srs = sqrt(rs);
    const T q1 = R(2 * p.A) * (R(p.b1) * srs + R(p.b2) * rs + R(p.b3) * rs * srs + R(p.b4) * rs * rs);
    const T dq1 = R(2 * p.A) * (R(p.b1) / (R(2) * srs) + R(p.b2) + R(1.5 * p.b3) * srs + R(2 * p.b4) * rs);
    return R(-2 * p.A * p.a1) * log(R(1) + R(1) / q1) + R(2 * p.A) * (R(1) + R(p.a1) * rs) * dq1 / (q1 * q1 + q1);
}

template <class T, class R>
CGB_HDN T pw_eps(const T& rs, const T& z, const T& opz, const T& omz, T* deps) {
    constexpr PwPar E0{0.0310907, 0.21370, 7.5957, 3.5876, 1.6382, 0.49294};
    constexpr PwPar E1{0.01554535, 0.20548, 14.1189, 6.1977, 3.3662, 0.62517};
    constexpr PwPar AC{0.0168869, 0.11125, 10.357, 3.6231, 0.88026, 0.49671};
    const R fpp = R(1.709920934161365617563962776245);
    const T f = fzeta<T, R>(opz, omz);
    const T z2 = z * z, z4 = z2 * z2;
    const T e0 = pw_G<T, R>(rs, E0), e1 = pw_G<T, R>(rs, E1), mac = pw_G<T, R>(rs, AC);
    if (deps) {
        const T d0 = pw_dG<T, R>(rs, E0), d1 = pw_dG<T, R>(rs, E1), dm = pw_dG<T, R>(rs, AC);
        *deps = d0 - dm * f * (R(1) - z4) / fpp + (d1 - d0) * f * z4;
    }
    return e0 - mac * f * (R(1) - z4) / fpp + (e1 - e0) * f * z4;
}

// ------------------------------------------------------------------- GGA
template <class T, class R>
CGB_HD T p_red(const T& n, const T& sig) {
    // sig / (4 (3 pi^2)^(2/3) n^(8/3))
    return sig / (R(4.0 * 9.570780000627305) * pow3(n, 8));
}

// sum over spins of 1/2 e_unif(2 rho_s) F(n = 2 rho_s, 4 sigma_ss, 2 tau_s)
template <class T, class R, class F>
CGB_HDN T spin_exchange(const XIn<T>& v, F fx) {
    T out(R(0));
    if (val(v.ra) > R(0.5 * kDensThr)) out = out + ex_unif_half<T, R>(v.ra) * fx(R(2) * v.ra, R(4) * v.saa, R(2) * v.ta);
    if (val(v.rb) > R(0.5 * kDensThr)) out = out + ex_unif_half<T, R>(v.rb) * fx(R(2) * v.rb, R(4) * v.sbb, R(2) * v.tb);
    return out;
}

template <class T, class R>
CGB_HD T fx_pbe(const T& n, const T& sig, R kappa, R mu) {
    const T p = p_red<T, R>(n, sig);
    return R(1) + kappa - kappa / (R(1) + mu * p / kappa);
}

template <class T, class R>
CGB_HDN T e_b88(const XIn<T>& v) {
    const R beta = R(0.0042);
    const R cx = R(1.5 * 0.62035049089940001667);  // 1.5 (3/(4 pi))^(1/3)
    T out(R(0));
    const T rr[2] = {v.ra, v.rb};
    const T ss[2] = {v.saa, v.sbb};
#pragma unroll
    for (int s = 0; s < 2; s++) {
        if (val(rr[s]) <= R(0.5 * kDensThr)) continue;
        const T r43 = pow3(rr[s], 4);
        const T x = sqrt(ss[s]) / r43;
        out = out - cx * r43 - beta * r43 * x * x / (R(1) + R(6) * beta * x * asinh(x));
    }
    return out;
}

template <class T, class R>
CGB_HDN T e_lyp(const XIn<T>& v) {
    const R a = R(0.04918), b = R(0.132), c = R(0.2533), d = R(0.349);
    const R CF = R(0.3 * 9.570780000627305);  // 3/10 (3 pi^2)^(2/3)
    const T ra = v.ra, rb = v.rb, rho = ra + rb;
    const T saa = v.saa, sbb = v.sbb, sig = v.saa + R(2) * v.sab + v.sbb;
    const T rm13 = pow3(rho, -1);
    const T den = R(1) + d * rm13;
    const T omega = exp(-c * rm13) / den * pow3(rho, -11);
    const T delta = c * rm13 + d * rm13 / den;
    const T t1 = R(-4) * a / den * ra * rb / rho;
    const T inner = ra * rb * (R(12.699208415745595) * CF * (pow3(ra, 8) + pow3(rb, 8)) +
                               (R(47.0 / 18.0) - R(7.0 / 18.0) * delta) * sig -
                               (R(2.5) - delta / R(18)) * (saa + sbb) -
                               (delta - R(11)) / R(9) * (ra / rho * saa + rb / rho * sbb)) -
                    R(2.0 / 3.0) * rho * rho * sig + (R(2.0 / 3.0) * rho * rho - ra * ra) * sbb +
                    (R(2.0 / 3.0) * rho * rho - rb * rb) * saa;
    return t1 - a * b * omega * inner;
}

template <class T, class R>
CGB_HDN T pbe_c_eps(const T& rho, const T& z, const T& opz, const T& omz, const T& sig, R beta) {
    const R gamma = R(0.031090690869654895034);  // (1 - ln 2) / pi^2
    const T rs = pow3(R(3.0 / (4.0 * kPi)) / rho, 1);
    const T ec = pw_eps<T, R>(rs, z, opz, omz, nullptr);
    const T phi = (pow3(opz, 2) + pow3(omz, 2)) * R(0.5);
    const T phi3 = phi * phi * phi;
    const T kf = pow3(R(3.0 * kPi * kPi) * rho, 1);
    const T t2 = sig * R(kPi) / (R(16) * phi * phi * kf * rho * rho);
    const T A = (beta / gamma) / (exp(-ec / (gamma * phi3)) - R(1));
    const T At2 = A * t2;
    const T H = gamma * phi3 * log(R(1) + beta / gamma * t2 * (R(1) + At2) / (R(1) + At2 + At2 * At2));
    return ec + H;
}

template <class T, class R>
CGB_HD T e_pbe_c(const XIn<T>& v, R beta) {
    T rho, rs, z, opz, omz;
    rs_zeta<T, R>(v, rho, rs, z, opz, omz);
    const T sig = v.saa + R(2) * v.sab + v.sbb;
    return rho * pbe_c_eps<T, R>(rho, z, opz, omz, sig, beta);
}

// ------------------------------------------------------------------ mGGA
template <class T, class R>
CGB_HDN T fx_tpss(const T& n, const T& sig, const T& tau) {
    const R b = R(0.40), c = R(1.59096), e = R(1.537), kappa = R(0.804), mu = R(0.21951);
    const T p = p_red<T, R>(n, sig);
    const T tauw = sig / (R(8) * n);
    const T z = tauw / tau;
    const T tunif = R(0.3 * 9.570780000627305) * pow3(n, 5);
    const T alpha = (tau - tauw) / tunif;
    const T qb = R(0.45) * (alpha - R(1)) / sqrt(R(1) + b * alpha * (alpha - R(1))) + R(2.0 / 3.0) * p;
    const T z2 = z * z;
    const R se = Scal<R>::sqrt_(e);
    const T zz = R(0.6) * z;
    const T num = (R(10.0 / 81.0) + c * z2 / ((R(1) + z2) * (R(1) + z2))) * p + R(146.0 / 2025.0) * qb * qb -
                  R(73.0 / 405.0) * qb * sqrt(R(0.5) * zz * zz + R(0.5) * p * p) +
                  (R(1) / kappa) * R(100.0 / 6561.0) * p * p + R(2) * se * R(10.0 / 81.0) * zz * zz +
                  e * mu * p * p * p;
    const T den = R(1) + se * p;
    const T x = num / (den * den);
    return R(1) + kappa - kappa / (R(1) + x / kappa);
}

template <class T, class R>
CGB_HDN T e_tpss_c(const XIn<T>& v) {
    const R beta = R(0.06672455060314922), d = R(2.8);
    T rho, rs, z, opz, omz;
    rs_zeta<T, R>(v, rho, rs, z, opz, omz);
    const T sig = v.saa + R(2) * v.sab + v.sbb;
    const T tau = v.ta + v.tb;
    const T epbe = pbe_c_eps<T, R>(rho, z, opz, omz, sig, beta);
    const T rho2 = rho * rho;
    const T gz2 = R(4) * (v.rb * v.rb * v.saa - R(2) * v.ra * v.rb * v.sab + v.ra * v.ra * v.sbb) / (rho2 * rho2);
    const T xi2 = gz2 / (R(4) * pow3(R(3.0 * kPi * kPi) * rho, 2));
    const T zz2 = z * z;
    const T C0 = R(0.53) + R(0.87) * zz2 + R(0.50) * zz2 * zz2 + R(2.26) * zz2 * zz2 * zz2;
    const T den = R(1) + xi2 * (pow3(opz, -4) + pow3(omz, -4)) * R(0.5);
    const T den2 = den * den;
    const T C = C0 / (den2 * den2);
    const T rr[2] = {v.ra, v.rb};
    const T ss[2] = {v.saa, v.sbb};
    T sum(R(0));
#pragma unroll
    for (int s = 0; s < 2; s++) {
        if (val(rr[s]) <= R(0.5 * kDensThr)) continue;
        const T es = pbe_c_eps<T, R>(rr[s], T(R(1)), T(R(2)), T(R(kZetaThr)), ss[s], beta);
        sum = sum + rr[s] / rho * tmax(es, epbe);
    }
    const T tauw = sig / (R(8) * rho);
    const T q = tauw / tau;
    const T q2 = q * q;
    const T erev = epbe * (R(1) + C * q2) - (R(1) + C) * q2 * sum;
    return rho * erev * (R(1) + d * erev * q2 * q);
}

// r2SCAN interpolation functions f_x / f_c: degree-7 polynomial for
// alpha-bar <= 2.5, -d exp(c2 / (1 - alpha-bar)) above.
template <class T, class R>
CGB_HD T r2_fx(const T& a) {
    if (val(a) <= R(2.5)) {
        T s(R(-0.023185843322));
        s = s * a + R(0.234528941479);
        s = s * a + R(-0.887998041597);
        s = s * a + R(1.451297044490);
        s = s * a + R(-0.663086601049);
        s = s * a + R(-0.4445555);
        s = s * a + R(-0.667);
        return s * a + R(1.0);
    }
    return R(-1.24) * exp(R(0.8) / (R(1) - a));
}
template <class T, class R>
CGB_HD T r2_fc(const T& a) {
    if (val(a) <= R(2.5)) {
        T s(R(-0.051848879792));
        s = s * a + R(0.516884468372);
        s = s * a + R(-1.915710236206);
        s = s * a + R(3.061560252175);
        s = s * a + R(-1.535685604549);
        s = s * a + R(-0.4352);
        s = s * a + R(-0.64);
        return s * a + R(1.0);
    }
    return R(-0.7) * exp(R(1.5) / (R(1) - a));
}

constexpr double kR2Eta = 0.001;
constexpr double kR2Dp2 = 0.361;
// sum_{i>=1} i c_i of the two polynomials
constexpr double kR2Dfx = -0.667 * 1 - 0.4445555 * 2 - 0.663086601049 * 3 + 1.451297044490 * 4 -
                          0.887998041597 * 5 + 0.234528941479 * 6 - 0.023185843322 * 7;
constexpr double kR2Dfc = -0.64 * 1 - 0.4352 * 2 - 1.535685604549 * 3 + 3.061560252175 * 4 -
                          1.915710236206 * 5 + 0.516884468372 * 6 - 0.051848879792 * 7;

template <class T, class R>
CGB_HDN T fx_r2scan(const T& n, const T& sig, const T& tau) {
    const R k1 = R(0.065), hx0 = R(1.174), a1 = R(4.9479);
    const R mu_ak = R(10.0 / 81.0);
    const R Ceta = R(20.0 / 27.0 + kR2Eta * 5.0 / 3.0);
    const R C2 = R(-kR2Dfx * (1.0 - 1.174));
    const T p = p_red<T, R>(n, sig);
    const T tauw = sig / (R(8) * n);
    const T tunif = R(0.3 * 9.570780000627305) * pow3(n, 5);
    const T ab = (tau - tauw) / (tunif + R(kR2Eta) * tauw);
    const R dp24 = R(kR2Dp2 * kR2Dp2 * kR2Dp2 * kR2Dp2);
    const T x = (Ceta * C2 * exp(-(p * p) / dp24) + mu_ak) * p;
    const T hx1 = R(1) + k1 - k1 / (R(1) + x / k1);
    const T fx = r2_fx<T, R>(ab);
    const T gx = R(1) - exp(-a1 / sqrt(sqrt(p)));
    return (hx1 + fx * (hx0 - hx1)) * gx;
}

template <class T, class R>
CGB_HDN T e_r2scan_c(const XIn<T>& v) {
    const R b1c = R(0.0285764), b2c = R(0.0889), b3c = R(0.125541), chi = R(0.128026);
        const R gamma = R(0.031090690869654895034);
    T rho, rs, z, opz, omz;
    rs_zeta<T, R>(v, rho, rs, z, opz, omz);
    const T sig = v.saa + R(2) * v.sab + v.sbb;
    const T tau = v.ta + v.tb;
    const T phi = (pow3(opz, 2) + pow3(omz, 2)) * R(0.5);
    const T phi3 = phi * phi * phi;
    const T ds = (pow3(opz, 5) + pow3(omz, 5)) * R(0.5);
    const T dxz = (pow3(opz, 4) + pow3(omz, 4)) * R(0.5);
    const T p = p_red<T, R>(rho, sig);
    const T kf = pow3(R(3.0 * kPi * kPi) * rho, 1);
    const T t2 = sig * R(kPi) / (R(16) * phi * phi * kf * rho * rho);
    T de1;
    const T e1 = pw_eps<T, R>(rs, z, opz, omz, &de1);
    const T w1 = exp(-e1 / (gamma * phi3)) - R(1);
    const T betars = R(0.066725) * (R(1) + R(0.1) * rs) / (R(1) + R(0.1778) * rs);
    const T y = betars / (gamma * w1) * t2;
    const T srs = sqrt(rs);
    const T dd = R(1) + b2c * srs + b3c * rs;
    const T elda0 = -b1c / dd;
    const T delda0 = b1c * (b2c / (R(2) * srs) + b3c) / (dd * dd);
    const T z2 = z * z, z4 = z2 * z2;
    const T Gc = (R(1) - R(2.3631) * (dxz - R(1))) * (R(1) - z4 * z4 * z4);
    const T w0 = exp(-elda0 / b1c) - R(1);
    const T ginf = R(1) / sqrt(sqrt(R(1) + R(4) * chi * p));
    const T H0 = b1c * log(R(1) + w0 * (R(1) - ginf));
    const T e0 = (elda0 + H0) * Gc;
    const R dp24 = R(kR2Dp2 * kR2Dp2 * kR2Dp2 * kR2Dp2);
    const T dy = R(kR2Dfc) / (R(27) * gamma * ds * phi3 * w1) *
                 (R(20) * rs * (delda0 * Gc - de1) - R(45 * kR2Eta) * (elda0 * Gc - e1)) * p * exp(-(p * p) / dp24);
    const T g = R(1) / sqrt(sqrt(R(1) + R(4) * (y - dy)));
    const T H1 = gamma * phi3 * log(R(1) + w1 * (R(1) - g));
    const T ec1 = e1 + H1;
    const T tauw = sig / (R(8) * rho);
    const T tunif = R(0.3 * 9.570780000627305) * pow3(rho, 5) * ds;
    const T ab = (tau - tauw) / (tunif + R(kR2Eta) * tauw);
    const T fc = r2_fc<T, R>(ab);
    return rho * (ec1 + fc * (e0 - ec1));
}

// ------------------------------------------------------------- registry
// Energy density of one LDA or GGA libxc id (the ids that also have second
// derivatives, order "f"); zero for any other id.
template <class T, class R>
CGB_HD T e_id_gga(int id, const XIn<T>& v) {
    auto pbe_x = [](const T& n, const T& s, const T&) { return fx_pbe<T, R>(n, s, R(0.8040), R(0.2195149727645171)); };
    auto pbe_xg = [](const T& n, const T& s, const T&) { return fx_pbe<T, R>(n, s, R(0.804), R(0.2195164512208958)); };
    switch (id) {
        case 1: return e_lda_x<T, R>(v);
        case 7: return e_vwn<T, R>(v, false);
        case 8: return e_vwn<T, R>(v, true);
        case 101: return spin_exchange<T, R>(v, pbe_x);
        case 130: return e_pbe_c<T, R>(v, R(0.06672455060314922));
        case 321: return spin_exchange<T, R>(v, pbe_xg);
        case 322: return e_pbe_c<T, R>(v, R(0.066725));
        case 106: return e_b88<T, R>(v);
        case 131: return e_lyp<T, R>(v);
        case 402:
            return R(0.08) * e_lda_x<T, R>(v) + R(0.72) * e_b88<T, R>(v) + R(0.19) * e_vwn<T, R>(v, true) +
                   R(0.81) * e_lyp<T, R>(v);
        case 406: return R(0.75) * spin_exchange<T, R>(v, pbe_x) + e_pbe_c<T, R>(v, R(0.06672455060314922));
        case 436: return R(0.5) * e_b88<T, R>(v) + e_lyp<T, R>(v);
    }
    return T(R(0));
}

// Energy density of one libxc id; unknown ids contribute nothing (ids are
// validated on the host before any launch).
template <class T, class R>
CGB_HDN T e_id(int id, const XIn<T>& v) {
    auto tpss_x = [](const T& n, const T& s, const T& t) { return fx_tpss<T, R>(n, s, t); };
    auto r2_x = [](const T& n, const T& s, const T& t) { return fx_r2scan<T, R>(n, s, t); };
    switch (id) {
        case 202: return spin_exchange<T, R>(v, tpss_x);
        case 231: return e_tpss_c<T, R>(v);
        case 457: return R(0.9) * spin_exchange<T, R>(v, tpss_x) + e_tpss_c<T, R>(v);
        case 497: return spin_exchange<T, R>(v, r2_x);
        case 498: return e_r2scan_c<T, R>(v);
    }
    return e_id_gga<T, R>(id, v);
}

// Family of an id (0 LDA, 1 GGA, 2 mGGA), -1 if unknown; EXX fraction.
inline int family_of_id(int id) {
    switch (id) {
        case 1: case 7: case 8: return 0;
        case 101: case 130: case 321: case 322: case 106: case 131: case 402: case 406: case 436: return 1;
        case 202: case 231: case 457: case 497: case 498: return 2;
    }
    return -1;
}
inline double exx_of_id(int id) {
    switch (id) {
        case 402: return 0.20;
        case 406: return 0.25;
        case 436: return 0.50;
        case 457: return 0.10;
    }
    return 0.0;
}

struct FuncDesc {
    int nids;
    int ids[4];
};

template <class T, class R>
CGB_HD T e_sum(const FuncDesc& f, const XIn<T>& v) {
    T e(R(0));
    for (int i = 0; i < f.nids; i++) e = e + e_id<T, R>(f.ids[i], v);
    return e;
}

// Restricted point: inputs rho, sigma, tau (totals).  Outputs eps and, with
// DERIV, d e / d (rho, sigma, tau).  Returns false when below the density
// threshold.  Without DERIV no direction is seeded (Dual<R, 0>: the value
// alone, a fraction of the arithmetic).
template <class R, int FAM, bool DERIV>
CGB_HDN bool eval_unpol_t(const FuncDesc& f, R rho, R sigma, R tau, R& eps, R* dv) {
    constexpr int N = !DERIV ? 0 : (FAM == 0 ? 1 : (FAM == 1 ? 2 : 3));
    using T = Dual<R, N>;
    if (!(rho >= R(kDensThr))) {
        eps = R(0);
        for (int i = 0; i < N; i++) dv[i] = R(0);
        return false;
    }
    T r(rho), s(sigma), t(tau);
    if constexpr (N > 0) r.d[0] = R(1);
    if constexpr (N > 1) s.d[1] = R(1);
    if constexpr (N > 2) t.d[2] = R(1);
    s = tmax(s, T(R(1.0000000000000011e-40)));  // kDensThr^(8/3)
    if (FAM >= 2) {
        t = tmax(t, T(R(kTauThr)));
        s = tmin(s, R(8) * r * t);
    }
    XIn<T> v{r * R(0.5), r * R(0.5), s * R(0.25), s * R(0.25), s * R(0.25), t * R(0.5), t * R(0.5)};
    const T e = e_sum<T, R>(f, v);
    eps = e.v / rho;
    for (int i = 0; i < N; i++) dv[i] = e.d[i];
    return true;
}
template <class R, int FAM>
CGB_HD bool eval_unpol(const FuncDesc& f, R rho, R sigma, R tau, R& eps, R* dv) {
    return eval_unpol_t<R, FAM, true>(f, rho, sigma, tau, eps, dv);
}
// eps alone.
template <class R, int FAM>
CGB_HD bool eval_unpol_value(const FuncDesc& f, R rho, R sigma, R tau, R& eps) {
    return eval_unpol_t<R, FAM, false>(f, rho, sigma, tau, eps, nullptr);
}

// Unrestricted point: in = (ra, rb, saa, sab, sbb, ta, tb); dv in the same
// order (with DERIV; without it eps alone, as eval_unpol_t).
template <class R, int FAM, bool DERIV>
CGB_HDN bool eval_pol_t(const FuncDesc& f, const R* in, R& eps, R* dv) {
    constexpr int N = !DERIV ? 0 : (FAM == 0 ? 2 : (FAM == 1 ? 5 : 7));
    using T = Dual<R, N>;
    const R rt = in[0] + in[1];
    if (!(rt >= R(kDensThr))) {
        eps = R(0);
        for (int i = 0; i < N; i++) dv[i] = R(0);
        return false;
    }
    T x[7];
    for (int i = 0; i < 7; i++) {
        x[i] = T(in[i]);
        if constexpr (N > 0)
            if (i < N) x[i].d[i] = R(1);
    }
    XIn<T> v{x[0], x[1], x[2], x[3], x[4], x[5], x[6]};
    v.ra = tmax(v.ra, T(R(kDensThr)));
    v.rb = tmax(v.rb, T(R(kDensThr)));
    v.saa = tmax(v.saa, T(R(1.0000000000000011e-40)));
    v.sbb = tmax(v.sbb, T(R(1.0000000000000011e-40)));
    if (FAM >= 2) {
        v.ta = tmax(v.ta, T(R(kTauThr)));
        v.tb = tmax(v.tb, T(R(kTauThr)));
        v.saa = tmin(v.saa, R(8) * v.ra * v.ta);
        v.sbb = tmin(v.sbb, R(8) * v.rb * v.tb);
    }
    const T half = (v.saa + v.sbb) * R(0.5);
    v.sab = tmax(tmin(v.sab, half), -half);
    const T e = e_sum<T, R>(f, v);
    eps = e.v / rt;
    for (int i = 0; i < N; i++) dv[i] = e.d[i];
    return true;
}
template <class R, int FAM>
CGB_HD bool eval_pol(const FuncDesc& f, const R* in, R& eps, R* dv) {
    return eval_pol_t<R, FAM, true>(f, in, eps, dv);
}
template <class R, int FAM>
CGB_HD bool eval_pol_value(const FuncDesc& f, const R* in, R& eps) {
    return eval_pol_t<R, FAM, false>(f, in, eps, nullptr);
}

// ------------------------------------------------ second derivatives ("f")
// Jet2<R, N>: value, gradient and the upper triangle of the Hessian in N
// seeded inputs, propagated by the chain and product rules (second-order
// forward mode), so the kernel f_xc of ExchangeCorrelation::Evaluate("f")
// (ExchangeCorrelation.cpp:101-104, 126-133) is the exact Hessian of the
// same expression that gives eps and v_xc.  Entry (i, j), i <= j, is
// h[i N - i (i - 1) / 2 + j - i].
template <class R, int N>
struct Jet2 {
    static constexpr int NH = N * (N + 1) / 2;
    R v;
    R d[N];
    R h[NH];
    CGB_HD Jet2() {}
    CGB_HD Jet2(R x) : v(x) {
#pragma unroll
        for (int i = 0; i < N; i++) d[i] = R(0);
#pragma unroll
        for (int k = 0; k < NH; k++) h[k] = R(0);
    }
};

// f(a) with f' = f1 and f'' = f2 at a.v
template <class R, int N>
CGB_HD Jet2<R, N> chain2(const Jet2<R, N>& a, R f, R f1, R f2) {
    Jet2<R, N> r;
    r.v = f;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = f1 * a.d[i];
    int k = 0;
#pragma unroll
    for (int i = 0; i < N; i++)
#pragma unroll
        for (int j = i; j < N; j++, k++) r.h[k] = f1 * a.h[k] + f2 * a.d[i] * a.d[j];
    return r;
}

template <class R, int N>
CGB_HD Jet2<R, N> operator+(const Jet2<R, N>& a, const Jet2<R, N>& b) {
    Jet2<R, N> r;
    r.v = a.v + b.v;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = a.d[i] + b.d[i];
#pragma unroll
    for (int k = 0; k < Jet2<R, N>::NH; k++) r.h[k] = a.h[k] + b.h[k];
    return r;
}
template <class R, int N>
CGB_HD Jet2<R, N> operator-(const Jet2<R, N>& a) {
    Jet2<R, N> r;
    r.v = -a.v;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = -a.d[i];
#pragma unroll
    for (int k = 0; k < Jet2<R, N>::NH; k++) r.h[k] = -a.h[k];
    return r;
}
template <class R, int N>
CGB_HD Jet2<R, N> operator-(const Jet2<R, N>& a, const Jet2<R, N>& b) { return a + (-b); }
template <class R, int N>
CGB_HD Jet2<R, N> operator*(const Jet2<R, N>& a, const Jet2<R, N>& b) {
    Jet2<R, N> r;
    r.v = a.v * b.v;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
    int k = 0;
#pragma unroll
    for (int i = 0; i < N; i++)
#pragma unroll
        for (int j = i; j < N; j++, k++)
            r.h[k] = a.h[k] * b.v + a.v * b.h[k] + a.d[i] * b.d[j] + a.d[j] * b.d[i];
    return r;
}
// q = a / b from a = q b: q' = (a' - q b') / b, q'' = (a'' - q b'' - q'_i b'_j - q'_j b'_i) / b
template <class R, int N>
CGB_HD Jet2<R, N> operator/(const Jet2<R, N>& a, const Jet2<R, N>& b) {
    Jet2<R, N> r;
    const R ib = R(1) / b.v;
    r.v = a.v * ib;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
    int k = 0;
#pragma unroll
    for (int i = 0; i < N; i++)
#pragma unroll
        for (int j = i; j < N; j++, k++)
            r.h[k] = (a.h[k] - r.v * b.h[k] - r.d[i] * b.d[j] - r.d[j] * b.d[i]) * ib;
    return r;
}
template <class R, int N>
CGB_HD Jet2<R, N> operator+(const Jet2<R, N>& a, R b) {
    Jet2<R, N> r = a;
    r.v += b;
    return r;
}
template <class R, int N>
CGB_HD Jet2<R, N> operator+(R b, const Jet2<R, N>& a) { return a + b; }
template <class R, int N>
CGB_HD Jet2<R, N> operator-(const Jet2<R, N>& a, R b) { return a + (-b); }
template <class R, int N>
CGB_HD Jet2<R, N> operator-(R b, const Jet2<R, N>& a) { return (-a) + b; }
template <class R, int N>
CGB_HD Jet2<R, N> operator*(const Jet2<R, N>& a, R b) {
    Jet2<R, N> r;
    r.v = a.v * b;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = a.d[i] * b;
#pragma unroll
    for (int k = 0; k < Jet2<R, N>::NH; k++) r.h[k] = a.h[k] * b;
    return r;
}
template <class R, int N>
CGB_HD Jet2<R, N> operator*(R b, const Jet2<R, N>& a) { return a * b; }
template <class R, int N>
CGB_HD Jet2<R, N> operator/(const Jet2<R, N>& a, R b) { return a * (R(1) / b); }
template <class R, int N>
CGB_HD Jet2<R, N> operator/(R a, const Jet2<R, N>& b) {
    const R q = a / b.v;
    return chain2(b, q, -q / b.v, R(2) * q / (b.v * b.v));
}

template <class R, int N>
CGB_HD Jet2<R, N> exp(const Jet2<R, N>& a) {
    const R e = Scal<R>::exp_(a.v);
    return chain2(a, e, e, e);
}
template <class R, int N>
CGB_HD Jet2<R, N> log(const Jet2<R, N>& a) {
    const R i = R(1) / a.v;
    return chain2(a, Scal<R>::log_(a.v), i, -i * i);
}
template <class R, int N>
CGB_HD Jet2<R, N> sqrt(const Jet2<R, N>& a) {
    const R s = Scal<R>::sqrt_(a.v);
    return chain2(a, s, R(0.5) / s, R(-0.25) / (s * a.v));
}
template <class R, int N>
CGB_HD Jet2<R, N> pow(const Jet2<R, N>& a, R p) {
    const R f = Scal<R>::pow_(a.v, p);
    const R i = R(1) / a.v;
    return chain2(a, f, p * f * i, p * (p - R(1)) * f * i * i);
}
template <class R, int N>
CGB_HD Jet2<R, N> pow3(const Jet2<R, N>& a, int k) {
    const R f = pow_third(a.v, k), p = R(k) / R(3);
    const R i = R(1) / a.v;
    return chain2(a, f, p * f * i, p * (p - R(1)) * f * i * i);
}
template <class R, int N>
CGB_HD Jet2<R, N> atan(const Jet2<R, N>& a) {
    const R q = R(1) / (R(1) + a.v * a.v);
    return chain2(a, Scal<R>::atan_(a.v), q, R(-2) * a.v * q * q);
}
template <class R, int N>
CGB_HD Jet2<R, N> asinh(const Jet2<R, N>& a) {
    const R q = R(1) / Scal<R>::sqrt_(R(1) + a.v * a.v);
    return chain2(a, Scal<R>::asinh_(a.v), q, -a.v * q * q * q);
}
template <class R, int N>
CGB_HD R val(const Jet2<R, N>& a) { return a.v; }

template <class T, class R>
CGB_HD T e_sum_gga(const FuncDesc& f, const XIn<T>& v) {
    T e(R(0));
    for (int i = 0; i < f.nids; i++) e = e + e_id_gga<T, R>(f.ids[i], v);
    return e;
}

// Restricted point, LDA (FAM 0) or GGA (FAM 1): eps, dv = (vrho, vsigma)
// and d2 = (v2rho2, v2rhosigma, v2sigma2), derivatives in the total rho and
// sigma as libxc's unpolarized kernels.  Zeros below the density threshold.
template <class R, int FAM>
CGB_HDN bool eval_unpol2(const FuncDesc& f, R rho, R sigma, R& eps, R* dv, R* d2) {
    constexpr int N = FAM == 0 ? 1 : 2;
    using T = Jet2<R, N>;
    for (int i = 0; i < 2; i++) dv[i] = R(0);
    for (int i = 0; i < 3; i++) d2[i] = R(0);
    eps = R(0);
    if (!(rho >= R(kDensThr))) return false;
    T r(rho), s(sigma);
    r.d[0] = R(1);
    if (N > 1) s.d[N - 1] = R(1);
    s = tmax(s, T(R(1.0000000000000011e-40)));  // kDensThr^(8/3)
    XIn<T> v{r * R(0.5), r * R(0.5), s * R(0.25), s * R(0.25), s * R(0.25), T(R(0)), T(R(0))};
    const T e = e_sum_gga<T, R>(f, v);
    eps = e.v / rho;
    for (int i = 0; i < N; i++) dv[i] = e.d[i];
    for (int k = 0; k < T::NH; k++) d2[k] = e.h[k];
    return true;
}

// Unrestricted point: in = (ra, rb, saa, sab, sbb); dv in the same order;
// d2 = v2rho2 (aa, ab, bb), v2rhosigma (a-aa, a-ab, a-bb, b-aa, b-ab, b-bb),
// v2sigma2 (aa-aa, aa-ab, aa-bb, ab-ab, ab-bb, bb-bb): libxc's polarized layouts.
template <class R, int FAM>
CGB_HDN bool eval_pol2(const FuncDesc& f, const R* in, R& eps, R* dv, R* d2) {
    constexpr int N = FAM == 0 ? 2 : 5;
    using T = Jet2<R, N>;
    for (int i = 0; i < 5; i++) dv[i] = R(0);
    for (int i = 0; i < 15; i++) d2[i] = R(0);
    eps = R(0);
    const R rt = in[0] + in[1];
    if (!(rt >= R(kDensThr))) return false;
    T x[5];
    for (int i = 0; i < 5; i++) {
        x[i] = T(in[i]);
        if (i < N) x[i].d[i] = R(1);
    }
    XIn<T> v{x[0], x[1], x[2], x[3], x[4], T(R(0)), T(R(0))};
    v.ra = tmax(v.ra, T(R(kDensThr)));
    v.rb = tmax(v.rb, T(R(kDensThr)));
    v.saa = tmax(v.saa, T(R(1.0000000000000011e-40)));
    v.sbb = tmax(v.sbb, T(R(1.0000000000000011e-40)));
    const T half = (v.saa + v.sbb) * R(0.5);
    v.sab = tmax(tmin(v.sab, half), -half);
    const T e = e_sum_gga<T, R>(f, v);
    eps = e.v / rt;
    for (int i = 0; i < N; i++) dv[i] = e.d[i];
    // Hessian (i <= j) of inputs 0..N-1 into the three libxc blocks
    auto H = [&](int i, int j) { return e.h[i * N - i * (i - 1) / 2 + j - i]; };
    d2[0] = H(0, 0);
    d2[1] = H(0, 1);
    d2[2] = H(1, 1);
    if (FAM >= 1) {
        for (int a = 0; a < 2; a++)
            for (int x2 = 0; x2 < 3; x2++) d2[3 + 3 * a + x2] = H(a, 2 + x2);
        int k = 9;
        for (int p = 2; p < 5; p++)
            for (int q = p; q < 5; q++) d2[k++] = H(p, q);
    }
    return true;
}

}  // namespace xcf
}  // namespace cgb
