// Pointwise functional kernel (ExchangeCorrelation::Evaluate "ev",
// ExchangeCorrelation.cpp:165-248), the E_xc partial sums
// (EnergyEinSum W,Rho,Eps->E) and the per-point Fock coefficients that the
// V_xc kernel consumes:
//   fcoef(s, 0)   = 1/2 w vrho_s
//   fcoef(s, 1:4) = w (2 vsigma_ss grad rho_s + vsigma_ab grad rho_s')   (restricted: 2 w vsigma grad rho)
//   fcoef(s, 4)   = 1/4 w vtau_s
// so that V_s = sum_g [phi A + A^T phi] with A = c0 phi + c1 . grad phi (+ c2 grad phi grad phi),
// which equals GridFock.cpp:11-49 after its F + F^T step.
#include "common.h"
#include "kernels.h"

namespace cgb {
namespace {

constexpr int kThreads = 128;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Fixed-order CTA sum (deterministic for a given launch shape).
__device__ double cta_sum(double v) {
    __shared__ double s[32];
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) s[wid] = v;
    __syncthreads();
    double r = 0;
    if (wid == 0) {
        r = lane < (int)(blockDim.x >> 5) ? s[lane] : 0.0;
        r = warp_sum(r);
    }
    __syncthreads();
    return r;
}

// MODE 1: only the points whose total density is >= float_above: the
// potentials in FP32 (forward-mode derivatives of the FP32 expression) and
// the energy density eps at FP64 level (the value alone, in float-float
// arithmetic on the FP32 pipe; in FP64 at a point where that overflows
// FP32's range) -- float constants and float k/3 exponents shift an FP32 eps
// systematically by 1e-8..1e-7 relative, which E_xc = sum w rho eps would
// accumulate, while V takes FP32-level errors;
// MODE 2: only the others, in FP64 (float_above = +inf: every point).  The
// mixed path runs both launches (separate kernels: each gets the registers
// and occupancy of its own precision); accumulate adds the CTA's energy
// partial to the first launch's.
template <int FAM, int NS, int MODE>
__global__ void __launch_bounds__(kThreads) functional_kernel(xcf::FuncDesc f, long Gp, const double* __restrict__ w,
                                                              const double* __restrict__ rho,
                                                              const double* __restrict__ rho1,
                                                              const double* __restrict__ tau,
                                                              double* __restrict__ sigma, double* __restrict__ eps,
                                                              double* __restrict__ vrho, double* __restrict__ vsigma,
                                                              double* __restrict__ vtau, double* __restrict__ fcoef,
                                                              double* __restrict__ e_partial, double float_above,
                                                              bool accumulate) {
    const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
    double econtrib = 0;
    bool mine = g < Gp;
    if (mine) {
        const double tot_rho = NS == 1 ? rho[g] : rho[g] + rho[Gp + g];
        mine = (tot_rho >= float_above) == (MODE == 1);
    }
    if (mine) {
        const double wg = w[g];
        if (NS == 1) {
            const double r = rho[g];
            double gx = 0, gy = 0, gz = 0, s = 0, t = 0;
            if (FAM >= 1) {
                gx = rho1[g];
                gy = rho1[Gp + g];
                gz = rho1[2 * Gp + g];
                s = gx * gx + gy * gy + gz * gz;
                sigma[g] = s;
            }
            if (FAM >= 2) t = tau[g];
            double e, dv[3] = {0, 0, 0};
            if (MODE == 1) {  // mixed path: FP32 potentials, FP64 eps, above the low-density bound
                float ef, df[3] = {0, 0, 0};
                xcf::eval_unpol<float, FAM>(f, (float)r, (float)s, (float)t, ef, df);
                // the energy density in float-float (FP64-level, on the FP32 pipe);
                // FP64 where an intermediate left FP32's exponent range
                xcf::ff eff;
                xcf::eval_unpol_value<xcf::ff, FAM>(f, xcf::ff(r), xcf::ff(s), xcf::ff(t), eff);
                e = xcf::ff_value(eff);
                if (!isfinite(e)) xcf::eval_unpol_value<double, FAM>(f, r, s, t, e);
                for (int i = 0; i < 3; i++) dv[i] = df[i];
            } else {
                xcf::eval_unpol<double, FAM>(f, r, s, t, e, dv);
            }
            eps[g] = e;
            vrho[g] = dv[0];
            if (FAM >= 1) vsigma[g] = dv[1];
            if (FAM >= 2) vtau[g] = dv[2];
            econtrib = wg * r * e;
            fcoef[g] = 0.5 * wg * dv[0];
            const double c1 = FAM >= 1 ? 2.0 * wg * dv[1] : 0.0;
            fcoef[Gp + g] = c1 * gx;
            fcoef[2 * Gp + g] = c1 * gy;
            fcoef[3 * Gp + g] = c1 * gz;
            fcoef[4 * Gp + g] = FAM >= 2 ? 0.25 * wg * dv[2] : 0.0;
        } else {
            double in[7] = {rho[g], rho[Gp + g], 0, 0, 0, 0, 0};
            double ga[3] = {0, 0, 0}, gb[3] = {0, 0, 0};
            if (FAM >= 1) {
#pragma unroll
                for (int r = 0; r < 3; r++) {
                    ga[r] = rho1[r * Gp + g];
                    gb[r] = rho1[(3 + r) * Gp + g];
                }
                in[2] = ga[0] * ga[0] + ga[1] * ga[1] + ga[2] * ga[2];
                in[3] = ga[0] * gb[0] + ga[1] * gb[1] + ga[2] * gb[2];
                in[4] = gb[0] * gb[0] + gb[1] * gb[1] + gb[2] * gb[2];
                sigma[g] = in[2];
                sigma[Gp + g] = in[3];
                sigma[2 * Gp + g] = in[4];
            }
            if (FAM >= 2) {
                in[5] = tau[g];
                in[6] = tau[Gp + g];
            }
            double e, dv[7] = {0, 0, 0, 0, 0, 0, 0};
            if (MODE == 1) {
                float inf_[7], ef, df[7] = {0, 0, 0, 0, 0, 0, 0};
                for (int i = 0; i < 7; i++) inf_[i] = (float)in[i];
                xcf::eval_pol<float, FAM>(f, inf_, ef, df);
                xcf::ff inff[7], eff;
                for (int i = 0; i < 7; i++) inff[i] = xcf::ff(in[i]);
                xcf::eval_pol_value<xcf::ff, FAM>(f, inff, eff);
                e = xcf::ff_value(eff);
                if (!isfinite(e)) xcf::eval_pol_value<double, FAM>(f, in, e);
                for (int i = 0; i < 7; i++) dv[i] = df[i];
            } else {
                xcf::eval_pol<double, FAM>(f, in, e, dv);
            }
            eps[g] = e;
            vrho[g] = dv[0];
            vrho[Gp + g] = dv[1];
            if (FAM >= 1) {
                vsigma[g] = dv[2];
                vsigma[Gp + g] = dv[3];
                vsigma[2 * Gp + g] = dv[4];
            }
            if (FAM >= 2) {
                vtau[g] = dv[5];
                vtau[Gp + g] = dv[6];
            }
            econtrib = wg * (in[0] + in[1]) * e;
            // spin a then b: c1 = w (2 vsigma_ss grad rho_s + vsigma_ab grad rho_s')
            for (int s = 0; s < 2; s++) {
                double* fc = fcoef + (long)s * 5 * Gp;
                const double* gs = s == 0 ? ga : gb;
                const double* go = s == 0 ? gb : ga;
                const double vss = FAM >= 1 ? dv[s == 0 ? 2 : 4] : 0.0, vab = FAM >= 1 ? dv[3] : 0.0;
                fc[g] = 0.5 * wg * dv[s];
#pragma unroll
                for (int r = 0; r < 3; r++) fc[(1 + r) * Gp + g] = wg * (2.0 * vss * gs[r] + vab * go[r]);
                fc[4 * Gp + g] = FAM >= 2 ? 0.25 * wg * dv[5 + s] : 0.0;
            }
        }
    }
    const double tot = cta_sum(econtrib);
    if (threadIdx.x == 0) e_partial[blockIdx.x] = accumulate ? e_partial[blockIdx.x] + tot : tot;
}

__global__ void reduce_kernel(const double* __restrict__ partial, int n, double* __restrict__ out) {
    double v = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) v += partial[i];
    const double t = cta_sum(v);
    if (threadIdx.x == 0) out[0] = t;
}

__global__ void nelec_kernel(long Gp, int ns, const double* __restrict__ w, const double* __restrict__ rho,
                             double* __restrict__ partial) {
    const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0;
    if (g < Gp) {
        double wr = 0;
        for (int s = 0; s < ns; s++) wr += w[g] * rho[s * Gp + g];
        v = wr;
    }
    const double t = cta_sum(v);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

// GuessSCF.cpp:38-57: nearest tabulated radius (first minimum on ties), r += 1e-12.
__global__ void sap_kernel(long Gp, int natoms, const double* __restrict__ atoms, const double* __restrict__ table,
                           const double* __restrict__ radii, const double* __restrict__ px,
                           const double* __restrict__ py, const double* __restrict__ pz,
                           const double* __restrict__ w, double* __restrict__ fcoef) {
    const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= Gp) return;
    double acc = 0;
    for (int a = 0; a < natoms; a++) {
        const double x = px[g] - atoms[3 * a], y = py[g] - atoms[3 * a + 1], z = pz[g] - atoms[3 * a + 2];
        const double r = sqrt(x * x + y * y + z * z) + 1.e-12;
        // radii ascend: binary search for the last radius <= r, then compare neighbours
        int lo = 0, hi = 750;
        if (r <= radii[0]) hi = 0;
        else if (r >= radii[750]) lo = hi = 750;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (radii[mid] <= r) lo = mid;
            else hi = mid;
        }
        int k = lo;
        if (hi != lo && fabs(radii[hi] - r) < fabs(radii[lo] - r)) k = hi;
        acc += table[a * 751 + k] / r;
    }
    fcoef[g] = 0.5 * w[g] * acc;
    fcoef[Gp + g] = fcoef[2 * Gp + g] = fcoef[3 * Gp + g] = fcoef[4 * Gp + g] = 0.0;
}

template <int FAM, int NS>
__global__ void points_kernel(xcf::FuncDesc f, long n, const double* __restrict__ rho, const double* __restrict__ sigma,
                              const double* __restrict__ tau, double* __restrict__ eps, double* __restrict__ vrho,
                              double* __restrict__ vsigma, double* __restrict__ vtau) {
    const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n) return;
    if (NS == 1) {
        double e, dv[3] = {0, 0, 0};
        xcf::eval_unpol<double, FAM>(f, rho[g], FAM >= 1 ? sigma[g] : 0.0, FAM >= 2 ? tau[g] : 0.0, e, dv);
        eps[g] = e;
        vrho[g] = dv[0];
        if (FAM >= 1) vsigma[g] = dv[1];
        if (FAM >= 2) vtau[g] = dv[2];
    } else {
        double in[7] = {rho[g], rho[n + g], 0, 0, 0, 0, 0};
        if (FAM >= 1) {
            in[2] = sigma[g];
            in[3] = sigma[n + g];
            in[4] = sigma[2 * n + g];
        }
        if (FAM >= 2) {
            in[5] = tau[g];
            in[6] = tau[n + g];
        }
        double e, dv[7] = {0, 0, 0, 0, 0, 0, 0};
        xcf::eval_pol<double, FAM>(f, in, e, dv);
        eps[g] = e;
        vrho[g] = dv[0];
        vrho[n + g] = dv[1];
        if (FAM >= 1) {
            vsigma[g] = dv[2];
            vsigma[n + g] = dv[3];
            vsigma[2 * n + g] = dv[4];
        }
        if (FAM >= 2) {
            vtau[g] = dv[5];
            vtau[n + g] = dv[6];
        }
    }
}

}  // namespace

void launch_functional_fp64(const xcf::FuncDesc& f, int fam, int ns, long Gp, const double* w, const double* rho,
                            const double* rho1, const double* tau, double* sigma, double* eps, double* vrho,
                            double* vsigma, double* vtau, double* fcoef, double* e_partial, int* n_partial,
                            cudaStream_t s, double float_above) {
    const unsigned grid = (unsigned)((Gp + kThreads - 1) / kThreads);
    *n_partial = (int)grid;
    // FP32 points first (mixed path only), then the FP64 ones adding to the same CTA partials
    const bool split = float_above < __builtin_huge_val();
#define CGB_FN(FAM_, NS_, MODE_, ACC_)                                                                          \
    functional_kernel<FAM_, NS_, MODE_><<<grid, kThreads, 0, s>>>(f, Gp, w, rho, rho1, tau, sigma, eps, vrho, vsigma, \
                                                                  vtau, fcoef, e_partial, float_above, ACC_)
#define CGB_FN2(FAM_, NS_)                       \
    do {                                         \
        if (split) CGB_FN(FAM_, NS_, 1, false);  \
        CGB_FN(FAM_, NS_, 2, split);             \
    } while (0)
    if (ns == 1) {
        if (fam == 0) CGB_FN2(0, 1);
        else if (fam == 1) CGB_FN2(1, 1);
        else CGB_FN2(2, 1);
    } else {
        if (fam == 0) CGB_FN2(0, 2);
        else if (fam == 1) CGB_FN2(1, 2);
        else CGB_FN2(2, 2);
    }
#undef CGB_FN2
#undef CGB_FN
    CGB_CUDA(cudaGetLastError());
}

void launch_reduce_sum(const double* partial, int n, double* out, cudaStream_t s) {
    reduce_kernel<<<1, 1024, 0, s>>>(partial, n, out);
    CGB_CUDA(cudaGetLastError());
}

void launch_num_electrons(long Gp, int ns, const double* w, const double* rho, double* partial, int* n_partial,
                          cudaStream_t s) {
    const unsigned grid = (unsigned)((Gp + kThreads - 1) / kThreads);
    *n_partial = (int)grid;
    nelec_kernel<<<grid, kThreads, 0, s>>>(Gp, ns, w, rho, partial);
    CGB_CUDA(cudaGetLastError());
}

void launch_sap_coef(long Gp, int natoms, const double* atoms, const double* table, const double* radii,
                     const double* x, const double* y, const double* z, const double* w, double* fcoef,
                     cudaStream_t s) {
    const unsigned grid = (unsigned)((Gp + kThreads - 1) / kThreads);
    sap_kernel<<<grid, kThreads, 0, s>>>(Gp, natoms, atoms, table, radii, x, y, z, w, fcoef);
    CGB_CUDA(cudaGetLastError());
}

void launch_functional_points(const xcf::FuncDesc& f, int fam, int ns, long n, const double* rho, const double* sigma,
                              const double* tau, double* eps, double* vrho, double* vsigma, double* vtau,
                              cudaStream_t s) {
    const unsigned grid = (unsigned)((n + kThreads - 1) / kThreads);
#define CGB_PT(FAM_, NS_) points_kernel<FAM_, NS_><<<grid, kThreads, 0, s>>>(f, n, rho, sigma, tau, eps, vrho, vsigma, vtau)
    if (ns == 1) {
        if (fam == 0) CGB_PT(0, 1);
        else if (fam == 1) CGB_PT(1, 1);
        else CGB_PT(2, 1);
    } else {
        if (fam == 0) CGB_PT(0, 2);
        else if (fam == 1) CGB_PT(1, 2);
        else CGB_PT(2, 2);
    }
#undef CGB_PT
    CGB_CUDA(cudaGetLastError());
}

}  // namespace cgb
