// Response (coupled-perturbed) V_xc, FP64, LDA and GGA: the kernels behind
// ExchangeCorrelation::Evaluate("f") (ExchangeCorrelation.cpp:101-133,
// 192-199, 241-244), SubGrid::getDensityU (GridDensity.cpp:47-77) and
// SubGrid::getFockU<u_t> (GridFock.cpp:97-160).
//
// The response densities and the response V are the plain path's density
// and V kernels run with the (spin, matrix) pairs as their spin index; this
// file adds the second derivatives of the functional, the transposition that
// gives the reference's grad rho_U = 2 sum D_mu,nu grad phi_mu phi_nu
// orientation for a non-symmetric D_U, and the per-point coefficients
//   c0_s   = 1/2 w [sum_t f_(rho_s rho_t) rho_U,t + sum_x f_(rho_s sigma_x) sigma_U,x]
//   c1_s   = w sum_t S_st [dvsigma_(st) grad rho_t + vsigma_(st) grad rho_U,t]
//   dvsigma_x = sum_t f_(rho_t sigma_x) rho_U,t + sum_y f_(sigma_x sigma_y) sigma_U,y
// with sigma_U,(uv) = grad rho_U,u . grad rho_v + grad rho_u . grad rho_U,v and
// S = 2 on the spin diagonal, 1 across (restricted: totals, S = 2).  V_U built
// from them is the derivative of V_xc along D_U.
#include "common.h"
#include "kernels.h"

namespace cgb {
namespace {

constexpr int kThreads = 128;

template <int FAM, int NS>
__device__ __forceinline__ void fxc_point(const xcf::FuncDesc& f, const double* in, double* d2) {
    double e, dv[5];
    if (NS == 1) xcf::eval_unpol2<double, FAM>(f, in[0], in[2], e, dv, d2);
    else xcf::eval_pol2<double, FAM>(f, in, e, dv, d2);
}

// f2[k][Gp]: NS = 1: v2rho2, v2rhosigma, v2sigma2; NS = 2: the 3 + 6 + 6 libxc components.
template <int FAM, int NS>
__global__ void __launch_bounds__(kThreads) fxc_grid_kernel(xcf::FuncDesc f, long Gp, const double* __restrict__ rho,
                                                            const double* __restrict__ rho1, double* __restrict__ f2) {
    const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= Gp) return;
    constexpr int NK = NS == 1 ? 3 : 15;
    double in[5] = {rho[g], NS == 2 ? rho[Gp + g] : 0.0, 0, 0, 0};
    if (FAM >= 1) {
        double ga[3], gb[3] = {0, 0, 0};
#pragma unroll
        for (int r = 0; r < 3; r++) {
            ga[r] = rho1[r * Gp + g];
            if (NS == 2) gb[r] = rho1[(3 + r) * Gp + g];
        }
        in[2] = ga[0] * ga[0] + ga[1] * ga[1] + ga[2] * ga[2];
        if (NS == 2) {
            in[3] = ga[0] * gb[0] + ga[1] * gb[1] + ga[2] * gb[2];
            in[4] = gb[0] * gb[0] + gb[1] * gb[1] + gb[2] * gb[2];
        }
    }
    double d2[15];
    fxc_point<FAM, NS>(f, in, d2);
#pragma unroll
    for (int k = 0; k < NK; k++) f2[k * Gp + g] = d2[k];
}

// Caller arrays: rho (NS, n), sigma (1 or 3, n) -> v2rho2 (1 or 3, n), v2rhosigma (1 or 6, n), v2sigma2 (1 or 6, n).
template <int FAM, int NS>
__global__ void __launch_bounds__(kThreads) fxc_points_kernel(xcf::FuncDesc f, long n, const double* __restrict__ rho,
                                                              const double* __restrict__ sigma,
                                                              double* __restrict__ v2rho2,
                                                              double* __restrict__ v2rhosigma,
                                                              double* __restrict__ v2sigma2) {
    const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n) return;
    double in[5] = {rho[g], NS == 2 ? rho[n + g] : 0.0, 0, 0, 0};
    if (FAM >= 1) {
        in[2] = sigma[g];
        if (NS == 2) {
            in[3] = sigma[n + g];
            in[4] = sigma[2 * n + g];
        }
    }
    double d2[15];
    fxc_point<FAM, NS>(f, in, d2);
    if (NS == 1) {
        v2rho2[g] = d2[0];
        if (FAM >= 1) {
            v2rhosigma[g] = d2[1];
            v2sigma2[g] = d2[2];
        }
    } else {
#pragma unroll
        for (int k = 0; k < 3; k++) v2rho2[k * n + g] = d2[k];
        if (FAM >= 1) {
#pragma unroll
            for (int k = 0; k < 6; k++) {
                v2rhosigma[k * n + g] = d2[3 + k];
                v2sigma2[k * n + g] = d2[9 + k];
            }
        }
    }
}

// out[q](i, j) = in[q](j, i) for nq column-major n x n matrices (32 x 32 tiles through shared memory).
__global__ void __launch_bounds__(256) transpose_kernel(int n, const double* __restrict__ in, double* __restrict__ out) {
    __shared__ double t[32][33];
    const long q = blockIdx.z;
    const double* src = in + q * n * n;
    double* dst = out + q * n * n;
    const int i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
    for (int k = threadIdx.y; k < 32; k += 8) {
        const int i = i0 + threadIdx.x, j = j0 + k;  // element (i, j) of in, column j
        if (i < n && j < n) t[k][threadIdx.x] = src[(long)j * n + i];
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += 8) {
        const int j = j0 + threadIdx.x, i = i0 + k;  // out(j, i) = in(i, j), column i of out
        if (i < n && j < n) dst[(long)i * n + j] = t[threadIdx.x][k];
    }
}

// fcoefU[(q * 5 + k) * Gp + g] for q = s * nmat + m; component 4 (meta-GGA) is zero.
template <int FAM, int NS>
__global__ void __launch_bounds__(kThreads) response_coef_kernel(long Gp, int nmat, const double* __restrict__ w,
                                                                 const double* __restrict__ rho1,
                                                                 const double* __restrict__ vsigma,
                                                                 const double* __restrict__ f2,
                                                                 const double* __restrict__ rhoU,
                                                                 const double* __restrict__ rho1U,
                                                                 double* __restrict__ fcoefU) {
    const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int m = blockIdx.y;
    if (g >= Gp) return;
    const double wg = w[g];
    double rU[NS], gU[NS][3], gr[NS][3];
#pragma unroll
    for (int s = 0; s < NS; s++) {
        const long q = (long)s * nmat + m;
        rU[s] = rhoU[q * Gp + g];
#pragma unroll
        for (int r = 0; r < 3; r++) {
            gU[s][r] = FAM >= 1 ? rho1U[(q * 3 + r) * Gp + g] : 0.0;
            gr[s][r] = FAM >= 1 ? rho1[(s * 3 + r) * Gp + g] : 0.0;
        }
    }
    auto dot = [](const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
    double c0[NS], c1[NS][3];
    if (NS == 1) {
        const double frr = f2[g], frs = FAM >= 1 ? f2[Gp + g] : 0.0, fss = FAM >= 1 ? f2[2 * Gp + g] : 0.0;
        const double sU = 2.0 * dot(gU[0], gr[0]);
        c0[0] = 0.5 * wg * (frr * rU[0] + frs * sU);
        const double t1 = 2.0 * (frs * rU[0] + fss * sU);
        const double vs = FAM >= 1 ? vsigma[g] : 0.0;
#pragma unroll
        for (int r = 0; r < 3; r++) c1[0][r] = wg * (t1 * gr[0][r] + 2.0 * vs * gU[0][r]);
    } else {
        // f2 rows: rho-rho (aa, ab, bb) 0..2; rho_t-sigma_x 3 + 3 t + x; sigma-sigma upper triangle 9..14
        double sU[3] = {0, 0, 0};
        if (FAM >= 1) {
            sU[0] = 2.0 * dot(gU[0], gr[0]);
            sU[1] = dot(gU[0], gr[1]) + dot(gr[0], gU[1]);
            sU[2] = 2.0 * dot(gU[1], gr[1]);
        }
        auto F = [&](int k) { return f2[(long)k * Gp + g]; };
        auto fss = [&](int x, int y) {
            const int a = x < y ? x : y, b = x < y ? y : x;
            return F(9 + a * 3 - a * (a - 1) / 2 + b - a);
        };
        double dvs[3] = {0, 0, 0}, vs[3] = {0, 0, 0};
        if (FAM >= 1) {
#pragma unroll
            for (int x = 0; x < 3; x++) {
                dvs[x] = F(3 + x) * rU[0] + F(6 + x) * rU[1];
#pragma unroll
                for (int y = 0; y < 3; y++) dvs[x] += fss(x, y) * sU[y];
                vs[x] = vsigma[(long)x * Gp + g];
            }
        }
#pragma unroll
        for (int s = 0; s < 2; s++) {
            double t0 = F(s) * rU[0] + F(s + 1) * rU[1];  // f_(rho_s rho_a), f_(rho_s rho_b)
            if (FAM >= 1)
#pragma unroll
                for (int x = 0; x < 3; x++) t0 += F(3 + 3 * s + x) * sU[x];
            c0[s] = 0.5 * wg * t0;
#pragma unroll
            for (int r = 0; r < 3; r++) {
                double c = 0;
#pragma unroll
                for (int t = 0; t < 2; t++) {
                    const int x = s + t;
                    const double S = s == t ? 2.0 : 1.0;
                    c += S * (dvs[x] * gr[t][r] + vs[x] * gU[t][r]);
                }
                c1[s][r] = wg * c;
            }
        }
    }
#pragma unroll
    for (int s = 0; s < NS; s++) {
        double* o = fcoefU + ((long)s * nmat + m) * 5 * Gp + g;
        o[0] = c0[s];
#pragma unroll
        for (int r = 0; r < 3; r++) o[(1 + r) * Gp] = FAM >= 1 ? c1[s][r] : 0.0;
        o[4 * Gp] = 0.0;
    }
}

}  // namespace

void launch_fxc(const xcf::FuncDesc& f, int fam, int ns, long Gp, const double* rho, const double* rho1, double* f2,
                cudaStream_t s) {
    CGB_CHECK(fam <= 1, XC_ERR_UNSUPPORTED, "second derivatives cover LDA and GGA (as the reference's Evaluate(\"f\"))");
    if (Gp == 0) return;
    const unsigned grid = (unsigned)((Gp + kThreads - 1) / kThreads);
    if (ns == 1) {
        if (fam == 0) fxc_grid_kernel<0, 1><<<grid, kThreads, 0, s>>>(f, Gp, rho, rho1, f2);
        else fxc_grid_kernel<1, 1><<<grid, kThreads, 0, s>>>(f, Gp, rho, rho1, f2);
    } else {
        if (fam == 0) fxc_grid_kernel<0, 2><<<grid, kThreads, 0, s>>>(f, Gp, rho, rho1, f2);
        else fxc_grid_kernel<1, 2><<<grid, kThreads, 0, s>>>(f, Gp, rho, rho1, f2);
    }
    CGB_CUDA(cudaGetLastError());
}

void launch_fxc_points(const xcf::FuncDesc& f, int fam, int ns, long n, const double* rho, const double* sigma,
                       double* v2rho2, double* v2rhosigma, double* v2sigma2, cudaStream_t s) {
    CGB_CHECK(fam <= 1, XC_ERR_UNSUPPORTED, "second derivatives cover LDA and GGA (as the reference's Evaluate(\"f\"))");
    if (n == 0) return;
    const unsigned grid = (unsigned)((n + kThreads - 1) / kThreads);
#define CGB_FX(FAM_, NS_) \
    fxc_points_kernel<FAM_, NS_><<<grid, kThreads, 0, s>>>(f, n, rho, sigma, v2rho2, v2rhosigma, v2sigma2)
    if (ns == 1) {
        if (fam == 0) CGB_FX(0, 1);
        else CGB_FX(1, 1);
    } else {
        if (fam == 0) CGB_FX(0, 2);
        else CGB_FX(1, 2);
    }
#undef CGB_FX
    CGB_CUDA(cudaGetLastError());
}

void launch_transpose_batch(int n, long nmat, const double* in, double* out, cudaStream_t s) {
    if (n == 0 || nmat == 0) return;
    CGB_CHECK(nmat <= 65535, XC_ERR_ARG, "at most 65535 matrices per transposition");
    const unsigned t = (unsigned)((n + 31) / 32);
    transpose_kernel<<<dim3(t, t, (unsigned)nmat), dim3(32, 8), 0, s>>>(n, in, out);
    CGB_CUDA(cudaGetLastError());
}

void launch_response_coef(int fam, int ns, long Gp, int nmat, const double* w, const double* rho1,
                          const double* vsigma, const double* f2, const double* rhoU, const double* rho1U,
                          double* fcoefU, cudaStream_t s) {
    CGB_CHECK(fam <= 1, XC_ERR_UNSUPPORTED, "response V_xc covers LDA and GGA (as the reference's getFockU)");
    CGB_CHECK(nmat >= 1 && nmat <= 65535, XC_ERR_ARG, "between 1 and 65535 response matrices per launch");
    if (Gp == 0) return;
    const dim3 grid((unsigned)((Gp + kThreads - 1) / kThreads), (unsigned)nmat);
#define CGB_RC(FAM_, NS_) \
    response_coef_kernel<FAM_, NS_><<<grid, kThreads, 0, s>>>(Gp, nmat, w, rho1, vsigma, f2, rhoU, rho1U, fcoefU)
    if (ns == 1) {
        if (fam == 0) CGB_RC(0, 1);
        else CGB_RC(1, 1);
    } else {
        if (fam == 0) CGB_RC(0, 2);
        else CGB_RC(1, 2);
    }
#undef CGB_RC
    CGB_CUDA(cudaGetLastError());
}

}  // namespace cgb
