// Allocation-free variant of the functional + E_xc kernel pair.
//
// Who needs it: callers that may not call cudaMalloc / cudaFree -- for
// instance code whose device memory is owned entirely by another allocator
// (a framework's caching pool or a pre-reserved arena leaves nothing for a
// second allocator), or code that must not issue cudaMalloc / cudaFree in a
// hot loop because those calls synchronise the device and stall work queued
// on other streams.  Such a caller owns its input and output buffers and
// calls xc_functional_energy_static(); the per-CTA energy partials, the only
// scratch this computation needs, live in a fixed array compiled into the
// library instead of being allocated.
//
// The array holds kStaticPartials doubles (128 KiB) on every GPU that loads
// the library, until the process exits.  One partial per 128 points bounds a
// call to kStaticPartials * 128 = 2 097 152 points.  All calls share the
// array: each call overwrites the partials it uses before reading them, so
// nothing has to start at zero, but two calls whose kernels overlap on the
// GPU (different streams, or different host threads) race on it and must be
// serialised by the caller.
#include <mutex>

#include "common.h"
#include "functional.cuh"
#include "xc_state.h"

namespace cgb {
namespace {

constexpr int kStaticThreads = 128;
constexpr int kStaticPartials = 16384;
constexpr long kStaticMaxPoints = (long)kStaticPartials * kStaticThreads;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_energy_partials[kStaticPartials];

// Device address of g_energy_partials per device, looked up with that device
// current (the host-side symbol is only a stand-in).  Only a successful
// lookup is kept: a failed one (for instance a first call made while the
// stream is being captured) is retried by the next call.
std::mutex g_partials_mu;
double* g_partials_addr[kMaxDevices] = {};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__device__ double block_sum(double v) {
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

// eps, potentials and sum_g w_g rho_g eps_g partial of this CTA's points.
template <int FAM, int NS>
__global__ void __launch_bounds__(kStaticThreads) static_energy_kernel(
    xcf::FuncDesc f, long n, const double* __restrict__ w, const double* __restrict__ rho,
    const double* __restrict__ sigma, const double* __restrict__ tau, double* __restrict__ eps,
    double* __restrict__ vrho, double* __restrict__ vsigma, double* __restrict__ vtau, double* __restrict__ partials) {
    const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
    double contrib = 0;
    if (g < n) {
        if (NS == 1) {
            double e, dv[3] = {0, 0, 0};
            const double r = rho[g];
            xcf::eval_unpol<double, FAM>(f, r, FAM >= 1 ? sigma[g] : 0.0, FAM >= 2 ? tau[g] : 0.0, e, dv);
            eps[g] = e;
            vrho[g] = dv[0];
            if (FAM >= 1) vsigma[g] = dv[1];
            if (FAM >= 2) vtau[g] = dv[2];
            contrib = w[g] * r * e;
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
            contrib = w[g] * (in[0] + in[1]) * e;
        }
    }
    const double tot = block_sum(contrib);
    if (threadIdx.x == 0) partials[blockIdx.x] = tot;
}

// Fixed-order sum of the first np partials into E.
__global__ void static_reduce_kernel(const double* __restrict__ partials, int np, double* __restrict__ E) {
    double v = 0;
    for (int i = threadIdx.x; i < np; i += blockDim.x) v += partials[i];
    const double t = block_sum(v);
    if (threadIdx.x == 0) E[0] = t;
}

}  // namespace
}  // namespace cgb

using namespace cgb;

extern "C" int xc_functional_energy_static(const xc_functional* fh, long npoints, const double* d_w,
                                           const double* d_rho, const double* d_sigma, const double* d_tau,
                                           double* d_eps, double* d_vrho, double* d_vsigma, double* d_vtau,
                                           double* d_E, void* stream) {
    return guard([&] {
        CGB_CHECK(fh && d_w && d_rho && d_eps && d_vrho && d_E, XC_ERR_ARG, "null argument");
        CGB_CHECK(npoints > 0, XC_ERR_ARG, "npoints must be positive");
        CGB_CHECK(npoints <= kStaticMaxPoints, XC_ERR_ARG,
                  "xc_functional_energy_static: npoints exceeds the static scratch limit of 2097152 points "
                  "(16384 partials x 128); split the call or use the allocating entry points");
        const Functional& F = fh->f;
        CGB_CHECK(F.family < 1 || (d_sigma && d_vsigma), XC_ERR_ARG, "sigma arrays required for GGA");
        CGB_CHECK(F.family < 2 || (d_tau && d_vtau), XC_ERR_ARG, "tau arrays required for meta-GGA");
        int dev = -1;
        CGB_CUDA(cudaGetDevice(&dev));
        CGB_CHECK(dev >= 0 && dev < kMaxDevices, XC_ERR_CUDA, "device index out of range");
        // first successful call on this device: resolve the array's device address
        double* partials = nullptr;
        {
            std::lock_guard<std::mutex> lk(g_partials_mu);
            if (!g_partials_addr[dev]) {
                void* p = nullptr;
                const cudaError_t st = cudaGetSymbolAddress(&p, g_energy_partials);
                if (st != cudaSuccess || !p) {
                    cudaGetLastError();  // not sticky: the next call looks the address up again
                    throw Error(XC_ERR_CUDA, std::string("cudaGetSymbolAddress of the static energy scratch failed (") +
                                                 cudaGetErrorString(st) + "); the next call retries the lookup");
                }
                g_partials_addr[dev] = (double*)p;
            }
            partials = g_partials_addr[dev];
        }
        cudaStream_t s = (cudaStream_t)stream;
        const unsigned grid = (unsigned)((npoints + kStaticThreads - 1) / kStaticThreads);
#define CGB_ST(FAM_, NS_)                                                                                  \
    static_energy_kernel<FAM_, NS_><<<grid, kStaticThreads, 0, s>>>(F.desc, npoints, d_w, d_rho, d_sigma, \
                                                                    d_tau, d_eps, d_vrho, d_vsigma, d_vtau, partials)
        if (F.nspin == 1) {
            if (F.family == 0) CGB_ST(0, 1);
            else if (F.family == 1) CGB_ST(1, 1);
            else CGB_ST(2, 1);
        } else {
            if (F.family == 0) CGB_ST(0, 2);
            else if (F.family == 1) CGB_ST(1, 2);
            else CGB_ST(2, 2);
        }
#undef CGB_ST
        CGB_CUDA(cudaGetLastError());
        static_reduce_kernel<<<1, 1024, 0, s>>>(partials, (int)grid, d_E);
        CGB_CUDA(cudaGetLastError());
    });
}
