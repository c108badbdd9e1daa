// Per-atom-pair MLP of the learned starting density: training (FP32 forward,
// backward, Adam) and inference (BF16 weights, FP32 accumulation) kernels.
//
// Network: x (nin) -> [Linear, SiLU] x nlayers (width nh) -> Linear (nout).
// Parameters are one flat FP32 vector, layer by layer: W (fan_in x fan_out,
// row-major) then b (fan_out).  Activations are row-major (batch x width).
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "common.h"
#include "xc_state.h"

namespace cgb {
namespace {

constexpr int kT = 64, kTK = 16, kGemmThreads = 256;

// C (M x N) = op(A) (M x K) * op(B) (K x N) [+ bias] ; row-major storage.
// TA: A stored K x M; TB: B stored N x K.  WB: B element type (float or bf16).
template <bool TA, bool TB, class WB>
__global__ void __launch_bounds__(kGemmThreads) gemm_kernel(int M, int N, int K, const float* __restrict__ A,
                                                            const WB* __restrict__ B, const float* __restrict__ bias,
                                                            float* __restrict__ C, int accumulate) {
    __shared__ float As[kTK][kT + 1], Bs[kTK][kT + 1];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int m0 = blockIdx.y * kT, n0 = blockIdx.x * kT;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += kTK) {
        for (int i = threadIdx.x; i < kTK * kT; i += kGemmThreads) {
            const int kk = i / kT, mm = i % kT;
            const int m = m0 + mm, k = k0 + kk;
            float a = 0.f;
            if (m < M && k < K) a = TA ? A[(size_t)k * M + m] : A[(size_t)m * K + k];
            As[kk][mm] = a;
            const int n = n0 + mm;
            float b = 0.f;
            if (n < N && k < K) b = (float)(TB ? B[(size_t)n * K + k] : B[(size_t)k * N + n]);
            Bs[kk][mm] = b;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kTK; kk++) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; i++) a[i] = As[kk][ty * 4 + i];
#pragma unroll
            for (int j = 0; j < 4; j++) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int m = m0 + ty * 4 + i, n = n0 + tx * 4 + j;
            if (m < M && n < N) {
                float v = acc[i][j] + (bias ? (float)bias[n] : 0.f);
                if (accumulate) v += C[(size_t)m * N + n];
                C[(size_t)m * N + n] = v;
            }
        }
}

__device__ __forceinline__ float silu(float z) { return z / (1.f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
    const float s = 1.f / (1.f + __expf(-z));
    return s * (1.f + z * (1.f - s));
}

__global__ void silu_kernel(long n, const float* __restrict__ z, float* __restrict__ h) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) h[i] = silu(z[i]);
}

// dz = dh * silu'(z)
__global__ void dsilu_kernel(long n, const float* __restrict__ z, const float* __restrict__ dh, float* __restrict__ dz) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dz[i] = dh[i] * dsilu(z[i]);
}

// db[j] = sum_i dz[i, j]
__global__ void colsum_kernel(int M, int N, const float* __restrict__ dz, float* __restrict__ db) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N) return;
    float s = 0.f;
    for (int i = 0; i < M; i++) s += dz[(size_t)i * N + j];
    db[j] = s;
}

// masked MSE: dY = 2 mask (y - t) / sum(mask); per-row partial losses
__global__ void mse_kernel(long n, const float* __restrict__ y, const float* __restrict__ t, const float* __restrict__ mask,
                           float inv_count, float* __restrict__ dy, float* __restrict__ loss_part) {
    __shared__ float red[256];
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.f;
    if (i < n) {
        const float d = (y[i] - t[i]) * mask[i];
        dy[i] = 2.f * d * inv_count;
        l = d * d * inv_count;
    }
    red[threadIdx.x] = l;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) loss_part[blockIdx.x] = red[0];
}

__global__ void adam_kernel(long n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

__global__ void to_bf16_kernel(long n, const float* __restrict__ x, __nv_bfloat16* __restrict__ y) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = __float2bfloat16_rn(x[i]);
}

template <bool TA, bool TB, class WB>
void gemm(int M, int N, int K, const float* A, const WB* B, const float* bias, float* C, bool acc, cudaStream_t s) {
    dim3 grid((N + kT - 1) / kT, (M + kT - 1) / kT);
    gemm_kernel<TA, TB, WB><<<grid, kGemmThreads, 0, s>>>(M, N, K, A, B, bias, C, acc ? 1 : 0);
    CGB_CUDA(cudaGetLastError());
}

unsigned blocks_for(long n) { return (unsigned)((n + 255) / 256); }

}  // namespace

struct Mlp {
    int nin, nh, nl, nout;
    std::vector<int> fan_in, fan_out;
    std::vector<long> w_off, b_off;
    long np = 0;
    int batch_cap = 0;
    DevBuf<float> p, g, m, v, x, y, t, mask, dy, loss_part;
    DevBuf<__nv_bfloat16> pb;  // bf16 copy of the parameters for inference
    bool pb_valid = false;
    std::vector<DevBuf<float>> z, h, dh, dz;  // per layer
    long step = 0;

    void init(int nin_, int nh_, int nl_, int nout_) {
        nin = nin_, nh = nh_, nl = nl_, nout = nout_;
        for (int l = 0; l <= nl; l++) {
            const int fi = l == 0 ? nin : nh, fo = l == nl ? nout : nh;
            fan_in.push_back(fi);
            fan_out.push_back(fo);
            w_off.push_back(np);
            np += (long)fi * fo;
            b_off.push_back(np);
            np += fo;
        }
        p.alloc(np);
        g.alloc(np);
        m.alloc(np);
        v.alloc(np);
        m.zero();
        v.zero();
        p.zero();
        z.resize(nl + 1);
        h.resize(nl + 1);
        dh.resize(nl + 1);
        dz.resize(nl + 1);
    }
    void ensure_batch(int B) {
        if (B <= batch_cap) return;
        batch_cap = B;
        x.alloc((size_t)B * nin);
        y.alloc((size_t)B * nout);
        t.alloc((size_t)B * nout);
        mask.alloc((size_t)B * nout);
        dy.alloc((size_t)B * nout);
        loss_part.alloc(((size_t)B * nout + 255) / 256);
        for (int l = 0; l <= nl; l++) {
            z[l].alloc((size_t)B * fan_out[l]);
            h[l].alloc((size_t)B * fan_out[l]);
            dh[l].alloc((size_t)B * fan_out[l]);
            dz[l].alloc((size_t)B * fan_out[l]);
        }
    }
    // FP32 forward on x (device); result in y.
    void forward(int B, cudaStream_t s) {
        const float* in = x.p;
        for (int l = 0; l <= nl; l++) {
            float* out = l == nl ? y.p : z[l].p;
            gemm<false, false, float>(B, fan_out[l], fan_in[l], in, p.p + w_off[l], p.p + b_off[l], out, false, s);
            if (l < nl) {
                silu_kernel<<<blocks_for((long)B * fan_out[l]), 256, 0, s>>>((long)B * fan_out[l], z[l].p, h[l].p);
                in = h[l].p;
            }
        }
    }
    // BF16-weight forward (inference).
    void forward_bf16(int B, cudaStream_t s) {
        if (!pb_valid) {
            pb.alloc(np);
            to_bf16_kernel<<<blocks_for(np), 256, 0, s>>>(np, p.p, pb.p);
            pb_valid = true;
        }
        const float* in = x.p;
        for (int l = 0; l <= nl; l++) {
            float* out = l == nl ? y.p : z[l].p;
            // bias stays FP32 (read from p)
            gemm<false, false, __nv_bfloat16>(B, fan_out[l], fan_in[l], in, pb.p + w_off[l], p.p + b_off[l], out, false, s);
            if (l < nl) {
                silu_kernel<<<blocks_for((long)B * fan_out[l]), 256, 0, s>>>((long)B * fan_out[l], z[l].p, h[l].p);
                in = h[l].p;
            }
        }
    }
    // Backward from dy (device) after forward(B); gradient into g.
    void backward(int B, cudaStream_t s) {
        const float* dout = dy.p;
        for (int l = nl; l >= 0; l--) {
            const float* dzl = dout;
            if (l < nl) {
                dsilu_kernel<<<blocks_for((long)B * fan_out[l]), 256, 0, s>>>((long)B * fan_out[l], z[l].p, dout, dz[l].p);
                dzl = dz[l].p;
            }
            const float* in = l == 0 ? x.p : h[l - 1].p;
            // dW = in^T dz  (fan_in x fan_out)
            gemm<true, false, float>(fan_in[l], fan_out[l], B, in, dzl, nullptr, g.p + w_off[l], false, s);
            colsum_kernel<<<(fan_out[l] + 127) / 128, 128, 0, s>>>(B, fan_out[l], dzl, g.p + b_off[l]);
            if (l > 0) {
                // dh_{l-1} = dz W^T  (B x fan_in)
                gemm<false, true, float>(B, fan_in[l], fan_out[l], dzl, p.p + w_off[l], nullptr, dh[l - 1].p, false, s);
                dout = dh[l - 1].p;
            }
        }
    }
};

}  // namespace cgb

using namespace cgb;

struct xc_mlp {
    Mlp m;
    cudaStream_t s = nullptr;
};

extern "C" {

int xc_mlp_create(int nin, int nhidden, int nlayers, int nout, xc_mlp** out) {
    return guard([&] {
        CGB_CHECK(nin > 0 && nhidden > 0 && nlayers >= 1 && nout > 0 && out, XC_ERR_ARG, "bad MLP shape");
        ensure_device();
        auto* h = new xc_mlp;
        try {
            h->m.init(nin, nhidden, nlayers, nout);
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
    });
}

int xc_mlp_destroy(xc_mlp* h) {
    delete h;
    return XC_OK;
}

int xc_mlp_nparams(const xc_mlp* h, long* n) {
    return guard([&] {
        CGB_CHECK(h && n, XC_ERR_ARG, "null argument");
        *n = h->m.np;
    });
}

int xc_mlp_set_params(xc_mlp* h, const float* params) {
    return guard([&] {
        CGB_CHECK(h && params, XC_ERR_ARG, "null argument");
        CGB_CUDA(cudaMemcpy(h->m.p.p, params, h->m.np * sizeof(float), cudaMemcpyHostToDevice));
        h->m.m.zero();
        h->m.v.zero();
        h->m.step = 0;
        h->m.pb_valid = false;
    });
}

int xc_mlp_get_params(const xc_mlp* h, float* params) {
    return guard([&] {
        CGB_CHECK(h && params, XC_ERR_ARG, "null argument");
        CGB_CUDA(cudaMemcpy(params, h->m.p.p, h->m.np * sizeof(float), cudaMemcpyDeviceToHost));
    });
}

int xc_mlp_forward(xc_mlp* h, int batch, const float* X, float* Y, int bf16) {
    return guard([&] {
        CGB_CHECK(h && X && Y && batch > 0, XC_ERR_ARG, "bad arguments");
        Mlp& m = h->m;
        m.ensure_batch(batch);
        CGB_CUDA(cudaMemcpy(m.x.p, X, (size_t)batch * m.nin * sizeof(float), cudaMemcpyHostToDevice));
        if (bf16) m.forward_bf16(batch, h->s);
        else m.forward(batch, h->s);
        CGB_CUDA(cudaMemcpy(Y, m.y.p, (size_t)batch * m.nout * sizeof(float), cudaMemcpyDeviceToHost));
    });
}

int xc_mlp_backward(xc_mlp* h, int batch, const float* X, const float* dY, float* grad) {
    return guard([&] {
        CGB_CHECK(h && X && dY && grad && batch > 0, XC_ERR_ARG, "bad arguments");
        Mlp& m = h->m;
        m.ensure_batch(batch);
        CGB_CUDA(cudaMemcpy(m.x.p, X, (size_t)batch * m.nin * sizeof(float), cudaMemcpyHostToDevice));
        m.forward(batch, h->s);
        CGB_CUDA(cudaMemcpy(m.dy.p, dY, (size_t)batch * m.nout * sizeof(float), cudaMemcpyHostToDevice));
        m.backward(batch, h->s);
        CGB_CUDA(cudaMemcpy(grad, m.g.p, m.np * sizeof(float), cudaMemcpyDeviceToHost));
    });
}

int xc_mlp_train_step(xc_mlp* h, int batch, const float* X, const float* T, const float* mask, float lr, float* loss) {
    return guard([&] {
        CGB_CHECK(h && X && T && mask && loss && batch > 0 && lr > 0, XC_ERR_ARG, "bad arguments");
        Mlp& m = h->m;
        m.ensure_batch(batch);
        const size_t ny = (size_t)batch * m.nout;
        CGB_CUDA(cudaMemcpy(m.x.p, X, (size_t)batch * m.nin * sizeof(float), cudaMemcpyHostToDevice));
        CGB_CUDA(cudaMemcpy(m.t.p, T, ny * sizeof(float), cudaMemcpyHostToDevice));
        CGB_CUDA(cudaMemcpy(m.mask.p, mask, ny * sizeof(float), cudaMemcpyHostToDevice));
        double cnt = 0;
        for (size_t i = 0; i < ny; i++) cnt += mask[i];
        CGB_CHECK(cnt > 0, XC_ERR_ARG, "empty mask");
        m.forward(batch, h->s);
        const unsigned nb = blocks_for((long)ny);
        mse_kernel<<<nb, 256, 0, h->s>>>((long)ny, m.y.p, m.t.p, m.mask.p, (float)(1.0 / cnt), m.dy.p, m.loss_part.p);
        m.backward(batch, h->s);
        m.step++;
        const float b1 = 0.9f, b2 = 0.999f;
        adam_kernel<<<blocks_for(m.np), 256, 0, h->s>>>(m.np, m.p.p, m.g.p, m.m.p, m.v.p, lr, b1, b2, 1e-8f,
                                                        1.f - std::pow(b1, (float)m.step), 1.f - std::pow(b2, (float)m.step));
        m.pb_valid = false;
        std::vector<float> parts(nb);
        CGB_CUDA(cudaMemcpy(parts.data(), m.loss_part.p, nb * sizeof(float), cudaMemcpyDeviceToHost));
        double l = 0;
        for (float x : parts) l += x;
        *loss = (float)l;
    });
}

}  // extern "C"
