// Per-atom-pair MLP of the learned starting density: training (FP32-level
// forward, backward, Adam) and inference (BF16 weights, FP32 activations).
//
// Network: x (nin) -> [Linear, SiLU] x nlayers (width nh) -> Linear (nout).
// Parameters are one flat FP32 vector, layer by layer: W (fan_in x fan_out,
// row-major) then b (fan_out).  Activations are row-major (batch x width).
//
// Every product runs on the tensor cores (tc_gemm, k_tcgemm.cu): training
// splits both operands into three BF16 planes (six cross products, FP32-level
// sums); inference keeps the weights as one BF16 plane (cached until the
// parameters change) against three activation planes.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "common.h"
#include "mixed.h"
#include "xc_state.h"

namespace cgb {
namespace {

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

unsigned blocks_for(long n) { return (unsigned)((n + 255) / 256); }

}  // namespace

struct Mlp {
    int nin, nh, nl, nout;
    std::vector<int> fan_in, fan_out;
    std::vector<long> w_off, b_off;
    long np = 0;
    int batch_cap = 0;
    DevBuf<float> p, g, m, v, x, y, t, mask, dy, loss_part;
    DevBuf<__nv_bfloat16> pa, pb;          // operand planes of the current product
    std::vector<DevBuf<__nv_bfloat16>> wt;  // inference: W^T of each layer, one BF16 plane
    bool wt_valid = false;
    DevBuf<int> err;
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
        err.alloc(1);
        err.zero();
        z.resize(nl + 1);
        h.resize(nl + 1);
        dh.resize(nl + 1);
        dz.resize(nl + 1);
        wt.resize(nl + 1);
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
    // Planes of src(r, k) = src[r*ld_r + k*ld_k] (rows x kdim) in buf.
    static void planes(DevBuf<__nv_bfloat16>& buf, const float* src, int rows, int kdim, long ld_r, long ld_k, int np_,
                       cudaStream_t s) {
        const size_t need = (size_t)np_ * tc_pad_rows(rows) * tc_pad_k(kdim);
        if (buf.n < need) buf.alloc(need);
        tc_to_planes(src, rows, kdim, ld_r, ld_k, np_, buf.p, s);
    }
    // Y (B x fo) = X (B x fi) W + b for layer l; weights 3 planes (training) or
    // the cached BF16 plane (inference).
    void linear(int l, int B, const float* in, float* out, bool bf16, cudaStream_t s) {
        const int fi = fan_in[l], fo = fan_out[l];
        planes(pa, in, B, fi, fi, 1, 3, s);
        const __nv_bfloat16* wb;
        if (bf16) {
            wb = wt[l].p;
        } else {
            planes(pb, p.p + w_off[l], fo, fi, 1, fo, 3, s);  // W^T: row n, column k = W[k][n]
            wb = pb.p;
        }
        tc_gemm(pa.p, 3, wb, bf16 ? 1 : 3, B, fo, fi, p.p + b_off[l], out, fo, false, err.p, s);
    }
    void forward_any(int B, bool bf16, cudaStream_t s) {
        if (bf16 && !wt_valid) {
            for (int l = 0; l <= nl; l++) planes(wt[l], p.p + w_off[l], fan_out[l], fan_in[l], 1, fan_out[l], 1, s);
            wt_valid = true;
        }
        const float* in = x.p;
        for (int l = 0; l <= nl; l++) {
            float* out = l == nl ? y.p : z[l].p;
            linear(l, B, in, out, bf16, s);
            if (l < nl) {
                silu_kernel<<<blocks_for((long)B * fan_out[l]), 256, 0, s>>>((long)B * fan_out[l], z[l].p, h[l].p);
                in = h[l].p;
            }
        }
    }
    // FP32-level forward on x (device); result in y.
    void forward(int B, cudaStream_t s) { forward_any(B, false, s); }
    // BF16-weight forward (inference).
    void forward_bf16(int B, cudaStream_t s) { forward_any(B, true, s); }
    // Backward from dy (device) after forward(B); gradient into g.
    void backward(int B, cudaStream_t s) {
        const float* dout = dy.p;
        for (int l = nl; l >= 0; l--) {
            const int fi = fan_in[l], fo = fan_out[l];
            const float* dzl = dout;
            if (l < nl) {
                dsilu_kernel<<<blocks_for((long)B * fo), 256, 0, s>>>((long)B * fo, z[l].p, dout, dz[l].p);
                dzl = dz[l].p;
            }
            const float* in = l == 0 ? x.p : h[l - 1].p;
            // dW (fi x fo) = in^T dz: A(i, b) = in[b][i], B(j, b) = dz[b][j]
            planes(pa, in, fi, B, 1, fi, 3, s);
            planes(pb, dzl, fo, B, 1, fo, 3, s);
            tc_gemm(pa.p, 3, pb.p, 3, fi, fo, B, nullptr, g.p + w_off[l], fo, false, err.p, s);
            colsum_kernel<<<(fo + 127) / 128, 128, 0, s>>>(B, fo, dzl, g.p + b_off[l]);
            if (l > 0) {
                // dh_{l-1} (B x fi) = dz W^T: A(b, j) = dz[b][j], B(i, j) = W[i][j]
                planes(pa, dzl, B, fo, fo, 1, 3, s);
                planes(pb, p.p + w_off[l], fi, fo, fo, 1, 3, s);
                tc_gemm(pa.p, 3, pb.p, 3, B, fi, fo, nullptr, dh[l - 1].p, fi, false, err.p, s);
                dout = dh[l - 1].p;
            }
        }
    }
    // XC_ERR_TIMEOUT (and a cleared flag) when a tensor-core wait gave up.
    void check_error(cudaStream_t s) {
        int e = 0;
        CGB_CUDA(cudaMemcpyAsync(&e, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
        CGB_CUDA(cudaStreamSynchronize(s));
        if (e) {
            CGB_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), s));
            throw Error(e, "MLP tensor-core GEMM: a pipeline wait timed out");
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
        h->m.wt_valid = false;
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
        m.check_error(h->s);
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
        m.check_error(h->s);
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
        m.wt_valid = false;
        m.check_error(h->s);
        std::vector<float> parts(nb);
        CGB_CUDA(cudaMemcpy(parts.data(), m.loss_part.p, nb * sizeof(float), cudaMemcpyDeviceToHost));
        double l = 0;
        for (float x : parts) l += x;
        *loss = (float)l;
    });
}

}  // extern "C"
