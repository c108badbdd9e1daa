// Tensor-core GEMM of the learned guess's network (the pair MLP of
// k_mlp.cu): C (M x N, FP32) = A (M x K) B (N x K)^T [+ bias] [+ C], on
// tcgen05.mma kind::f16 with FP32 accumulators in TMEM.
//
// Operands arrive as BF16 planes, K-major: plane p of A is [Mpad][Kpad]
// (rows of K contiguous), of B [Npad][Kpad]; tc_to_planes makes them from
// FP32 matrices in any orientation (it also transposes and zero-pads).  With
// three planes (x = h + m + l, exact for an FP32 x) the product sums the
// cross terms of order <= 2 -- FP32-level training; inference takes the
// weights as one BF16 plane against three activation planes (BF16 weights,
// FP32 activations).  The leading product accumulates apart from the
// corrections (two TMEM accumulators), as in the XC kernels.
//
// One CTA per 128 x 128 tile of C, 128 threads: thread 0 issues the TMA
// loads (two stages, 128-byte swizzle, one 128 x 64 box per plane), thread 32
// the MMAs, and all four warps drain TMEM (warp w: rows 32w..32w+31) into C.
// Every wait is bounded; a timeout records XC_ERR_TIMEOUT and unwinds.
#include "common.h"
#include "mixed.h"
#include "tc.cuh"

namespace cgb {
namespace {

using bf16 = __nv_bfloat16;
constexpr int kTile = 128, kKStep = 64;
constexpr uint32_t kPlane = kTile * kKStep * 2;  // one 128 x 64 BF16 box, 16 KB

__global__ void to_planes_kernel(const float* __restrict__ src, int rows, int kdim, long ld_r, long ld_k, int nplanes,
                                 int rows_pad, int k_pad, bf16* __restrict__ dst) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long n = (long)rows_pad * k_pad;
    if (i >= n) return;
    const int r = (int)(i / k_pad), k = (int)(i - (long)r * k_pad);
    const float v = (r < rows && k < kdim) ? src[(long)r * ld_r + (long)k * ld_k] : 0.f;
    if (nplanes == 1) {
        dst[i] = __float2bfloat16_rn(v);
    } else {
        bf16 h, m, l;
        tc::split3f(v, h, m, l);
        dst[i] = h;
        dst[n + i] = m;
        dst[2 * n + i] = l;
    }
}

template <int NPA, int NPB>
__global__ void __launch_bounds__(128, 1) tc_gemm_kernel(const __grid_constant__ CUtensorMap ta,
                                                         const __grid_constant__ CUtensorMap tb, int Mpad, int Npad,
                                                         int Kpad, int M, int N, const float* __restrict__ bias,
                                                         float* __restrict__ C, int ldc, int accumulate, int* err) {
    constexpr uint32_t kStage = (NPA + NPB) * kPlane;
    constexpr bool kCorr = NPA > 1 || NPB > 1;
    constexpr uint32_t kCols = kCorr ? 256 : 128;  // hh | corrections
    extern __shared__ uint8_t smem_raw[];
    __shared__ uint64_t full[2], empty[2], done;
    __shared__ uint32_t tmem_slot;
    __shared__ int abort_flag;
    uint8_t* smem = smem_raw + (((tc::smem_u32(smem_raw) + 1023u) & ~1023u) - tc::smem_u32(smem_raw));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.y * kTile, n0 = blockIdx.x * kTile;
    if (threadIdx.x == 0) {
        for (int s = 0; s < 2; s++) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        tc::mbar_init(&done, 1);
        abort_flag = 0;
        tc::fence_mbar_init();
    }
    if (warp == 0) tc::tmem_alloc(&tmem_slot, kCols);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_slot;
    const int nk = Kpad / kKStep;
    if (threadIdx.x == 0) {  // TMA producer
        for (int kc = 0; kc < nk; kc++) {
            const int s = kc & 1;
            if (abort_flag || !tc::mbar_wait(&empty[s], ((kc >> 1) & 1) ^ 1)) {
                atomicExch(err, XC_ERR_TIMEOUT);
                atomicExch(&abort_flag, 1);
                break;
            }
            uint8_t* st = smem + (size_t)s * kStage;
            tc::mbar_arrive_expect_tx(&full[s], kStage);
            for (int p = 0; p < NPA; p++) tc::tma_load_2d(st + p * kPlane, &ta, kc * kKStep, p * Mpad + m0, &full[s]);
            for (int p = 0; p < NPB; p++)
                tc::tma_load_2d(st + (NPA + p) * kPlane, &tb, kc * kKStep, p * Npad + n0, &full[s]);
        }
    } else if (threadIdx.x == 32) {  // MMA issuer
        constexpr uint32_t idesc = tc::idesc_bf16(kTile, kTile);
        bool started_corr = false;
        for (int kc = 0; kc < nk; kc++) {
            const int s = kc & 1;
            if (abort_flag || !tc::mbar_wait(&full[s], (kc >> 1) & 1)) {
                atomicExch(err, XC_ERR_TIMEOUT);
                atomicExch(&abort_flag, 1);
                break;
            }
            tc::fence_after_sync();
            const uint32_t a0 = tc::smem_u32(smem + (size_t)s * kStage), b0 = a0 + NPA * kPlane;
#pragma unroll
            for (int i = 0; i < NPA; i++)
#pragma unroll
                for (int j = 0; j < NPB; j++) {
                    if (i + j > 2) continue;
                    const bool lead = i == 0 && j == 0;
                    const uint32_t d = tmem + (lead ? 0u : 128u);
                    const uint64_t ad = tc::smem_desc_sw128(a0 + i * kPlane), bd = tc::smem_desc_sw128(b0 + j * kPlane);
#pragma unroll
                    for (int k = 0; k < kKStep / 16; k++) {
                        const bool fresh = k == 0 && (lead ? kc == 0 : !started_corr);
                        tc::mma_bf16(d, ad + 2 * k, bd + 2 * k, idesc, fresh ? 0u : 1u);
                    }
                    if (!lead) started_corr = true;
                }
            tc::mma_commit(&empty[s]);
        }
        tc::mma_commit(&done);
    }
    __syncwarp();
    // epilogue: all warps, row = this thread's TMEM lane
    bool ok = !abort_flag && tc::mbar_wait(&done, 0);
    ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;  // one decision per warp (collective TMEM loads)
    if (!ok) {
        if (lane == 0) atomicExch(err, XC_ERR_TIMEOUT);
    } else {
        tc::fence_after_sync();
        const int row = warp * 32 + lane, m = m0 + row;
        const uint32_t base = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
        for (int c16 = 0; c16 < kTile / 16; c16++) {
            float a[16], b[16];
            if (kCorr) {
                tc::tmem_ld16x2_nomem(base + c16 * 16, base + 128 + c16 * 16, a, b);
            } else {
                tc::tmem_ld16_nomem(base + c16 * 16, a);
#pragma unroll
                for (int j = 0; j < 16; j++) b[j] = 0.f;
            }
            if (m < M) {
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    const int n = n0 + c16 * 16 + j;
                    if (n < N) {
                        float v = a[j] + b[j];
                        if (bias) v += bias[n];
                        float* c = C + (size_t)m * ldc + n;
                        *c = accumulate ? *c + v : v;
                    }
                }
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, kCols);
}

template <int NPA, int NPB>
void launch_gemm(const CUtensorMap& ta, const CUtensorMap& tb, int Mpad, int Npad, int Kpad, int M, int N,
                 const float* bias, float* C, int ldc, bool acc, int* err, cudaStream_t s) {
    const size_t smem = 2 * (NPA + NPB) * kPlane + 1024;
    static bool attr = false;
    if (!attr) {
        CGB_CUDA(cudaFuncSetAttribute(tc_gemm_kernel<NPA, NPB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
        attr = true;
    }
    dim3 grid(Npad / kTile, Mpad / kTile);
    tc_gemm_kernel<NPA, NPB><<<grid, 128, smem, s>>>(ta, tb, Mpad, Npad, Kpad, M, N, bias, C, ldc, acc ? 1 : 0, err);
    CGB_CUDA(cudaGetLastError());
}

}  // namespace

int tc_pad_rows(int n) { return (n + kTile - 1) / kTile * kTile; }
int tc_pad_k(int n) { return (n + kKStep - 1) / kKStep * kKStep; }

void tc_to_planes(const float* src, int rows, int kdim, long ld_r, long ld_k, int nplanes, __nv_bfloat16* dst,
                  cudaStream_t s) {
    CGB_CHECK(nplanes == 1 || nplanes == 3, XC_ERR_INTERNAL, "1 or 3 planes");
    const int rp = tc_pad_rows(rows), kp = tc_pad_k(kdim);
    const long n = (long)rp * kp;
    to_planes_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(src, rows, kdim, ld_r, ld_k, nplanes, rp, kp, dst);
    CGB_CUDA(cudaGetLastError());
}

void tc_gemm(const __nv_bfloat16* A, int npa, const __nv_bfloat16* B, int npb, int M, int N, int K, const float* bias,
             float* C, int ldc, bool accumulate, int* err, cudaStream_t s) {
    const int Mpad = tc_pad_rows(M), Npad = tc_pad_rows(N), Kpad = tc_pad_k(K);
    CUtensorMap ta, tb;
    make_tmap_bf16(&ta, A, Kpad, (uint64_t)npa * Mpad, kKStep, kTile);
    make_tmap_bf16(&tb, B, Kpad, (uint64_t)npb * Npad, kKStep, kTile);
    if (npa == 3 && npb == 3) launch_gemm<3, 3>(ta, tb, Mpad, Npad, Kpad, M, N, bias, C, ldc, accumulate, err, s);
    else if (npa == 3 && npb == 1) launch_gemm<3, 1>(ta, tb, Mpad, Npad, Kpad, M, N, bias, C, ldc, accumulate, err, s);
    else if (npa == 1 && npb == 1) launch_gemm<1, 1>(ta, tb, Mpad, Npad, Kpad, M, N, bias, C, ldc, accumulate, err, s);
    else throw Error(XC_ERR_INTERNAL, "unsupported plane counts");
}

}  // namespace cgb
