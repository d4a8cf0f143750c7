// learn.cu - kernels of the learned ring-down extrapolator (training and inference, sm_103a).
//
// The network (em_lab_gb300/extrap.py) is a 1-D convolutional encoder of the early port V(t), I(t)
// and a 4-layer MLP head; every layer is a GEMM with BF16 operands and FP32 accumulation:
//  * nn_gemm: C[M][N] = sum_k A(m, k) B(n, k) on the tcgen05 tensor cores (kind::f16 with BF16
//    operands, FP32 accumulator in tensor memory). A CTA of four warps owns a 128 x 128 tile of C;
//    for each 64-wide K chunk the threads stage A and B (strided loads: the same kernel serves the
//    forward product X W^T and the backward products dZ W and dZ^T X) into the no-swizzle K-major
//    core-matrix layout (8 rows x 16 bytes per core matrix, 128 B between core matrices along K,
//    1024 B between 8-row groups), one thread issues four MMAs of K 16 and commits them to an
//    mbarrier, and after the last chunk each warp reads its 32 accumulator lanes with tcgen05.ld.
//    Waits are bounded; on expiry the CTA records an error, frees its tensor memory and leaves.
//  * elementwise kernels: bias + ReLU with the BF16 copy for the next layer, ReLU backward, bias
//    gradients, im2col / col2im of the strided convolutions, the MSE loss gradient, Adam (FP32
//    master weights, BF16 copies for the GEMMs).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "../../include/emlab_nn.h"
#include "emlab_internal.h"

namespace emlab {
namespace {

constexpr int kTM = 128, kTN = 128, kTK = 64;
constexpr int kTileBytes = kTM * kTK * 2;  // 16 KB per operand tile
constexpr int kResidencyPad = 24 * 1024;

__device__ unsigned g_nn_err;  // nonzero: a bounded wait of nn_gemm expired

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t desc_kmajor(const void* p) {
    // start >> 4, LBO 128 B >> 4 at bit 16, SBO 1024 B >> 4 at bit 32, descriptor version 1 at bit 46
    const uint64_t a = saddr(p);
    return ((a & 0x3FFFFull) >> 4) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(1024 >> 4) << 32) | (1ull << 46);
}

// kind::f16 instruction descriptor: D FP32 (bits 4-5 = 1), A and B BF16 (bits 7-9, 10-12 = 1),
// both K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t bf16_idesc(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ bool wait_bounded(uint64_t* bar, uint32_t parity) {
    for (int i = 0; i < (1 << 20); ++i) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(saddr(bar)), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

// One row (of A or B) of a 64-wide K chunk into the K-major core-matrix layout: the row's eight
// 16-byte pieces go to (row / 8) * 1024 + piece * 128 + (row % 8) * 16. A row that is contiguous
// along K and 16-byte aligned (vec) is read as eight 16-byte pieces, all in flight together; any
// other stride, and the chunk that reaches past K, element by element.
__device__ __forceinline__ void stage_row(unsigned char* tile, int row, const __nv_bfloat16* src, long long s_k,
                                          bool live, int k0, int K, bool vec) {
    const __nv_bfloat16 zero = __float2bfloat16(0.0f);
    if (vec && k0 + kTK <= K) {
        uint4 piece[kTK / 8];
#pragma unroll
        for (int j = 0; j < kTK / 8; ++j)
            piece[j] = live ? __ldg(reinterpret_cast<const uint4*>(src + k0 + j * 8)) : make_uint4(0, 0, 0, 0);
#pragma unroll
        for (int j = 0; j < kTK / 8; ++j)
            *reinterpret_cast<uint4*>(tile + (row >> 3) * 1024 + j * 128 + (row & 7) * 16) = piece[j];
        return;
    }
#pragma unroll
    for (int j = 0; j < kTK / 8; ++j) {
        __align__(16) __nv_bfloat16 v[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int k = k0 + j * 8 + q;
            v[q] = (live && k < K) ? src[(long long)k * s_k] : zero;
        }
        *reinterpret_cast<uint4*>(tile + (row >> 3) * 1024 + j * 128 + (row & 7) * 16) = *reinterpret_cast<uint4*>(v);
    }
}

__global__ void __launch_bounds__(128) nn_gemm_kernel(int M, int N, int K, const __nv_bfloat16* A, long long sam,
                                                      long long sak, const __nv_bfloat16* B, long long sbn,
                                                      long long sbk, float* C, long long ldc) {
    __shared__ __align__(1024) unsigned char sa[kTileBytes];
    __shared__ __align__(1024) unsigned char sb[kTileBytes];
    __shared__ uint64_t bar;
    __shared__ uint32_t tslot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * kTM, n0 = blockIdx.y * kTN;
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(saddr(&bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(&tslot)), "r"(kTN)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tslot;
    constexpr uint32_t idesc = bf16_idesc(kTM, kTN);

    const int am = m0 + tid, bn = n0 + tid;  // the A row and the B row this thread stages
    const __nv_bfloat16* arow = A + (long long)min(am, M - 1) * sam;
    const __nv_bfloat16* brow = B + (long long)min(bn, N - 1) * sbn;
    const bool vec_a = sak == 1 && (sam % 8) == 0 && (reinterpret_cast<uintptr_t>(A) & 15) == 0;
    const bool vec_b = sbk == 1 && (sbn % 8) == 0 && (reinterpret_cast<uintptr_t>(B) & 15) == 0;
    uint32_t phase = 0;
    bool ok = true;
    const int chunks = (K + kTK - 1) / kTK;
    for (int c = 0; c < chunks && ok; ++c) {
        stage_row(sa, tid, arow, sak, am < M, c * kTK, K, vec_a);
        stage_row(sb, tid, brow, sbk, bn < N, c * kTK, K, vec_b);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // generic stores -> tensor-core reads
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
            for (int s = 0; s < kTK / 16; ++s) {
                const uint64_t ad = desc_kmajor(sa + s * 256), bd = desc_kmajor(sb + s * 256);
                const uint32_t acc = (c > 0 || s > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             saddr(&bar))
                         : "memory");
        }
        ok = wait_bounded(&bar, phase);  // the MMAs have read the tiles: they may be restaged
        phase ^= 1u;
        if (__syncthreads_or(!ok)) {
            ok = false;
            if (tid == 0) {
                atomicOr(&g_nn_err, 1u);
                wait_bounded(&bar, phase ^ 1u);  // give the MMAs in flight a bounded time to finish
            }
        }
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (ok && chunks > 0) {
        const int m = m0 + warp * 32 + lane;
        for (int j = 0; j < kTN / 32; ++j) {
            float d[32];
            tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(j * 32), d);
            if (m >= M) continue;
            float* crow = C + (long long)m * ldc;
            const int nb = n0 + j * 32;
            if (nb + 32 <= N && (ldc % 4) == 0 && (reinterpret_cast<uintptr_t>(C) & 15) == 0) {
#pragma unroll
                for (int q = 0; q < 32; q += 4)
                    *reinterpret_cast<float4*>(crow + nb + q) = make_float4(d[q], d[q + 1], d[q + 2], d[q + 3]);
                continue;
            }
#pragma unroll
            for (int q = 0; q < 32; ++q) {
                const int n = nb + q;
                if (n < N) crow[n] = d[q];
            }
        }
    } else if (chunks == 0) {
        const int m = m0 + warp * 32 + lane;
        if (m < M)
            for (int n = n0; n < min(N, n0 + kTN); ++n) C[(long long)m * ldc + n] = 0.0f;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTN) : "memory");
}

// z[m][n] = c[m][n] + bias[n % bias_n] (in place); a = relu ? max(z, 0) : z, as BF16 at
// out[m * ldo + off + n]. bias_n < N serves a convolution whose rows hold several positions.
__global__ void nn_bias_act_kernel(float* z, const float* bias, int M, int N, int bias_n, int relu,
                                   __nv_bfloat16* out, long long ldo, int off) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= (long long)M * N) return;
    const int m = (int)(i / N), n = (int)(i - (long long)m * N);
    const float v = z[i] + (bias ? bias[n % bias_n] : 0.0f);
    z[i] = v;
    if (out) out[(long long)m * ldo + off + n] = __float2bfloat16(relu && v < 0.0f ? 0.0f : v);
}

// dz = dy * (z > 0) (relu) or dy; BF16 copy for the GEMMs
__global__ void nn_act_grad_kernel(const float* dy, long long ldy, int off, const float* z, int M, int N, int relu,
                                   float* dz, __nv_bfloat16* dz_bf) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= (long long)M * N) return;
    const int m = (int)(i / N), n = (int)(i - (long long)m * N);
    float g = dy[(long long)m * ldy + off + n];
    if (relu && !(z[i] > 0.0f)) g = 0.0f;
    dz[i] = g;
    dz_bf[i] = __float2bfloat16(g);
}

// out[n] = sum_m d[m][n] (one thread per column, FP32 in row order)
__global__ void nn_col_sum_kernel(const float* d, int M, int N, float* out) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    float s = 0.0f;
    for (int m = 0; m < M; ++m) s += d[(long long)m * N + n];
    out[n] = s;
}

// x: [B][Lin][C] (position-major); cols: [B * Lout][k * C], column (j, c) = x[b][l * stride - pad + j][c]
__global__ void nn_im2col_kernel(const __nv_bfloat16* x, int B, int Lin, int Cc, int k, int stride, int pad,
                                 int Lout, __nv_bfloat16* cols) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long total = (long long)B * Lout * k * Cc;
    if (i >= total) return;
    const int c = (int)(i % Cc);
    const int j = (int)((i / Cc) % k);
    const long long bl = i / ((long long)Cc * k);
    const int l = (int)(bl % Lout), b = (int)(bl / Lout);
    const int p = l * stride - pad + j;
    cols[i] = (p >= 0 && p < Lin) ? x[((long long)b * Lin + p) * Cc + c] : __float2bfloat16(0.0f);
}

// dx[b][p][c] = sum over (l, j) with l * stride - pad + j = p of dcols[(b, l)][(j, c)] (FP32)
__global__ void nn_col2im_kernel(const float* dcols, int B, int Lin, int Cc, int k, int stride, int pad, int Lout,
                                 float* dx) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long total = (long long)B * Lin * Cc;
    if (i >= total) return;
    const int c = (int)(i % Cc);
    const int p = (int)((i / Cc) % Lin);
    const int b = (int)(i / ((long long)Cc * Lin));
    float s = 0.0f;
    for (int j = 0; j < k; ++j) {
        const int q = p + pad - j;
        if (q < 0 || q % stride) continue;
        const int l = q / stride;
        if (l >= Lout) continue;
        s += dcols[((long long)b * Lout + l) * ((long long)k * Cc) + (long long)j * Cc + c];
    }
    dx[i] = s;
}

// mean squared error over n values: dy = 2 (y - t) / n, loss += sum (y - t)^2 / n (per block, atomic)
__global__ void nn_mse_kernel(const float* y, const float* t, long long n, float* dy, float* loss) {
    __shared__ float red[256];
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    float e = 0.0f;
    if (i < n) {
        const float d = y[i] - t[i];
        dy[i] = 2.0f * d / (float)n;
        e = d * d / (float)n;
    }
    red[threadIdx.x] = e;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0 && loss) atomicAdd(loss, red[0]);
}

// Adam (FP32 master weights); the BF16 copy is refreshed for the next GEMMs
__global__ void nn_adam_kernel(float* w, float* m, float* v, const float* g, long long n, float lr, float b1, float b2,
                               float eps, float bc1, float bc2, __nv_bfloat16* w_bf) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi, v[i] = vi;
    const float wi = w[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    w[i] = wi;
    if (w_bf) w_bf[i] = __float2bfloat16(wi);
}

__global__ void nn_to_bf16_kernel(const float* x, long long n, __nv_bfloat16* out, long long ldo, int cols, int off) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const long long r = i / cols, c = i - r * cols;
    out[r * ldo + off + c] = __float2bfloat16(x[i]);
}

inline unsigned blocks(long long n, int t = 256) { return (unsigned)((n + t - 1) / t); }

}  // namespace
}  // namespace emlab

using namespace emlab;

#define NN_STREAM(s) reinterpret_cast<cudaStream_t>(s)
#define NN_CHECK()                                                                          \
    do {                                                                                    \
        const cudaError_t e_ = cudaGetLastError();                                          \
        if (e_ != cudaSuccess) return report_error(EMLAB_ERR_CUDA, cudaGetErrorString(e_)); \
    } while (0)

extern "C" {

int emlab_nn_gemm(int M, int N, int K, const void* A, long long sam, long long sak, const void* B, long long sbn,
                  long long sbk, float* C, long long ldc, void* stream) {
    if (M <= 0 || N <= 0 || K < 0 || !A || !B || !C) return report_error(EMLAB_ERR_INVALID, "bad GEMM arguments");
    const dim3 grid((M + kTM - 1) / kTM, (N + kTN - 1) / kTN);
    // 24 KB of unused dynamic shared memory holds residency to four CTAs per SM: 4 x 128 tensor-
    // memory columns = the SM's 512, so no CTA waits in tcgen05.alloc
    static const bool sized = cudaFuncSetAttribute(nn_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   kResidencyPad) == cudaSuccess;
    if (!sized) return report_error(EMLAB_ERR_CUDA, "GEMM shared-memory attribute");
    nn_gemm_kernel<<<grid, 128, kResidencyPad, NN_STREAM(stream)>>>(M, N, K, static_cast<const __nv_bfloat16*>(A), sam, sak,
                                                        static_cast<const __nv_bfloat16*>(B), sbn, sbk, C, ldc);
    count_launches(1);
    NN_CHECK();
    return EMLAB_OK;
}

int emlab_nn_status(void* stream) {
    unsigned err = 0;
    if (cudaStreamSynchronize(NN_STREAM(stream)) != cudaSuccess ||
        cudaMemcpyFromSymbol(&err, g_nn_err, 4) != cudaSuccess)
        return report_error(EMLAB_ERR_CUDA, "nn status read failed");
    if (err) {
        const unsigned zero = 0;
        cudaMemcpyToSymbol(g_nn_err, &zero, 4);
        return report_error(EMLAB_ERR_TIMEOUT, "a tensor-core GEMM gave up a bounded wait on the device");
    }
    return EMLAB_OK;
}

int emlab_nn_bias_act(float* z, const float* bias, int M, int N, int bias_n, int relu, void* out_bf16, long long ldo,
                      int off, void* stream) {
    if (bias_n <= 0) return report_error(EMLAB_ERR_INVALID, "bias length must be positive");
    nn_bias_act_kernel<<<blocks((long long)M * N), 256, 0, NN_STREAM(stream)>>>(
        z, bias, M, N, bias_n, relu, static_cast<__nv_bfloat16*>(out_bf16), ldo, off);
    count_launches(1);
    NN_CHECK();
    return EMLAB_OK;
}

int emlab_nn_act_grad(const float* dy, long long ldy, int off, const float* z, int M, int N, int relu, float* dz,
                      void* dz_bf16, void* stream) {
    nn_act_grad_kernel<<<blocks((long long)M * N), 256, 0, NN_STREAM(stream)>>>(
        dy, ldy, off, z, M, N, relu, dz, static_cast<__nv_bfloat16*>(dz_bf16));
    count_launches(1);
    NN_CHECK();
    return EMLAB_OK;
}

int emlab_nn_col_sum(const float* d, int M, int N, float* out, void* stream) {
    nn_col_sum_kernel<<<blocks(N, 128), 128, 0, NN_STREAM(stream)>>>(d, M, N, out);
    count_launches(1);
    NN_CHECK();
    return EMLAB_OK;
}

int emlab_nn_im2col(const void* x, int B, int Lin, int C, int k, int stride, int pad, int Lout, void* cols,
                    void* stream) {
    nn_im2col_kernel<<<blocks((long long)B * Lout * k * C), 256, 0, NN_STREAM(stream)>>>(
        static_cast<const __nv_bfloat16*>(x), B, Lin, C, k, stride, pad, Lout, static_cast<__nv_bfloat16*>(cols));
    count_launches(1);
    NN_CHECK();
    return EMLAB_OK;
}

int emlab_nn_col2im(const float* dcols, int B, int Lin, int C, int k, int stride, int pad, int Lout, float* dx,
                    void* stream) {
    nn_col2im_kernel<<<blocks((long long)B * Lin * C), 256, 0, NN_STREAM(stream)>>>(dcols, B, Lin, C, k, stride, pad,
                                                                                    Lout, dx);
    count_launches(1);
    NN_CHECK();
    return EMLAB_OK;
}

int emlab_nn_mse(const float* y, const float* t, long long n, float* dy, float* loss, void* stream) {
    nn_mse_kernel<<<blocks(n), 256, 0, NN_STREAM(stream)>>>(y, t, n, dy, loss);
    count_launches(1);
    NN_CHECK();
    return EMLAB_OK;
}

int emlab_nn_adam(float* w, float* m, float* v, const float* g, long long n, float lr, float b1, float b2, float eps,
                  int t, void* w_bf16, void* stream) {
    const float bc1 = 1.0f - powf(b1, (float)t), bc2 = 1.0f - powf(b2, (float)t);
    nn_adam_kernel<<<blocks(n), 256, 0, NN_STREAM(stream)>>>(w, m, v, g, n, lr, b1, b2, eps, bc1, bc2,
                                                             static_cast<__nv_bfloat16*>(w_bf16));
    count_launches(1);
    NN_CHECK();
    return EMLAB_OK;
}

int emlab_nn_to_bf16(const float* x, long long n, void* out, long long ldo, int cols, int off, void* stream) {
    nn_to_bf16_kernel<<<blocks(n), 256, 0, NN_STREAM(stream)>>>(x, n, static_cast<__nv_bfloat16*>(out), ldo, cols, off);
    count_launches(1);
    NN_CHECK();
    return EMLAB_OK;
}

}  // extern "C"
