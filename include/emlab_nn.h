/* emlab_nn.h - kernels of the learned ring-down extrapolator (no reference counterpart: the
 * reference has no learned component; the learned antenna-sweep workload).
 *
 * Device pointers and sizes only; `stream` is a cudaStream_t (NULL = the legacy default stream).
 * BF16 operands are __nv_bfloat16 arrays, everything else FP32. Return EMLAB_OK or an error code
 * with emlab_last_error() set. */
#ifndef EMLAB_NN_H
#define EMLAB_NN_H

#ifdef __cplusplus
extern "C" {
#endif

/* C[m * ldc + n] = sum_k A(m, k) B(n, k), A(m, k) = A[m * sam + k * sak], B(n, k) = B[n * sbn + k * sbk]
 * (BF16), FP32 accumulation on the tensor cores (tcgen05, 128 x 128 tiles). */
int emlab_nn_gemm(int M, int N, int K, const void* A, long long sam, long long sak, const void* B, long long sbn,
                  long long sbk, float* C, long long ldc, void* stream);
/* Synchronises the stream; EMLAB_ERR_TIMEOUT if a GEMM gave up a bounded wait since the last call. */
int emlab_nn_status(void* stream);
/* z[m][n] += bias[n % bias_n] in place; out_bf16[m * ldo + off + n] = relu ? max(z, 0) : z (BF16). */
int emlab_nn_bias_act(float* z, const float* bias, int M, int N, int bias_n, int relu, void* out_bf16, long long ldo,
                      int off, void* stream);
/* dz = dy[m * ldy + off + n] * (relu ? z > 0 : 1), with a BF16 copy. */
int emlab_nn_act_grad(const float* dy, long long ldy, int off, const float* z, int M, int N, int relu, float* dz,
                      void* dz_bf16, void* stream);
/* out[n] = sum_m d[m][n]. */
int emlab_nn_col_sum(const float* d, int M, int N, float* out, void* stream);
/* x (B, Lin, C) BF16 -> cols (B * Lout, k * C): column (j, c) of row (b, l) = x[b][l * stride - pad + j][c]. */
int emlab_nn_im2col(const void* x, int B, int Lin, int C, int k, int stride, int pad, int Lout, void* cols,
                    void* stream);
/* The adjoint of emlab_nn_im2col on FP32: dx (B, Lin, C) from dcols (B * Lout, k * C). */
int emlab_nn_col2im(const float* dcols, int B, int Lin, int C, int k, int stride, int pad, int Lout, float* dx,
                    void* stream);
/* dy = 2 (y - t) / n; *loss += sum (y - t)^2 / n. */
int emlab_nn_mse(const float* y, const float* t, long long n, float* dy, float* loss, void* stream);
/* One Adam step at time t (>= 1) on n FP32 weights; w_bf16 (optional) receives their BF16 copy. */
int emlab_nn_adam(float* w, float* m, float* v, const float* g, long long n, float lr, float b1, float b2, float eps,
                  int t, void* w_bf16, void* stream);
/* out_bf16[r * ldo + off + c] = x[r * cols + c] for the n = rows * cols values. */
int emlab_nn_to_bf16(const float* x, long long n, void* out, long long ldo, int cols, int off, void* stream);

#ifdef __cplusplus
}
#endif
#endif
