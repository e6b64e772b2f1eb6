// Internal declarations of the surrogate network kernels (mlp.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace clode {
namespace mlp {

constexpr int kWidth = 256;  // hidden width
constexpr int kIn = 2;       // inputs

typedef __nv_bfloat16 bf16;

void linear_relu(const bf16 *X, int M, const bf16 *Wt, const float *b, bf16 *Y, int *err, int sms, cudaStream_t s);
void linear_heads(const bf16 *X, int M, const bf16 *Wt, const float *b, float *Y, int n_out, int *err, int sms,
                  cudaStream_t s);
void linear_back_hidden(const bf16 *dZ, int M, const bf16 *Wk, const bf16 *mask, bf16 *dX, int *err, int sms,
                        cudaStream_t s);
void linear_back_heads(const bf16 *dZ, int M, const bf16 *Wk, const bf16 *mask, bf16 *dX, int n_out, int *err,
                       int sms, cudaStream_t s);
void input_layer(const float *x, int M, const float *W1, const float *b1, bf16 *h1, cudaStream_t s);
void mse(const float *out, const float *y, int M, int H, int K, bf16 *dz, float *loss, cudaStream_t s);
void weight_grad_bf16(const bf16 *A, int Kd, const bf16 *D, int N, int M, float *G, float *g, cudaStream_t s);
void weight_grad_f32(const float *A, int Kd, const bf16 *D, int N, int M, float *G, float *g, cudaStream_t s);
void adam(float *w, const float *grad, float *m1, float *m2, int rows, int cols, float lr, const int *step,
          bf16 *wt, bf16 *wk, cudaStream_t s);
void step_increment(int *step, cudaStream_t s);
void gather_batch(const float *xs, const float *ys, int n_rows, int K, int B, int *cursor, float *xb, float *yb,
                  cudaStream_t s);
void cursor_increment(int *cursor, cudaStream_t s);
void head_stats(const float *out, long long M, int H, int K, float *mean, float *spread, cudaStream_t s);
void screen_grid(const float *mean, const float *spread, int nx, int ny, int K, const float *spread_thr,
                 const float *jump_thr, int *flags, cudaStream_t s);

}  // namespace mlp
}  // namespace clode
