// Internal declarations of the surrogate network kernels (mlp.cu).
//
// Every BF16 matrix the tensor cores read (activations, back-propagated
// gradients, weight copies) is stored in core-matrix order: element (r, c)
// of an R x W matrix sits at tiled_offset(r, c, W).  Rows come in groups of
// 8, each group is W / 8 core matrices of 8 rows x 16 bytes, so a block of
// 128 rows is one contiguous 128 * W * 2-byte tile that a single bulk copy
// puts into shared memory in the layout the MMA descriptors describe.
// Buffers hold whole 128-row tiles (rows rounded up).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstddef>

namespace clode {
namespace mlp {

constexpr int kWidth = 256;  // hidden width
constexpr int kIn = 2;       // inputs
constexpr int kTileM = 128;  // rows per tensor-core tile

typedef __nv_bfloat16 bf16;

__host__ __device__ inline size_t tiled_offset(long long r, int c, int W)
{
    return (size_t)(r >> 3) * (size_t)(W * 8) + (size_t)((c >> 3) * 64) + (size_t)((r & 7) * 8) + (size_t)(c & 7);
}

__host__ __device__ inline long long tiled_rows(long long rows) { return (rows + kTileM - 1) / kTileM * kTileM; }

// BF16 copies of one weight matrix W [K_in x N_out] (row-major FP32 master):
// fwd image: rows N_out, width K_in (operand B of Y = X W);
// bwd image: rows K_in, width N_out (operand B of dX = dZ W^T)
struct WeightImages {
    size_t offset;  // of W in the parameter vector
    int k_in, n_out;
    bf16 *fwd, *bwd;
};

void linear_relu(const bf16 *X, int M, const bf16 *Wfwd, const float *b, bf16 *Y, int *err, int sms, cudaStream_t s);
void linear_heads(const bf16 *X, int M, const bf16 *Wfwd, const float *b, float *Y, int n_out, int *err, int sms,
                  cudaStream_t s);
// dX = (dZ W^T) * (mask > 0)   (ReLU layers)
void linear_back_relu(const bf16 *dZ, int M, const bf16 *Wbwd, const bf16 *mask, bf16 *dX, int *err, int sms,
                      cudaStream_t s);
// dX = (dZ W^T) * mask        (the sine layer: mask = cos of its pre-activation)
void linear_back_mul(const bf16 *dZ, int M, const bf16 *Wbwd, const bf16 *mask, bf16 *dX, int *err, int sms,
                     cudaStream_t s);
void linear_back_heads(const bf16 *dZ, int M, const bf16 *Wbwd, const bf16 *mask, bf16 *dX, int n_out, int *err,
                       int sms, cudaStream_t s);
// h1 = sin(x W1 + b1), c1 = cos(x W1 + b1)  (tiled BF16, width 256)
void input_layer(const float *x, int M, const float *W1, const float *b1, bf16 *h1, bf16 *c1, cudaStream_t s);
void mse(const float *out, const float *y, int M, int H, int K, bf16 *dz, float *loss, cudaStream_t s);
// G += A^T D, g += column sums of D on the tensor cores (A: tiled BF16 width
// 256, D: tiled BF16 width N in {16, 32, 64, 256}, zero rows past M; G, g
// 16-byte aligned, zeroed by the caller)
void weight_grad(const bf16 *A, const bf16 *D, int N, int M, float *G, float *g, int *err, cudaStream_t s);
// G1 += x^T D, g1 += column sums of D  (x FP32 [M x 2], D tiled BF16 width 256)
void weight_grad_input(const float *x, const bf16 *D, int M, float *G, float *g, cudaStream_t s);
void adam_all(float *w, const float *grad, float *m1, float *m2, size_t n, float lr, const int *step,
              const WeightImages *img, int n_img, int *cursor, const float *loss, float *loss_hist, int *hist_index,
              cudaStream_t s);
void write_images(const float *w, const WeightImages *img, int n_img, cudaStream_t s);
void gather_batch(const float *xs, const float *ys, int n_rows, int K, int B, const int *cursor, float *xb, float *yb,
                  int *step, float *loss, cudaStream_t s);
void head_stats(const float *out, long long M, int H, int K, float *mean, float *spread, cudaStream_t s,
                const float *scale = nullptr, const float *offset = nullptr, float *scaled = nullptr);
void grid_inputs(int nx, int ny, long long r0, int rows, float *xb, cudaStream_t s);
void screen_grid(const float *mean, const float *spread, int nx, int ny, int K, const float *spread_thr,
                 const float *jump_thr, int *flags, cudaStream_t s);

}  // namespace mlp
}  // namespace clode
