// Kernels of the learned surrogate: a multilayer perceptron
//   x (2) -> 256 -> 256 -> 256 -> H heads x K outputs,  ReLU hidden layers,
// trained on feature maps computed by the ensemble engine, used to screen
// large parameter grids.
//
// The 256-wide layers and the heads run on the 5th-generation tensor cores:
// tcgen05.mma (kind::f16, BF16 operands, FP32 accumulation in tensor memory),
// one 128-row tile of activations per MMA group, the layer's weights resident
// in shared memory for the whole persistent CTA, the accumulator read back
// with tcgen05.ld for a fused epilogue (bias + ReLU, or the ReLU-derivative
// mask in the backward pass).  Operand tiles are written to shared memory in
// the canonical K-major, non-swizzled core-matrix layout (8 rows x 16 bytes
// per core matrix; LBO = 128 B between core matrices along K, SBO = K * 16 B
// between 8-row groups) that the shared-memory matrix descriptors describe.
// Weight-gradient reductions over the batch (X^T dZ), the 2-wide input layer,
// the loss and Adam are small and run on the CUDA cores.
//
// Every wait on an mbarrier is bounded: one thread polls with an iteration
// limit, publishes the outcome through shared memory, and on a timeout the
// CTA records an error flag, skips its remaining tiles, frees its tensor
// memory and returns.
#include "common.hpp"
#include "mlp.hpp"

#include <cuda_bf16.h>

namespace clode {
namespace mlp {

typedef __nv_bfloat16 bf16;

// ------------------------------------------------------------------ PTX --
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0u;
}

__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// D[tmem] (+)= A[smem] * B[smem]^T, M x N x 16, BF16 in, FP32 accumulate
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.u32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 32 lanes x 16 columns of FP32: this thread's row, columns [col, col+16)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 16; ++k)
        v[k] = __uint_as_float(r[k]);
}

// shared-memory matrix descriptor: K-major, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1u << 46;  // descriptor version of the 5th-generation tensor core
    return d;                 // base offset 0, absolute LBO mode 0, layout type 0 (no swizzle)
}

// instruction descriptor, kind::f16: D FP32, A and B BF16, both K-major
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// byte offset of element (r, k) of a K-wide K-major tile in core-matrix layout
__device__ __forceinline__ uint32_t cm_offset(int r, int k, int K)
{
    return (uint32_t)((r >> 3) * (K * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// ------------------------------------------------------- tensor-core layer --
// Y[m, n] = epilogue( sum_k X[m, k] * B[n, k] + bias[n] ),  m < M, n < N
//   X: BF16 [M x K] row-major, B: BF16 [N x K] row-major (K-major operand)
//   EPI_RELU_BF16:  Y = max(. + bias, 0)  -> BF16 [M x N]
//   EPI_BIAS_F32:   Y = . + bias          -> FP32 [M x N]
//   EPI_MASK_BF16:  Y = . * (mask[m, n] > 0) -> BF16 [M x N]  (no bias)
enum { EPI_RELU_BF16 = 0, EPI_BIAS_F32 = 1, EPI_MASK_BF16 = 2 };

constexpr int kTileM = 128;
constexpr long kSpinLimit = 1L << 26;

template <int K, int N, int EPI>
__global__ void __launch_bounds__(128, 1) k_linear_tc(const bf16 *__restrict__ X, int M, const bf16 *__restrict__ B,
                                                       const float *__restrict__ bias,
                                                       const bf16 *__restrict__ mask, void *__restrict__ Y,
                                                       int *__restrict__ err)
{
    static_assert(K % 16 == 0 && N % 16 == 0 && N >= 16 && N <= 256, "tile shape");
    constexpr uint32_t kCols = N <= 32 ? 32 : (N <= 64 ? 64 : (N <= 128 ? 128 : 256));
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *sA = smem;                         // kTileM x K bf16
    unsigned char *sB = smem + kTileM * K * 2;        // N x K bf16
    uint64_t *bar = (uint64_t *)(sB + N * K * 2);
    uint32_t *tslot = (uint32_t *)(bar + 1);
    volatile int *sflag = (volatile int *)(tslot + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (warp == 0)
        tmem_alloc(tslot, kCols);
    if (tid == 0) {
        mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *sflag = 0;
    }
    // weights: resident for the whole CTA
    for (int idx = tid; idx < N * (K / 8); idx += blockDim.x) {
        int r = idx / (K / 8), c = idx % (K / 8);
        uint4 v = *(const uint4 *)(B + (size_t)r * K + c * 8);
        *(uint4 *)(sB + cm_offset(r, c * 8, K)) = v;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    const uint32_t idesc = idesc_bf16(kTileM, N);
    uint32_t parity = 0;
    bool failed = false;

    for (int tile = blockIdx.x; tile * kTileM < M && !failed; tile += gridDim.x) {
        const int row0 = tile * kTileM;
        for (int idx = tid; idx < kTileM * (K / 8); idx += blockDim.x) {
            int r = idx / (K / 8), c = idx % (K / 8);
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (row0 + r < M)
                v = *(const uint4 *)(X + (size_t)(row0 + r) * K + c * 8);
            *(uint4 *)(sA + cm_offset(r, c * 8, K)) = v;
        }
        fence_async_smem();  // generic-proxy stores -> visible to the tensor core
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
            const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
#pragma unroll
            for (int s = 0; s < K / 16; ++s)
                mma_bf16(tmem, smem_desc(a0 + s * 256, 128, K * 16), smem_desc(b0 + s * 256, 128, K * 16), idesc,
                         s > 0 ? 1u : 0u);
            mma_commit(bar);
            bool done = false;
            for (long it = 0; it < kSpinLimit && !done; ++it)
                done = mbar_test(bar, parity);
            *sflag = done ? 0 : 1;
        }
        __syncthreads();
        if (*sflag) {
            failed = true;
            if (tid == 0 && err)
                atomicExch(err, 1);
            break;
        }
        parity ^= 1u;
        tc_fence_after();
        const int m = row0 + warp * 32 + lane;
        const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
        for (int c0 = 0; c0 < N; c0 += 16) {
            float v[16];
            tmem_ld16(trow + (uint32_t)c0, v);
            if (m < M) {
                if (EPI == EPI_BIAS_F32) {
                    float *y = (float *)Y + (size_t)m * N + c0;
#pragma unroll
                    for (int k = 0; k < 16; k += 4) {
                        float4 o = make_float4(v[k] + bias[c0 + k], v[k + 1] + bias[c0 + k + 1],
                                               v[k + 2] + bias[c0 + k + 2], v[k + 3] + bias[c0 + k + 3]);
                        *(float4 *)(y + k) = o;
                    }
                } else {
                    __align__(16) bf16 o[16];
                    if (EPI == EPI_RELU_BF16) {
#pragma unroll
                        for (int k = 0; k < 16; ++k)
                            o[k] = __float2bfloat16_rn(fmaxf(v[k] + bias[c0 + k], 0.0f));
                    } else {
                        const bf16 *mk = mask + (size_t)m * N + c0;
#pragma unroll
                        for (int k = 0; k < 16; ++k)
                            o[k] = __float2bfloat16_rn(__bfloat162float(mk[k]) > 0.0f ? v[k] : 0.0f);
                    }
                    bf16 *y = (bf16 *)Y + (size_t)m * N + c0;
                    *(uint4 *)y = *(const uint4 *)&o[0];
                    *(uint4 *)(y + 8) = *(const uint4 *)&o[8];
                }
            }
        }
        tc_fence_before();
        __syncthreads();  // every warp has read its accumulators before the next tile's MMA
        tc_fence_after();
    }
    if (failed && tid == 0) {
        // the MMA group never signalled: give it one more bounded chance to
        // finish before its tensor memory is released
        for (long it = 0; it < kSpinLimit; ++it)
            if (mbar_test(bar, parity))
                break;
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        tmem_dealloc(tmem, kCols);
}

template <int K, int N, int EPI>
size_t linear_smem_bytes()
{
    return (size_t)kTileM * K * 2 + (size_t)N * K * 2 + 64;
}

template <int K, int N, int EPI>
void launch_linear(const bf16 *X, int M, const bf16 *B, const float *bias, const bf16 *mask, void *Y, int *err,
                   int sms, cudaStream_t s)
{
    if (M <= 0)
        return;
    size_t smem = linear_smem_bytes<K, N, EPI>();
    check_cuda(cudaFuncSetAttribute(k_linear_tc<K, N, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
               "tensor-core layer shared memory");
    int tiles = (M + kTileM - 1) / kTileM;
    int grid = tiles < sms ? tiles : sms;
    k_linear_tc<K, N, EPI><<<grid, 128, smem, s>>>(X, M, B, bias, mask, Y, err);
    count_launch();
    check_cuda(cudaGetLastError(), "tensor-core layer launch");
}

// ---------------------------------------------------------- CUDA-core parts --
// input layer: h1 = relu(x W1 + b1), x FP32 [M x 2], W1 FP32 [2 x 256]
__global__ void k_input_layer(const float *__restrict__ x, int M, const float *__restrict__ W1,
                              const float *__restrict__ b1, bf16 *__restrict__ h1)
{
    size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    size_t total = (size_t)M * kWidth;
    for (; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
        size_t m = idx / kWidth;
        int n = (int)(idx % kWidth);
        float z = x[2 * m] * W1[n] + x[2 * m + 1] * W1[kWidth + n] + b1[n];
        h1[idx] = __float2bfloat16_rn(fmaxf(z, 0.0f));
    }
}

// loss: heads predict the same K targets; out FP32 [M x H*K], y FP32 [M x K]
// dz = 2 (out - y) / (M * H * K) as BF16, loss accumulates the mean square error
__global__ void k_mse(const float *__restrict__ out, const float *__restrict__ y, int M, int H, int K,
                      bf16 *__restrict__ dz, float *__restrict__ loss)
{
    const int HK = H * K;
    size_t total = (size_t)M * HK;
    float local = 0.0f;
    const float scale = 2.0f / (float)total;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        size_t m = idx / HK;
        int k = (int)(idx % HK) % K;
        float d = out[idx] - y[m * K + k];
        local += d * d;
        dz[idx] = __float2bfloat16_rn(scale * d);
    }
    for (int off = 16; off > 0; off >>= 1)
        local += __shfl_down_sync(0xffffffffu, local, off);
    if ((threadIdx.x & 31) == 0)
        atomicAdd(loss, local / (float)total);
}

__device__ __forceinline__ float to_f(float v) { return v; }
__device__ __forceinline__ float to_f(bf16 v) { return __bfloat162float(v); }

// weight gradient: G[k, n] = sum_m A[m, k] * D[m, n]  (A BF16 or FP32 [M x Kd], D BF16 [M x N]),
// bias gradient g[n] = sum_m D[m, n];  one 16 x 16 output tile per block
template <typename TA>
__global__ void k_weight_grad(const TA *__restrict__ A, int Kd, const bf16 *__restrict__ D, int N, int M,
                              float *__restrict__ G, float *__restrict__ g)
{
    __shared__ float sa[64][17];
    __shared__ float sd[64][17];
    const int k0 = blockIdx.x * 16, n0 = blockIdx.y * 16;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;  // 256 threads: (k, n) = (ty, tx)
    float acc = 0.0f, bacc = 0.0f;
    for (int m0 = 0; m0 < M; m0 += 64) {
        for (int i = threadIdx.x; i < 64 * 16; i += 256) {
            int mm = i / 16, c = i % 16;
            int m = m0 + mm;
            float av = 0.0f, dv = 0.0f;
            if (m < M) {
                if (k0 + c < Kd)
                    av = to_f(A[(size_t)m * Kd + k0 + c]);
                if (n0 + c < N)
                    dv = __bfloat162float(D[(size_t)m * N + n0 + c]);
            }
            sa[mm][c] = av;
            sd[mm][c] = dv;
        }
        __syncthreads();
#pragma unroll 8
        for (int mm = 0; mm < 64; ++mm) {
            acc += sa[mm][ty] * sd[mm][tx];
            bacc += sd[mm][tx];
        }
        __syncthreads();
    }
    if (k0 + ty < Kd && n0 + tx < N)
        G[(size_t)(k0 + ty) * N + n0 + tx] = acc;
    if (g && blockIdx.x == 0 && ty == 0 && n0 + tx < N)
        g[n0 + tx] = bacc;
}

// Adam on FP32 master weights; refreshes the BF16 copies the tensor cores read:
// wt[n, k] = w[k, n] (forward operand) and wk[k, n] = w[k, n] (backward operand)
__global__ void k_adam(float *__restrict__ w, const float *__restrict__ grad, float *__restrict__ m1,
                       float *__restrict__ m2, int rows, int cols, float lr, float b1, float b2, float eps,
                       const int *__restrict__ step, bf16 *__restrict__ wt, bf16 *__restrict__ wk)
{
    const int t = *step;
    const float c1 = 1.0f - powf(b1, (float)t), c2 = 1.0f - powf(b2, (float)t);
    size_t total = (size_t)rows * cols;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        float gr = grad[idx];
        float a = b1 * m1[idx] + (1.0f - b1) * gr;
        float b = b2 * m2[idx] + (1.0f - b2) * gr * gr;
        m1[idx] = a;
        m2[idx] = b;
        float v = w[idx] - lr * (a / c1) / (sqrtf(b / c2) + eps);
        w[idx] = v;
        int r = (int)(idx / cols), c = (int)(idx % cols);
        if (wt)
            wt[(size_t)c * rows + r] = __float2bfloat16_rn(v);
        if (wk)
            wk[idx] = __float2bfloat16_rn(v);
    }
}

__global__ void k_step_increment(int *step) { *step += 1; }

// rows [cursor*B, cursor*B + B) of the epoch's shuffled data into the batch buffers
__global__ void k_gather_batch(const float *__restrict__ xs, const float *__restrict__ ys, int n_rows, int K,
                               int B, int *__restrict__ cursor, float *__restrict__ xb, float *__restrict__ yb)
{
    const int c = *cursor;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B; i += gridDim.x * blockDim.x) {
        int r = (int)(((long long)c * B + i) % n_rows);
        xb[2 * i] = xs[2 * r];
        xb[2 * i + 1] = xs[2 * r + 1];
        for (int k = 0; k < K; ++k)
            yb[(size_t)i * K + k] = ys[(size_t)r * K + k];
    }
}

__global__ void k_cursor_increment(int *cursor) { *cursor += 1; }

// head statistics: mean and standard deviation over the H heads
__global__ void k_head_stats(const float *__restrict__ out, long long M, int H, int K, float *__restrict__ mean,
                             float *__restrict__ spread)
{
    const long long total = M * K;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        long long m = idx / K;
        int k = (int)(idx % K);
        float s = 0.0f, s2 = 0.0f;
        for (int h = 0; h < H; ++h) {
            float v = out[m * H * K + h * K + k];
            s += v;
            s2 += v * v;
        }
        float mu = s / H;
        mean[idx] = mu;
        spread[idx] = sqrtf(fmaxf(s2 / H - mu * mu, 0.0f));
    }
}

// Screening on an nx x ny grid (member m = iy * nx + ix): flag a point when
// the heads disagree (spread above its threshold) or when a feature jumps to
// one of its 4 neighbours by more than its threshold (a discontinuity of the
// feature map near which the network is not trusted).
__global__ void k_screen(const float *__restrict__ mean, const float *__restrict__ spread, int nx, int ny, int K,
                         const float *__restrict__ spread_thr, const float *__restrict__ jump_thr,
                         int *__restrict__ flags)
{
    const long long total = (long long)nx * ny;
    for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < total;
         m += (long long)gridDim.x * blockDim.x) {
        int ix = (int)(m % nx), iy = (int)(m / nx);
        int f = 0;
        for (int k = 0; k < K; ++k) {
            float v = mean[m * K + k];
            if (spread[m * K + k] > spread_thr[k])
                f |= 1;
            float j = 0.0f;
            if (ix > 0) j = fmaxf(j, fabsf(v - mean[(m - 1) * K + k]));
            if (ix + 1 < nx) j = fmaxf(j, fabsf(v - mean[(m + 1) * K + k]));
            if (iy > 0) j = fmaxf(j, fabsf(v - mean[(m - nx) * K + k]));
            if (iy + 1 < ny) j = fmaxf(j, fabsf(v - mean[(m + nx) * K + k]));
            if (j > jump_thr[k])
                f |= 2;
        }
        flags[m] = f;
    }
}

// ---------------------------------------------------------------- launchers --
namespace {
constexpr int kThreads = 256;
unsigned int grid_for(size_t n)
{
    size_t b = (n + kThreads - 1) / kThreads;
    return (unsigned int)(b < 1 ? 1 : (b > 8192 ? 8192 : b));
}
void after_launch(const char *what)
{
    count_launch();
    check_cuda(cudaGetLastError(), what);
}
}  // namespace

void linear_relu(const bf16 *X, int M, const bf16 *Wt, const float *b, bf16 *Y, int *err, int sms, cudaStream_t s)
{
    launch_linear<kWidth, kWidth, EPI_RELU_BF16>(X, M, Wt, b, nullptr, Y, err, sms, s);
}

void linear_heads(const bf16 *X, int M, const bf16 *Wt, const float *b, float *Y, int n_out, int *err, int sms,
                  cudaStream_t s)
{
    if (n_out == 16)
        launch_linear<kWidth, 16, EPI_BIAS_F32>(X, M, Wt, b, nullptr, Y, err, sms, s);
    else if (n_out == 32)
        launch_linear<kWidth, 32, EPI_BIAS_F32>(X, M, Wt, b, nullptr, Y, err, sms, s);
    else if (n_out == 64)
        launch_linear<kWidth, 64, EPI_BIAS_F32>(X, M, Wt, b, nullptr, Y, err, sms, s);
    else
        fail(CLODE_ERR_INVALID_ARGUMENT, "heads x outputs must be 16, 32 or 64 (got %d)", n_out);
}

void linear_back_hidden(const bf16 *dZ, int M, const bf16 *Wk, const bf16 *mask, bf16 *dX, int *err, int sms,
                        cudaStream_t s)
{
    launch_linear<kWidth, kWidth, EPI_MASK_BF16>(dZ, M, Wk, nullptr, mask, dX, err, sms, s);
}

void linear_back_heads(const bf16 *dZ, int M, const bf16 *Wk, const bf16 *mask, bf16 *dX, int n_out, int *err,
                       int sms, cudaStream_t s)
{
    if (n_out == 16)
        launch_linear<16, kWidth, EPI_MASK_BF16>(dZ, M, Wk, nullptr, mask, dX, err, sms, s);
    else if (n_out == 32)
        launch_linear<32, kWidth, EPI_MASK_BF16>(dZ, M, Wk, nullptr, mask, dX, err, sms, s);
    else if (n_out == 64)
        launch_linear<64, kWidth, EPI_MASK_BF16>(dZ, M, Wk, nullptr, mask, dX, err, sms, s);
    else
        fail(CLODE_ERR_INVALID_ARGUMENT, "heads x outputs must be 16, 32 or 64 (got %d)", n_out);
}

void input_layer(const float *x, int M, const float *W1, const float *b1, bf16 *h1, cudaStream_t s)
{
    k_input_layer<<<grid_for((size_t)M * kWidth), kThreads, 0, s>>>(x, M, W1, b1, h1);
    after_launch("input layer launch");
}

void mse(const float *out, const float *y, int M, int H, int K, bf16 *dz, float *loss, cudaStream_t s)
{
    k_mse<<<grid_for((size_t)M * H * K), kThreads, 0, s>>>(out, y, M, H, K, dz, loss);
    after_launch("loss launch");
}

void weight_grad_bf16(const bf16 *A, int Kd, const bf16 *D, int N, int M, float *G, float *g, cudaStream_t s)
{
    dim3 grid((Kd + 15) / 16, (N + 15) / 16);
    k_weight_grad<bf16><<<grid, 256, 0, s>>>(A, Kd, D, N, M, G, g);
    after_launch("weight gradient launch");
}

void weight_grad_f32(const float *A, int Kd, const bf16 *D, int N, int M, float *G, float *g, cudaStream_t s)
{
    dim3 grid((Kd + 15) / 16, (N + 15) / 16);
    k_weight_grad<float><<<grid, 256, 0, s>>>(A, Kd, D, N, M, G, g);
    after_launch("weight gradient launch");
}

void adam(float *w, const float *grad, float *m1, float *m2, int rows, int cols, float lr, const int *step,
          bf16 *wt, bf16 *wk, cudaStream_t s)
{
    k_adam<<<grid_for((size_t)rows * cols), kThreads, 0, s>>>(w, grad, m1, m2, rows, cols, lr, 0.9f, 0.999f, 1e-8f,
                                                              step, wt, wk);
    after_launch("Adam launch");
}

void step_increment(int *step, cudaStream_t s)
{
    k_step_increment<<<1, 1, 0, s>>>(step);
    after_launch("step counter launch");
}

void gather_batch(const float *xs, const float *ys, int n_rows, int K, int B, int *cursor, float *xb, float *yb,
                  cudaStream_t s)
{
    k_gather_batch<<<grid_for((size_t)B), kThreads, 0, s>>>(xs, ys, n_rows, K, B, cursor, xb, yb);
    after_launch("batch gather launch");
}

void cursor_increment(int *cursor, cudaStream_t s)
{
    k_cursor_increment<<<1, 1, 0, s>>>(cursor);
    after_launch("cursor launch");
}

void head_stats(const float *out, long long M, int H, int K, float *mean, float *spread, cudaStream_t s)
{
    k_head_stats<<<grid_for((size_t)M * K), kThreads, 0, s>>>(out, M, H, K, mean, spread);
    after_launch("head statistics launch");
}

void screen_grid(const float *mean, const float *spread, int nx, int ny, int K, const float *spread_thr,
                 const float *jump_thr, int *flags, cudaStream_t s)
{
    k_screen<<<grid_for((size_t)nx * ny), kThreads, 0, s>>>(mean, spread, nx, ny, K, spread_thr, jump_thr, flags);
    after_launch("screening launch");
}

}  // namespace mlp
}  // namespace clode
