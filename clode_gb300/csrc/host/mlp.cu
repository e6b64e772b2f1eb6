// Kernels of the learned surrogate: a multilayer perceptron
//   x (2) -> 256 (sine) -> 256 (ReLU) -> 256 (ReLU) -> H heads x K outputs,
// trained on feature maps computed by the ensemble engine, used to screen
// large parameter grids.  The sine first layer (a learned Fourier
// encoding of the two parameters) lets the network resolve the sharp but
// smooth ridges of a feature map that a ReLU first layer blurs.
//
// The 256-wide layers and the heads run on the 5th-generation tensor cores:
// tcgen05.mma (kind::f16, BF16 operands, FP32 accumulation in tensor memory),
// one 128-row tile of activations per MMA group, the layer's weights resident
// in shared memory for the whole persistent CTA, the accumulator read back
// with tcgen05.ld for a fused epilogue (bias + ReLU, or the derivative of the
// activation in the backward pass).  All BF16 operands live in global memory
// in core-matrix order (mlp.hpp), so the weights and each 128-row activation
// tile arrive in shared memory by one bulk asynchronous copy each
// (cp.async.bulk, completion on an mbarrier), and the next tile's copy is
// issued as soon as the MMA group has consumed the current one.  Weight
// gradients (X^T dZ, a reduction over the batch) run on the tensor cores too,
// reading the same tiles as MN-major operands.  The 2-wide input layer, its
// gradient, the loss and Adam are small and run on the CUDA cores.
//
// Every wait on an mbarrier is bounded: one thread polls with an iteration
// limit, publishes the outcome through shared memory, and on a timeout the
// CTA records an error flag, skips its remaining tiles, gives the operation
// in flight a second bounded wait, frees its tensor memory and returns.
#include "common.hpp"
#include "mlp.hpp"

#include <cuda_bf16.h>

namespace clode {
namespace mlp {

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

constexpr long kSpinLimit = 1L << 26;

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity)
{
    for (long it = 0; it < kSpinLimit; ++it)
        if (mbar_test(bar, parity))
            return true;
    return false;
}

// arrive on the barrier and expect `bytes` of asynchronous copies in this phase
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// global -> shared bulk copy (16-byte aligned addresses, size a multiple of 16)
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    constexpr uint32_t kChunk = 32768;
    const char *s = (const char *)src;
    char *d = (char *)dst;
    for (uint32_t off = 0; off < bytes; off += kChunk) {
        uint32_t n = bytes - off < kChunk ? bytes - off : kChunk;
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                smem_u32(d + off)),
            "l"(__cvta_generic_to_global(s + off)), "r"(n), "r"(smem_u32(bar))
            : "memory");
    }
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

// ------------------------------------------------------- tensor-core layer --
// Y[m, n] = epilogue( sum_k X[m, k] * B[n, k] + bias[n] ),  m < M, n < N
//   X: BF16 [M x K] core-matrix order (whole 128-row tiles), B: BF16 [N x K] core-matrix order
//   EPI_RELU_BF16:  Y = max(. + bias, 0)        -> BF16 [M x N] core-matrix order
//   EPI_BIAS_F32:   Y = . + bias                -> FP32 [M x N] row-major
//   EPI_MASK_BF16:  Y = . * (mask[m, n] > 0)    -> BF16 core-matrix order (no bias)
//   EPI_MUL_BF16:   Y = . * mask[m, n]          -> BF16 core-matrix order (no bias)
enum { EPI_RELU_BF16 = 0, EPI_BIAS_F32 = 1, EPI_MASK_BF16 = 2, EPI_MUL_BF16 = 3 };

// The N output columns are split in N / NS slices of NS columns; CTA c owns
// slice c % (N / NS) (its NS x K weight rows stay in shared memory) and
// walks the row tiles c / (N / NS), + gridDim.x / (N / NS), ...
template <int K, int N, int EPI, int NS>
__global__ void __launch_bounds__(128, 1) k_linear_tc(const bf16 *__restrict__ X, int M, const bf16 *__restrict__ B,
                                                       const float *__restrict__ bias,
                                                       const bf16 *__restrict__ mask, void *__restrict__ Y,
                                                       int *__restrict__ err)
{
    static_assert(K % 16 == 0 && N % NS == 0 && NS % 16 == 0 && NS >= 16 && NS <= 256, "tile shape");
    constexpr int kSlices = N / NS;
    constexpr uint32_t kCols = NS <= 32 ? 32 : (NS <= 64 ? 64 : (NS <= 128 ? 128 : 256));
    constexpr uint32_t kABytes = kTileM * K * 2, kBBytes = NS * K * 2;
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *sA = smem;             // kTileM x K bf16, core-matrix order
    unsigned char *sB = smem + kABytes;   // N x K bf16, core-matrix order
    uint64_t *bar_ld = (uint64_t *)(sB + kBBytes);
    uint64_t *bar_mma = bar_ld + 1;
    uint32_t *tslot = (uint32_t *)(bar_mma + 1);
    volatile int *sflag = (volatile int *)(tslot + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tiles = (M + kTileM - 1) / kTileM;
    const int slice = blockIdx.x % kSlices, col0 = slice * NS;
    const int tile_step = gridDim.x / kSlices;
    int tile = blockIdx.x / kSlices;
    if (warp == 0)
        tmem_alloc(tslot, kCols);
    if (tid == 0) {
        mbar_init(bar_ld, 1);
        mbar_init(bar_mma, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *sflag = 0;
        if (tile < tiles) {  // the weight slice and the first tile arrive on the first phase
            mbar_expect_tx(bar_ld, kBBytes + kABytes);
            bulk_g2s(sB, B + (size_t)col0 * K, kBBytes, bar_ld);
            bulk_g2s(sA, X + (size_t)tile * kTileM * K, kABytes, bar_ld);
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    const uint32_t idesc = idesc_bf16(kTileM, NS);
    uint32_t ph_ld = 0, ph_mma = 0;
    int pending = 0;  // thread 0: 1 = a copy may be in flight, 2 = an MMA group may be in flight
    bool failed = false;

    for (; tile < tiles; tile += tile_step) {
        const int row0 = tile * kTileM;
        if (tid == 0) {
            int st = 0;
            if (!mbar_wait_bounded(bar_ld, ph_ld)) {
                st = 1;
                pending = 1;
            } else {
                tc_fence_after();
                const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
#pragma unroll
                for (int s = 0; s < K / 16; ++s)
                    mma_bf16(tmem, smem_desc(a0 + s * 256, 128, K * 16), smem_desc(b0 + s * 256, 128, K * 16), idesc,
                             s > 0 ? 1u : 0u);
                mma_commit(bar_mma);
                if (!mbar_wait_bounded(bar_mma, ph_mma)) {
                    st = 2;
                    pending = 2;
                } else {
                    // the MMA group has consumed sA: fetch the next tile behind the epilogue
                    const int next = tile + tile_step;
                    if (next < tiles) {
                        mbar_expect_tx(bar_ld, kABytes);
                        bulk_g2s(sA, X + (size_t)next * kTileM * K, kABytes, bar_ld);
                    }
                }
            }
            *sflag = st;
        }
        ph_ld ^= 1u;
        ph_mma ^= 1u;
        __syncthreads();
        if (*sflag) {
            failed = true;
            if (tid == 0 && err)
                atomicExch(err, 1);
            break;
        }
        tc_fence_after();
        const int m = row0 + warp * 32 + lane;
        const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
        for (int c = 0; c < NS; c += 16) {
            const int c0 = col0 + c;  // column in the full output
            float v[16];
            tmem_ld16(trow + (uint32_t)c, v);
            if (m >= M && EPI != EPI_BIAS_F32) {
                // rows past M in the last tile are zero, so that batch
                // reductions over whole tiles see nothing there
                bf16 *y = (bf16 *)Y;
                *(uint4 *)(y + tiled_offset(m, c0, N)) = make_uint4(0u, 0u, 0u, 0u);
                *(uint4 *)(y + tiled_offset(m, c0 + 8, N)) = make_uint4(0u, 0u, 0u, 0u);
            } else if (m < M) {
                if (EPI == EPI_BIAS_F32) {
                    float *y = (float *)Y + (size_t)m * N + c0;
#pragma unroll
                    for (int k = 0; k < 16; k += 4) {
                        float4 o = make_float4(v[k] + bias[c0 + k], v[k + 1] + bias[c0 + k + 1],
                                               v[k + 2] + bias[c0 + k + 2], v[k + 3] + bias[c0 + k + 3]);
                        *(float4 *)(y + k) = o;
                    }
                } else {
                    const size_t o0 = tiled_offset(m, c0, N), o1 = tiled_offset(m, c0 + 8, N);
                    __align__(16) bf16 o[16];
                    if (EPI == EPI_RELU_BF16) {
#pragma unroll
                        for (int k = 0; k < 16; ++k)
                            o[k] = __float2bfloat16_rn(fmaxf(v[k] + bias[c0 + k], 0.0f));
                    } else {
                        __align__(16) bf16 mk[16];
                        *(uint4 *)&mk[0] = *(const uint4 *)(mask + o0);
                        *(uint4 *)&mk[8] = *(const uint4 *)(mask + o1);
#pragma unroll
                        for (int k = 0; k < 16; ++k) {
                            float g = __bfloat162float(mk[k]);
                            o[k] = __float2bfloat16_rn(EPI == EPI_MUL_BF16 ? v[k] * g : (g > 0.0f ? v[k] : 0.0f));
                        }
                    }
                    bf16 *y = (bf16 *)Y;
                    *(uint4 *)(y + o0) = *(const uint4 *)&o[0];
                    *(uint4 *)(y + o1) = *(const uint4 *)&o[8];
                }
            }
        }
        tc_fence_before();
        __syncthreads();  // every warp has read its accumulators before the next tile's MMA
        tc_fence_after();
    }
    if (failed && tid == 0) {
        // the copy or MMA group never signalled: one more bounded chance to
        // finish before the shared and tensor memory are released
        if (pending == 1)
            mbar_wait_bounded(bar_ld, ph_ld ^ 1u);
        else if (pending == 2)
            mbar_wait_bounded(bar_mma, ph_mma ^ 1u);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        tmem_dealloc(tmem, kCols);
}

// NS: output columns per CTA
template <int K, int N, int EPI, int NS>
void launch_linear_ns(const bf16 *X, int M, const bf16 *B, const float *bias, const bf16 *mask, void *Y, int *err,
                      int sms, cudaStream_t s)
{
    constexpr int kSlices = N / NS;
    const size_t smem = (size_t)kTileM * K * 2 + (size_t)NS * K * 2 + 64;
    check_cuda(cudaFuncSetAttribute(k_linear_tc<K, N, EPI, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem),
               "tensor-core layer shared memory");
    const int tiles = (M + kTileM - 1) / kTileM;
    int per_slice = sms / kSlices;  // CTAs per column slice
    if (per_slice < 1)
        per_slice = 1;
    if (per_slice > tiles)
        per_slice = tiles;
    k_linear_tc<K, N, EPI, NS><<<per_slice * kSlices, 128, smem, s>>>(X, M, B, bias, mask, Y, err);
    count_launch();
    check_cuda(cudaGetLastError(), "tensor-core layer launch");
}

// Few row tiles (a training batch): the 256 output columns split over 4 CTAs
// per tile, so that the layer occupies 4x as many SMs.  Many row tiles (a
// grid prediction): one CTA per tile and all columns, so each activation tile
// is read once.
template <int K, int N, int EPI>
void launch_linear(const bf16 *X, int M, const bf16 *B, const float *bias, const bf16 *mask, void *Y, int *err,
                   int sms, cudaStream_t s)
{
    if (M <= 0)
        return;
    constexpr int kNarrow = N > 64 ? 64 : N;
    const int tiles = (M + kTileM - 1) / kTileM;
    if (kNarrow < N && tiles < sms)
        launch_linear_ns<K, N, EPI, kNarrow>(X, M, B, bias, mask, Y, err, sms, s);
    else
        launch_linear_ns<K, N, EPI, N>(X, M, B, bias, mask, Y, err, sms, s);
}

// ---------------------------------------------------------- CUDA-core parts --
// thread index -> (row m, 8-column chunk c8) of a W-wide core-matrix-order
// matrix such that a warp writes contiguous 16-byte pieces
__device__ __forceinline__ void chunk_coords(size_t idx, int W, long long &m, int &c8)
{
    const int chunks = W / 8;
    long long grp = (long long)(idx / (size_t)(chunks * 8));
    int rem = (int)(idx % (size_t)(chunks * 8));
    c8 = rem / 8;
    m = grp * 8 + (rem & 7);
}

// input layer: z = x W1 + b1 (x FP32 [M x 2], W1 FP32 [2 x 256]);
// h1 = sin z, c1 = cos z (BF16, core-matrix order)
__global__ void k_input_layer(const float *__restrict__ x, int M, const float *__restrict__ W1,
                              const float *__restrict__ b1, bf16 *__restrict__ h1, bf16 *__restrict__ c1)
{
    const size_t total = (size_t)tiled_rows(M) * (kWidth / 8);
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        long long m;
        int c8;
        chunk_coords(idx, kWidth, m, c8);
        const size_t o = tiled_offset(m, c8 * 8, kWidth);
        if (m >= M) {  // zero padding rows of the last tile
            *(uint4 *)(h1 + o) = make_uint4(0u, 0u, 0u, 0u);
            *(uint4 *)(c1 + o) = make_uint4(0u, 0u, 0u, 0u);
            continue;
        }
        const float x0 = x[2 * m], x1 = x[2 * m + 1];
        __align__(16) bf16 hs[8], hc[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int n = c8 * 8 + j;
            const float z = x0 * W1[n] + x1 * W1[kWidth + n] + b1[n];
            float sz, cz;
            sincosf(z, &sz, &cz);
            hs[j] = __float2bfloat16_rn(sz);
            hc[j] = __float2bfloat16_rn(cz);
        }
        *(uint4 *)(h1 + o) = *(const uint4 *)hs;
        *(uint4 *)(c1 + o) = *(const uint4 *)hc;
    }
}

// loss: heads predict the same K targets; out FP32 [M x H*K] row-major, y FP32 [M x K];
// dz = 2 (out - y) / (M * H * K) as BF16 (core-matrix order, width H*K);
// loss accumulates the mean square error
__global__ void k_mse(const float *__restrict__ out, const float *__restrict__ y, int M, int H, int K,
                      bf16 *__restrict__ dz, float *__restrict__ loss)
{
    const int HK = H * K;
    const size_t total = (size_t)tiled_rows(M) * (HK / 8);
    const float scale = 2.0f / ((float)M * (float)HK);
    float local = 0.0f;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        long long m;
        int c8;
        chunk_coords(idx, HK, m, c8);
        if (m >= M) {  // zero padding rows of the last tile
            *(uint4 *)(dz + tiled_offset(m, c8 * 8, HK)) = make_uint4(0u, 0u, 0u, 0u);
            continue;
        }
        __align__(16) bf16 o[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int c = c8 * 8 + j;
            const float d = out[(size_t)m * HK + c] - y[(size_t)m * K + c % K];
            local += d * d;
            o[j] = __float2bfloat16_rn(scale * d);
        }
        *(uint4 *)(dz + tiled_offset(m, c8 * 8, HK)) = *(const uint4 *)o;
    }
    for (int off = 16; off > 0; off >>= 1)
        local += __shfl_down_sync(0xffffffffu, local, off);
    if ((threadIdx.x & 31) == 0)
        atomicAdd(loss, local / ((float)M * (float)HK));
}

// instruction descriptor with operand majors: a_mn / b_mn select MN-major A / B
__host__ __device__ constexpr uint32_t idesc_bf16_major(int M, int N, bool a_mn, bool b_mn)
{
    return idesc_bf16(M, N) | (a_mn ? (1u << 15) : 0u) | (b_mn ? (1u << 16) : 0u);
}

// A core-matrix-order tile (W wide, rows = the reduction) read as an MN-major
// operand: 8-row groups along K are W * 16 bytes apart (LBO), core matrices
// along MN 128 bytes apart (SBO)
__device__ __forceinline__ uint64_t smem_desc_mn(uint32_t addr, int W) { return smem_desc(addr, (uint32_t)W * 16u, 128u); }

// Weight gradient on the tensor cores:
//   G[k, n] += sum_m A[m, k] D[m, n]   (k in this CTA's half of A's 256 columns)
//   g[n]    += sum_m D[m, n]           (half 0; an MMA against an all-ones operand)
// A: BF16 [M x 256], D: BF16 [M x N], core-matrix order with zero rows past M.
// The batch is the reduction: each 128-row tile of A and D is read as an
// MN-major operand straight from its bulk copy, 8 K-steps of 16 rows,
// accumulating in tensor memory over this CTA's tiles; the sums are added
// into G and g with vector atomics.  Grid: 2 halves x batch splits.
template <int N>
__global__ void __launch_bounds__(128, 1) k_wgrad_tc(const bf16 *__restrict__ A, const bf16 *__restrict__ D, int M,
                                                      int tiles_per_cta, float *__restrict__ G, float *__restrict__ g,
                                                      int *__restrict__ err)
{
    static_assert(N % 16 == 0 && N >= 16 && N <= 256, "tile shape");
    constexpr int KD = kWidth;
    constexpr uint32_t kABytes = kTileM * KD * 2, kDBytes = kTileM * N * 2, kOnesBytes = kTileM * 16 * 2;
    constexpr uint32_t kCols = 2 * N <= 32 ? 32 : (2 * N <= 64 ? 64 : (2 * N <= 128 ? 128 : (2 * N <= 256 ? 256 : 512)));
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *sA = smem;
    unsigned char *sD = sA + kABytes;
    unsigned char *sOnes = sD + kDBytes;
    uint64_t *bar_ld = (uint64_t *)(sOnes + kOnesBytes);
    uint64_t *bar_mma = bar_ld + 1;
    uint32_t *tslot = (uint32_t *)(bar_mma + 1);
    volatile int *sflag = (volatile int *)(tslot + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int half = blockIdx.x & 1, split = blockIdx.x >> 1;
    const int tiles = (M + kTileM - 1) / kTileM;
    const int t_begin = split * tiles_per_cta;
    const int t_end = min(tiles, t_begin + tiles_per_cta);
    const bool with_bias = half == 0 && g != nullptr;
    for (int i = tid; i < (int)(kOnesBytes / 4); i += blockDim.x)
        ((uint32_t *)sOnes)[i] = 0x3F803F80u;  // BF16 1.0, 1.0
    if (warp == 0)
        tmem_alloc(tslot, kCols);
    if (tid == 0) {
        mbar_init(bar_ld, 1);
        mbar_init(bar_mma, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *sflag = 0;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the ones tile -> tensor core
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    const uint32_t id_main = idesc_bf16_major(kTileM, N, true, true);
    const uint32_t id_ones = idesc_bf16_major(kTileM, N, false, true);
    uint32_t ph_ld = 0, ph_mma = 0;
    int pending = 0;
    bool failed = false, any = false;

    for (int t = t_begin; t < t_end; ++t) {
        if (tid == 0) {
            int st = 0;
            mbar_expect_tx(bar_ld, kABytes + kDBytes);
            bulk_g2s(sA, A + (size_t)t * kTileM * KD, kABytes, bar_ld);
            bulk_g2s(sD, D + (size_t)t * kTileM * N, kDBytes, bar_ld);
            if (!mbar_wait_bounded(bar_ld, ph_ld)) {
                st = 1;
                pending = 1;
            } else {
                tc_fence_after();
                const uint32_t a0 = smem_u32(sA) + (uint32_t)half * 16u * 128u;  // 16 core matrices along MN
                const uint32_t d0 = smem_u32(sD), o0 = smem_u32(sOnes);
#pragma unroll
                for (int s = 0; s < kTileM / 16; ++s) {
                    const uint32_t acc = (t > t_begin || s > 0) ? 1u : 0u;
                    const uint64_t dd = smem_desc_mn(d0 + (uint32_t)s * 2u * N * 16u, N);
                    mma_bf16(tmem, smem_desc_mn(a0 + (uint32_t)s * 2u * KD * 16u, KD), dd, id_main, acc);
                    if (with_bias)
                        mma_bf16(tmem + (uint32_t)N, smem_desc(o0, 128, 256), dd, id_ones, acc);
                }
                mma_commit(bar_mma);
                if (!mbar_wait_bounded(bar_mma, ph_mma)) {
                    st = 2;
                    pending = 2;
                }
            }
            *sflag = st;
        }
        ph_ld ^= 1u;
        ph_mma ^= 1u;
        __syncthreads();
        if (*sflag) {
            failed = true;
            if (tid == 0 && err)
                atomicExch(err, 1);
            break;
        }
        any = true;
    }
    if (!failed && any) {
        tc_fence_after();
        const int k = half * 128 + warp * 32 + lane;
        const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
        for (int c0 = 0; c0 < N; c0 += 16) {
            float v[16];
            tmem_ld16(trow + (uint32_t)c0, v);
            float4 *dst = (float4 *)(G + (size_t)k * N + c0);
#pragma unroll
            for (int q = 0; q < 4; ++q)
                atomicAdd(dst + q, make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]));
        }
        if (with_bias && warp == 0) {  // every row of the second accumulator holds the column sums
#pragma unroll 1
            for (int c0 = 0; c0 < N; c0 += 16) {
                float v[16];
                tmem_ld16(trow + (uint32_t)(N + c0), v);
                if (lane == 0) {
                    float4 *dst = (float4 *)(g + c0);
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        atomicAdd(dst + q, make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]));
                }
            }
        }
    }
    if (failed && tid == 0) {
        if (pending == 1)
            mbar_wait_bounded(bar_ld, ph_ld ^ 1u);
        else if (pending == 2)
            mbar_wait_bounded(bar_mma, ph_mma ^ 1u);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        tmem_dealloc(tmem, kCols);
}

template <int N>
void launch_wgrad(const bf16 *A, const bf16 *D, int M, float *G, float *g, int *err, cudaStream_t s)
{
    if (M <= 0)
        return;
    const size_t smem = (size_t)kTileM * kWidth * 2 + (size_t)kTileM * N * 2 + (size_t)kTileM * 16 * 2 + 64;
    check_cuda(cudaFuncSetAttribute(k_wgrad_tc<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
               "weight-gradient shared memory");
    const int tiles = (M + kTileM - 1) / kTileM;
    const int per = (tiles + 31) / 32;
    const int splits = (tiles + per - 1) / per;
    k_wgrad_tc<N><<<2 * splits, 128, smem, s>>>(A, D, M, per, G, g, err);
    count_launch();
    check_cuda(cudaGetLastError(), "weight-gradient launch");
}

// input-layer gradient: G1[k, n] += sum_m x[m, k] D[m, n] (k < 2), g1[n] += sum_m D[m, n];
// one thread per column n, rows [blockIdx.x * rows_per_block, ...)
__global__ void __launch_bounds__(256) k_weight_grad_input(const float *__restrict__ x, const bf16 *__restrict__ D,
                                                           int M, int rows_per_block, float *__restrict__ G,
                                                           float *__restrict__ g)
{
    const int n = threadIdx.x;
    const int m_begin = blockIdx.x * rows_per_block;
    const int m_end = min(M, m_begin + rows_per_block);
    float a0 = 0.0f, a1 = 0.0f, ab = 0.0f;
#pragma unroll 8
    for (int m = m_begin; m < m_end; ++m) {
        const float d = __bfloat162float(D[tiled_offset(m, n, kWidth)]);
        a0 += x[2 * m] * d;
        a1 += x[2 * m + 1] * d;
        ab += d;
    }
    atomicAdd(&G[n], a0);
    atomicAdd(&G[kWidth + n], a1);
    atomicAdd(&g[n], ab);
}

// BF16 operand images of the tensor-core weights from the FP32 masters
struct ImageSet {
    WeightImages im[3];
    int n;
};

__device__ __forceinline__ void store_images(const ImageSet &set, size_t idx, float v)
{
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        if (q >= set.n)
            break;
        const WeightImages &w = set.im[q];
        const size_t size = (size_t)w.k_in * w.n_out;
        if (idx >= w.offset && idx < w.offset + size) {
            const int r = (int)((idx - w.offset) / w.n_out), c = (int)((idx - w.offset) % w.n_out);
            const bf16 b = __float2bfloat16_rn(v);
            w.fwd[tiled_offset(c, r, w.k_in)] = b;
            w.bwd[tiled_offset(r, c, w.n_out)] = b;
        }
    }
}

// Adam over the whole parameter vector; refreshes the BF16 images; thread 0
// also advances the batch cursor and appends the step's loss to the history
__global__ void k_adam_all(float *__restrict__ w, const float *__restrict__ grad, float *__restrict__ m1,
                           float *__restrict__ m2, size_t n, float lr, float b1, float b2, float eps,
                           const int *__restrict__ step, ImageSet set, int *__restrict__ cursor,
                           const float *__restrict__ loss, float *__restrict__ loss_hist, int *__restrict__ hist_index)
{
    const int t = *step;
    const float c1 = 1.0f - powf(b1, (float)t), c2 = 1.0f - powf(b2, (float)t);
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
        const float gr = grad[idx];
        const float a = b1 * m1[idx] + (1.0f - b1) * gr;
        const float b = b2 * m2[idx] + (1.0f - b2) * gr * gr;
        m1[idx] = a;
        m2[idx] = b;
        const float v = w[idx] - lr * (a / c1) / (sqrtf(b / c2) + eps);
        w[idx] = v;
        store_images(set, idx, v);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (cursor)
            *cursor += 1;
        if (loss_hist && hist_index) {
            loss_hist[*hist_index] = *loss;
            *hist_index += 1;
        }
    }
}

__global__ void k_write_images(const float *__restrict__ w, ImageSet set, size_t n)
{
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x)
        store_images(set, idx, w[idx]);
}

// rows [cursor*B, cursor*B + B) of the epoch's shuffled data into the batch
// buffers; thread 0 also advances the step counter and clears the loss
__global__ void k_gather_batch(const float *__restrict__ xs, const float *__restrict__ ys, int n_rows, int K,
                               int B, const int *__restrict__ cursor, float *__restrict__ xb, float *__restrict__ yb,
                               int *__restrict__ step, float *__restrict__ loss)
{
    const int c = *cursor;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B; i += gridDim.x * blockDim.x) {
        int r = (int)(((long long)c * B + i) % n_rows);
        xb[2 * i] = xs[2 * r];
        xb[2 * i + 1] = xs[2 * r + 1];
        for (int k = 0; k < K; ++k)
            yb[(size_t)i * K + k] = ys[(size_t)r * K + k];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *step += 1;
        *loss = 0.0f;
    }
}

// inputs of grid points [r0, r0 + rows) of an nx x ny grid (point iy * nx + ix),
// each coordinate mapped to [-1, 1]
__global__ void k_grid_inputs(int nx, int ny, long long r0, int rows, float *__restrict__ xb)
{
    const float sx = nx > 1 ? 2.0f / (float)(nx - 1) : 0.0f, sy = ny > 1 ? 2.0f / (float)(ny - 1) : 0.0f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += gridDim.x * blockDim.x) {
        const long long p = r0 + i;
        const int ix = (int)(p % nx), iy = (int)(p / nx);
        xb[2 * i] = nx > 1 ? (float)ix * sx - 1.0f : 0.0f;
        xb[2 * i + 1] = ny > 1 ? (float)iy * sy - 1.0f : 0.0f;
    }
}

// head statistics: mean and standard deviation over the H heads; when
// `scaled` is given it also receives mean * scale[k] + offset[k]
__global__ void k_head_stats(const float *__restrict__ out, long long M, int H, int K, float *__restrict__ mean,
                             float *__restrict__ spread, const float *__restrict__ scale,
                             const float *__restrict__ offset, float *__restrict__ scaled)
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
        if (scaled)
            scaled[idx] = mu * (scale ? scale[k] : 1.0f) + (offset ? offset[k] : 0.0f);
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
ImageSet image_set(const WeightImages *img, int n)
{
    if (n < 0 || n > 3)
        fail(CLODE_ERR_INTERNAL, "at most 3 weight images");
    ImageSet s{};
    for (int i = 0; i < n; ++i)
        s.im[i] = img[i];
    s.n = n;
    return s;
}
}  // namespace

void linear_relu(const bf16 *X, int M, const bf16 *Wfwd, const float *b, bf16 *Y, int *err, int sms, cudaStream_t s)
{
    launch_linear<kWidth, kWidth, EPI_RELU_BF16>(X, M, Wfwd, b, nullptr, Y, err, sms, s);
}

void linear_heads(const bf16 *X, int M, const bf16 *Wfwd, const float *b, float *Y, int n_out, int *err, int sms,
                  cudaStream_t s)
{
    if (n_out == 16)
        launch_linear<kWidth, 16, EPI_BIAS_F32>(X, M, Wfwd, b, nullptr, Y, err, sms, s);
    else if (n_out == 32)
        launch_linear<kWidth, 32, EPI_BIAS_F32>(X, M, Wfwd, b, nullptr, Y, err, sms, s);
    else if (n_out == 64)
        launch_linear<kWidth, 64, EPI_BIAS_F32>(X, M, Wfwd, b, nullptr, Y, err, sms, s);
    else
        fail(CLODE_ERR_INVALID_ARGUMENT, "heads x outputs must be 16, 32 or 64 (got %d)", n_out);
}

void linear_back_relu(const bf16 *dZ, int M, const bf16 *Wbwd, const bf16 *mask, bf16 *dX, int *err, int sms,
                      cudaStream_t s)
{
    launch_linear<kWidth, kWidth, EPI_MASK_BF16>(dZ, M, Wbwd, nullptr, mask, dX, err, sms, s);
}

void linear_back_mul(const bf16 *dZ, int M, const bf16 *Wbwd, const bf16 *mask, bf16 *dX, int *err, int sms,
                     cudaStream_t s)
{
    launch_linear<kWidth, kWidth, EPI_MUL_BF16>(dZ, M, Wbwd, nullptr, mask, dX, err, sms, s);
}

void linear_back_heads(const bf16 *dZ, int M, const bf16 *Wbwd, const bf16 *mask, bf16 *dX, int n_out, int *err,
                       int sms, cudaStream_t s)
{
    if (n_out == 16)
        launch_linear<16, kWidth, EPI_MASK_BF16>(dZ, M, Wbwd, nullptr, mask, dX, err, sms, s);
    else if (n_out == 32)
        launch_linear<32, kWidth, EPI_MASK_BF16>(dZ, M, Wbwd, nullptr, mask, dX, err, sms, s);
    else if (n_out == 64)
        launch_linear<64, kWidth, EPI_MASK_BF16>(dZ, M, Wbwd, nullptr, mask, dX, err, sms, s);
    else
        fail(CLODE_ERR_INVALID_ARGUMENT, "heads x outputs must be 16, 32 or 64 (got %d)", n_out);
}

void input_layer(const float *x, int M, const float *W1, const float *b1, bf16 *h1, bf16 *c1, cudaStream_t s)
{
    k_input_layer<<<grid_for((size_t)tiled_rows(M) * (kWidth / 8)), kThreads, 0, s>>>(x, M, W1, b1, h1, c1);
    after_launch("input layer launch");
}

void mse(const float *out, const float *y, int M, int H, int K, bf16 *dz, float *loss, cudaStream_t s)
{
    k_mse<<<grid_for((size_t)tiled_rows(M) * (H * K / 8)), kThreads, 0, s>>>(out, y, M, H, K, dz, loss);
    after_launch("loss launch");
}

namespace {
int rows_per_block_for(int M, int max_blocks)
{
    int r = (M + max_blocks - 1) / max_blocks;
    r = (r + 15) / 16 * 16;
    return r < 16 ? 16 : r;
}
}  // namespace

void weight_grad(const bf16 *A, const bf16 *D, int N, int M, float *G, float *g, int *err, cudaStream_t s)
{
    if (N == 256)
        launch_wgrad<256>(A, D, M, G, g, err, s);
    else if (N == 64)
        launch_wgrad<64>(A, D, M, G, g, err, s);
    else if (N == 32)
        launch_wgrad<32>(A, D, M, G, g, err, s);
    else if (N == 16)
        launch_wgrad<16>(A, D, M, G, g, err, s);
    else
        fail(CLODE_ERR_INVALID_ARGUMENT, "weight gradient: N must be 16, 32, 64 or 256 (got %d)", N);
}

void weight_grad_input(const float *x, const bf16 *D, int M, float *G, float *g, cudaStream_t s)
{
    if (M <= 0)
        return;
    const int rpb = rows_per_block_for(M, 256);
    k_weight_grad_input<<<(unsigned int)((M + rpb - 1) / rpb), kWidth, 0, s>>>(x, D, M, rpb, G, g);
    after_launch("input-layer gradient launch");
}

void adam_all(float *w, const float *grad, float *m1, float *m2, size_t n, float lr, const int *step,
              const WeightImages *img, int n_img, int *cursor, const float *loss, float *loss_hist, int *hist_index,
              cudaStream_t s)
{
    k_adam_all<<<grid_for(n), kThreads, 0, s>>>(w, grad, m1, m2, n, lr, 0.9f, 0.999f, 1e-8f, step,
                                                image_set(img, n_img), cursor, loss, loss_hist, hist_index);
    after_launch("Adam launch");
}

void write_images(const float *w, const WeightImages *img, int n_img, cudaStream_t s)
{
    size_t n = 0;
    for (int i = 0; i < n_img; ++i)
        n = n > img[i].offset + (size_t)img[i].k_in * img[i].n_out ? n : img[i].offset + (size_t)img[i].k_in * img[i].n_out;
    k_write_images<<<grid_for(n), kThreads, 0, s>>>(w, image_set(img, n_img), n);
    after_launch("weight image launch");
}

void gather_batch(const float *xs, const float *ys, int n_rows, int K, int B, const int *cursor, float *xb, float *yb,
                  int *step, float *loss, cudaStream_t s)
{
    k_gather_batch<<<grid_for((size_t)B), kThreads, 0, s>>>(xs, ys, n_rows, K, B, cursor, xb, yb, step, loss);
    after_launch("batch gather launch");
}

void head_stats(const float *out, long long M, int H, int K, float *mean, float *spread, cudaStream_t s,
                const float *scale, const float *offset, float *scaled)
{
    k_head_stats<<<grid_for((size_t)M * K), kThreads, 0, s>>>(out, M, H, K, mean, spread, scale, offset, scaled);
    after_launch("head statistics launch");
}

void grid_inputs(int nx, int ny, long long r0, int rows, float *xb, cudaStream_t s)
{
    k_grid_inputs<<<grid_for((size_t)rows), kThreads, 0, s>>>(nx, ny, r0, rows, xb);
    after_launch("grid inputs launch");
}

void screen_grid(const float *mean, const float *spread, int nx, int ny, int K, const float *spread_thr,
                 const float *jump_thr, int *flags, cudaStream_t s)
{
    k_screen<<<grid_for((size_t)nx * ny), kThreads, 0, s>>>(mean, spread, nx, ny, K, spread_thr, jump_thr, flags);
    after_launch("screening launch");
}

}  // namespace mlp
}  // namespace clode
