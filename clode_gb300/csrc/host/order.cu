// Longest-time-span-first member order for the persistent kernels, built on
// the device: keys are the members' span lengths t1 - t0 (FP32 is enough to
// order them), values the member indices, sorted descending by CUB's radix
// sort (stable, so equal spans keep index order).
#include <cub/device/device_radix_sort.cuh>

#include "common.hpp"

namespace clode {
namespace {

template <typename T>
__global__ void k_span_keys(const T *__restrict__ tspan, size_t n, float *__restrict__ keys, int *__restrict__ idx)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        keys[i] = (float)(tspan[2 * i + 1] - tspan[2 * i]);
        idx[i] = (int)i;
    }
}

template <typename T>
void order_impl(const T *tspan, size_t n, int *order, void *scratch, size_t *scratch_bytes, cudaStream_t s)
{
    // scratch: keys in, keys out, indices in, then CUB's temporary storage
    const size_t keys_bytes = (n * sizeof(float) + 255) & ~(size_t)255;
    const size_t idx_bytes = (n * sizeof(int) + 255) & ~(size_t)255;
    size_t temp = 0;
    check_cuda(cub::DeviceRadixSort::SortPairsDescending(nullptr, temp, (const float *)nullptr, (float *)nullptr,
                                                        (const int *)nullptr, (int *)nullptr, (int)n, 0, 32, s),
               "member order sort size");
    const size_t need = 2 * keys_bytes + idx_bytes + temp;
    if (!scratch) {
        *scratch_bytes = need;
        return;
    }
    if (*scratch_bytes < need)
        fail(CLODE_ERR_INTERNAL, "member order scratch too small");
    unsigned char *p = (unsigned char *)scratch;
    float *keys_in = (float *)p, *keys_out = (float *)(p + keys_bytes);
    int *idx_in = (int *)(p + 2 * keys_bytes);
    void *tmp = p + 2 * keys_bytes + idx_bytes;
    const unsigned int grid = (unsigned int)std::min<size_t>((n + 255) / 256, 4864);
    k_span_keys<T><<<grid, 256, 0, s>>>(tspan, n, keys_in, idx_in);
    count_launch();
    check_cuda(cudaGetLastError(), "member order keys");
    // CUB's kernels are library work: not counted among this library's launches
    check_cuda(cub::DeviceRadixSort::SortPairsDescending(tmp, temp, keys_in, keys_out, idx_in, order, (int)n, 0, 32, s),
               "member order sort");
}

__global__ void k_iota(size_t n, int *__restrict__ idx)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        idx[i] = (int)i;
}

}  // namespace

// Members by decreasing count (non-negative ints, e.g. warm-up steps); the
// same scratch layout as the span order
void order_by_count(const int *counts, size_t n, int *order, void *scratch, size_t *scratch_bytes, cudaStream_t s)
{
    const size_t keys_bytes = (n * sizeof(unsigned int) + 255) & ~(size_t)255;
    const size_t idx_bytes = (n * sizeof(int) + 255) & ~(size_t)255;
    size_t temp = 0;
    check_cuda(cub::DeviceRadixSort::SortPairsDescending(nullptr, temp, (const unsigned int *)nullptr,
                                                        (unsigned int *)nullptr, (const int *)nullptr, (int *)nullptr,
                                                        (int)n, 0, 32, s),
               "member order sort size");
    const size_t need = keys_bytes + idx_bytes + temp;
    if (!scratch) {
        *scratch_bytes = need;
        return;
    }
    if (*scratch_bytes < need)
        fail(CLODE_ERR_INTERNAL, "member order scratch too small");
    unsigned char *p = (unsigned char *)scratch;
    unsigned int *keys_out = (unsigned int *)p;
    int *idx_in = (int *)(p + keys_bytes);
    void *tmp = p + keys_bytes + idx_bytes;
    const unsigned int grid = (unsigned int)std::min<size_t>((n + 255) / 256, 4864);
    k_iota<<<grid, 256, 0, s>>>(n, idx_in);
    count_launch();
    check_cuda(cudaGetLastError(), "member order indices");
    // CUB's kernels are library work: not counted among this library's launches
    check_cuda(cub::DeviceRadixSort::SortPairsDescending(tmp, temp, (const unsigned int *)counts, keys_out, idx_in,
                                                        order, (int)n, 0, 32, s),
               "member order sort");
}

void order_by_span_f32(const float *tspan, size_t n, int *order, void *scratch, size_t *scratch_bytes, cudaStream_t s)
{
    order_impl<float>(tspan, n, order, scratch, scratch_bytes, s);
}

void order_by_span_f64(const double *tspan, size_t n, int *order, void *scratch, size_t *scratch_bytes, cudaStream_t s)
{
    order_impl<double>(tspan, n, order, scratch, scratch_bytes, s);
}

}  // namespace clode
