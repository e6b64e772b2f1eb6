// Ahead-of-time kernels of the host runtime (compiled into the library for
// sm_103a): precision conversion of the SoA host<->device transfers, RNG
// seeding, and fills.  All are grid-stride
// loops over HBM-resident vectors; each moves its bytes once.
#include "common.hpp"

namespace clode {
namespace {

constexpr int kThreads = 256;

inline unsigned int grid_for(size_t n)
{
    // enough blocks to cover n once, capped at 148 * 32 blocks; grid-stride beyond
    size_t b = (n + kThreads - 1) / kThreads;
    if (b < 1)
        b = 1;
    if (b > 4864)
        b = 4864;
    return (unsigned int)b;
}

__global__ void k_f64_to_f32(const double *__restrict__ src, float *__restrict__ dst, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = (float)src[i];
}

__global__ void k_f32_to_f64(const float *__restrict__ src, double *__restrict__ dst, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = (double)src[i];
}

// CLODE::seedRNG(int): state word k = seed + k in int arithmetic, widened
// with sign extension to u64 (clode/cpp/CLODE.cpp:447-453)
__global__ void k_seed_sequential(unsigned long long *rng, size_t n, int seed)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        unsigned int v = (unsigned int)seed + (unsigned int)i;
        rng[i] = (unsigned long long)(long long)(int)v;
    }
}

// CLODE::seedRNG(): independent random 64-bit words; splitmix64 of a random base
__global__ void k_seed_random(unsigned long long *rng, size_t n, unsigned long long base)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        unsigned long long z = base + 0x9e3779b97f4a7c15ull * (i + 1);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        rng[i] = z ^ (z >> 31);
    }
}

template <typename T>
__global__ void k_fill(T *dst, T v, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = v;
}

}  // namespace

void launch_f64_to_f32(const double *src, float *dst, size_t n, cudaStream_t s)
{
    if (!n) return;
    k_f64_to_f32<<<grid_for(n), kThreads, 0, s>>>(src, dst, n);
    count_launch();
    check_cuda(cudaGetLastError(),"f64->f32 conversion launch");
}

void launch_f32_to_f64(const float *src, double *dst, size_t n, cudaStream_t s)
{
    if (!n) return;
    k_f32_to_f64<<<grid_for(n), kThreads, 0, s>>>(src, dst, n);
    count_launch();
    check_cuda(cudaGetLastError(),"f32->f64 conversion launch");
}

void launch_seed_rng_sequential(unsigned long long *rng, size_t n, int seed, cudaStream_t s)
{
    if (!n) return;
    k_seed_sequential<<<grid_for(n), kThreads, 0, s>>>(rng, n, seed);
    count_launch();
    check_cuda(cudaGetLastError(),"RNG seeding launch");
}

void launch_seed_rng_random(unsigned long long *rng, size_t n, unsigned long long base, cudaStream_t s)
{
    if (!n) return;
    k_seed_random<<<grid_for(n), kThreads, 0, s>>>(rng, n, base);
    count_launch();
    check_cuda(cudaGetLastError(),"RNG seeding launch");
}

void launch_fill_f32(float *dst, float v, size_t n, cudaStream_t s)
{
    if (!n) return;
    k_fill<float><<<grid_for(n), kThreads, 0, s>>>(dst, v, n);
    count_launch();
    check_cuda(cudaGetLastError(),"fill launch");
}

void launch_fill_f64(double *dst, double v, size_t n, cudaStream_t s)
{
    if (!n) return;
    k_fill<double><<<grid_for(n), kThreads, 0, s>>>(dst, v, n);
    count_launch();
    check_cuda(cudaGetLastError(),"fill launch");
}

void launch_fill_i32(int *dst, int v, size_t n, cudaStream_t s)
{
    if (!n) return;
    k_fill<int><<<grid_for(n), kThreads, 0, s>>>(dst, v, n);
    count_launch();
    check_cuda(cudaGetLastError(),"fill launch");
}

}  // namespace clode
