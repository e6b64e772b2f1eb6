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

// Trajectory rows regrouped by member.  The trajectory kernel stores row r,
// column j of member i at [(r * width + j) * ld + i] (members fastest, so its
// stores coalesce); clODE's TrajectorySimulator.get_trajectory slices every
// member's rows out of that on the host (clode/trajectory.py:216-264).  This
// is the transpose of the (rows * width) x members matrix into member-major
// doubles, dst[(i - m0) * nc + c]: 32 x 32 tiles staged through shared
// memory, loads coalesced along members, stores along c, every element read
// once and written once.  Tiles are walked grid-stride so any number of rows
// fits one launch.
constexpr int kTile = 32, kTileRows = 8;

template <typename T>
__global__ void __launch_bounds__(kTile *kTileRows)
    k_regroup_by_member(const T *__restrict__ src, size_t ld, size_t m0, size_t nm, size_t nc,
                        double *__restrict__ dst)
{
    __shared__ double tile[kTile][kTile + 1];
    const size_t tiles_m = (nm + kTile - 1) / kTile;
    const size_t tiles = tiles_m * ((nc + kTile - 1) / kTile);
    for (size_t b = blockIdx.x; b < tiles; b += gridDim.x) {
        const size_t i0 = (b % tiles_m) * kTile, c0 = (b / tiles_m) * kTile;
        const size_t i = i0 + threadIdx.x;
        for (int k = threadIdx.y; k < kTile; k += kTileRows) {
            const size_t c = c0 + k;
            if (c < nc && i < nm)
                tile[k][threadIdx.x] = (double)src[c * ld + m0 + i];
        }
        __syncthreads();
        const size_t c = c0 + threadIdx.x;
        for (int k = threadIdx.y; k < kTile; k += kTileRows) {
            const size_t ii = i0 + k;
            if (c < nc && ii < nm)
                dst[ii * nc + c] = tile[threadIdx.x][k];
        }
        __syncthreads();
    }
}

template <typename T>
void launch_regroup(const T *src, size_t ld, size_t m0, size_t nm, size_t nc, double *dst, cudaStream_t s)
{
    if (!nm || !nc) return;
    const size_t tiles = ((nm + kTile - 1) / kTile) * ((nc + kTile - 1) / kTile);
    // 152 SMs x 8 resident 256-thread blocks; more tiles are walked grid-stride
    const unsigned int grid = (unsigned int)std::min<size_t>(tiles, 152 * 8);
    k_regroup_by_member<T><<<grid, dim3(kTile, kTileRows), 0, s>>>(src, ld, m0, nm, nc, dst);
    count_launch();
    check_cuda(cudaGetLastError(), "trajectory regroup launch");
}

}  // namespace

void launch_regroup_by_member_f32(const float *src, size_t ld, size_t m0, size_t nm, size_t nc, double *dst,
                                  cudaStream_t s)
{
    launch_regroup<float>(src, ld, m0, nm, nc, dst, s);
}

void launch_regroup_by_member_f64(const double *src, size_t ld, size_t m0, size_t nm, size_t nc, double *dst,
                                  cudaStream_t s)
{
    launch_regroup<double>(src, ld, m0, nm, nc, dst, s);
}

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
