// clode_sim_features_noalloc: a features run for callers that cannot
// allocate device memory.
//
// Some callers are not allowed to call cudaMalloc at run time: services
// whose device memory is carved up once at start-up and whose allocator
// refuses later requests, real-time pipelines that forbid allocation after
// initialisation because it can block on the driver, and plug-ins hosted by
// an application that owns every device allocation itself.  The regular
// features() path allocates its feature, state and scratch buffers on the
// device the first time it sees an ensemble size.  This entry point takes
// every input and output buffer from the caller and keeps its own scratch —
// the member work counter of the persistent schedule and the observer state
// parked at the end of each member — in one file-scope device array, so it
// calls no allocating routine at all.
//
// The array (kScratchBytes, 64 MiB) is created by the CUDA runtime when this
// library's device code is loaded on a GPU and stays there until the process
// exits, on every GPU that loads the library.
#include "common.hpp"
#include "../device/clode_args.h"

#include <cstring>
#include <mutex>
#include <type_traits>

namespace {

constexpr size_t kScratchBytes = 64ull << 20;
constexpr size_t kHeaderBytes = 256;  // work counter at offset 0, rest reserved
constexpr int kMaxDevices = 64;

// The shared scratch.  In host code this name is only a stand-in for the
// symbol, not a device address: its device address comes from
// cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

std::mutex g_mu;
void *g_scratch_addr[kMaxDevices] = {nullptr};

// Device address of g_scratch on `device`, which must be current; looked up
// once per device and remembered.  The remembered address belongs to the
// device's primary context (the one the CUDA runtime uses): it stays valid
// for the life of the process unless that context is destroyed
// (cudaDeviceReset), after which this entry point must not be called.
void *scratch_address(int device)
{
    std::lock_guard<std::mutex> lk(g_mu);
    if (device < 0 || device >= kMaxDevices)
        clode::fail(CLODE_ERR_NO_DEVICE, "device ordinal %d out of range", device);
    if (!g_scratch_addr[device]) {
        void *p = nullptr;
        clode::check_cuda(cudaGetSymbolAddress(&p, g_scratch), "cudaGetSymbolAddress(scratch)");
        g_scratch_addr[device] = p;
    }
    return g_scratch_addr[device];
}

template <typename A>
void launch_features(A &a, const clode::NoallocFeaturesLaunch &L, long long n_pts, const void *x0, const void *pars,
                     const void *tspan, unsigned long long *rng, void *dt, void *xf, void *tf, void *F, int *status,
                     unsigned char *base, dim3 grid, dim3 block, cudaStream_t s)
{
    using R = typename std::remove_reference<decltype(a.t0)>::type;
    a.nPts = (int)n_pts;
    a.i_begin = 0;
    a.i_end = (int)n_pts;
    a.i_stride = 1;
    a.fused_init = 1;
    a.tspan_pm = (const R *)tspan;
    a.x0 = (const R *)x0;
    a.pars = (const R *)pars;
    a.xf = (R *)xf;
    a.rng = rng;
    a.dt = (R *)dt;
    a.tf = (R *)tf;
    a.odata = (unsigned int *)(base + kHeaderBytes);
    a.F = (R *)F;
    a.status = status;
    a.stats = nullptr;
    a.work_next = (unsigned int *)base;
    a.time_budget_ns = 0ull;
    void *params[] = {&a};
    clode::check_cuda(cudaLaunchKernel(L.kernel, grid, block, params, 0, s), "features launch");
    clode::count_launch();
}

// Makes `device` current for the lifetime of the guard and gives the
// calling thread its previous current device back on every exit path.
struct CurrentDevice {
    int saved = -1;
    explicit CurrentDevice(int device)
    {
        clode::check_cuda(cudaGetDevice(&saved), "cudaGetDevice");
        if (saved != device)
            clode::check_cuda(cudaSetDevice(device), "cudaSetDevice");
    }
    ~CurrentDevice()
    {
        int now = -1;
        if (saved >= 0 && cudaGetDevice(&now) == cudaSuccess && now != saved)
            cudaSetDevice(saved);
    }
};

}  // namespace

extern "C" int clode_sim_features_noalloc(clode_sim *sim, long long n_pts, const void *x0, const void *pars,
                                          const void *tspan, unsigned long long *rng, void *dt, void *xf, void *tf,
                                          void *F, int *status, void *stream)
{
    try {
        clode::NoallocFeaturesLaunch L;
        clode::noalloc_features_prepare(sim, &L);
        if (n_pts < 0 || n_pts > 0x3fffffffLL)
            clode::fail(CLODE_ERR_INVALID_ARGUMENT, "n_pts=%lld out of range", n_pts);
        if (n_pts == 0) {
            clode::set_last_error_message("");
            return CLODE_OK;
        }
        const size_t per_member = (size_t)L.obs_words * 4u;
        const size_t need = kHeaderBytes + per_member * (size_t)n_pts;
        if (need > kScratchBytes)
            clode::fail(CLODE_ERR_INVALID_ARGUMENT,
                        "n_pts=%lld needs %zu bytes of observer scratch (%zu per member) but the fixed scratch holds "
                        "%zu bytes: at most %zu members per call for this observer",
                        n_pts, need, per_member, kScratchBytes, (kScratchBytes - kHeaderBytes) / per_member);
        if (!x0 || !rng || !dt || !xf || !tf || !F)
            clode::fail(CLODE_ERR_INVALID_ARGUMENT, "x0, rng, dt, xf, tf and F must be device pointers");
        if (L.n_par > 0 && !pars)
            clode::fail(CLODE_ERR_INVALID_ARGUMENT, "pars must be a device pointer: the model has %d parameters",
                        L.n_par);
        CurrentDevice on_device(L.device);
        unsigned char *base = (unsigned char *)scratch_address(L.device);
        cudaStream_t s = (cudaStream_t)stream;
        // the work counter must start at zero; the parked observer state of a
        // member is written by the initialisation pass before it is read
        clode::check_cuda(cudaMemsetAsync(base, 0, kHeaderBytes, s), "scratch reset");

        int per_sm = 0, sms = 0;
        clode::check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, L.kernel, L.block, 0),
                          "occupancy query");
        clode::check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, L.device), "SM count");
        unsigned long long blocks = (unsigned long long)(per_sm > 0 ? per_sm : 1) * sms;
        unsigned long long cover = ((unsigned long long)n_pts + L.block - 1) / L.block;
        dim3 grid((unsigned int)(blocks < cover ? blocks : cover)), block(L.block);
        if (L.single) {
            clode::ArgsT<float> a;
            memcpy(&a, L.args, sizeof a);
            launch_features(a, L, n_pts, x0, pars, tspan, rng, dt, xf, tf, F, status, base, grid, block, s);
        } else {
            clode::ArgsT<double> a;
            memcpy(&a, L.args, sizeof a);
            launch_features(a, L, n_pts, x0, pars, tspan, rng, dt, xf, tf, F, status, base, grid, block, s);
        }
        clode::set_last_error_message("");
        return CLODE_OK;
    } catch (const clode::Error &e) {
        clode::set_last_error_message(e.what());
        return e.code;
    } catch (const std::exception &e) {
        clode::set_last_error_message(e.what());
        return CLODE_ERR_INTERNAL;
    }
}
