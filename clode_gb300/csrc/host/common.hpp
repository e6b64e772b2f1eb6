// Internal declarations shared by the host runtime translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../../include/clode_gb300.h"

namespace clode {

// An error carrying a CLODE_ERR_* code; the C ABI converts it to a status.
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &msg) : std::runtime_error(msg), code(c) {}
};

[[noreturn]] void fail(int code, const char *fmt, ...);
void check_cuda(cudaError_t e, const char *what);

// ------------------------------------------------------------------ logging
// A process-wide logger with the levels of clODE's LogLevel enum; messages go
// to stdout, or to a sink installed with clode_log_set_sink().
void log_msg(int level, const char *fmt, ...);
int log_level();

// ----------------------------------------------------------------- devices
// Makes `device` current on this thread (and initialises its primary context).
void use_device(int device);
int device_count_or_zero();

// ------------------------------------------------------------ NVRTC programs
struct ProgramSpec {
    std::string rhs_source;
    std::string rhs_name;
    std::vector<std::string> defines;   // "-DNAME=VALUE"
    bool fmad = false;
    bool prec_div = true;               // IEEE division; false: approximate (2 ulp)
    bool ftz = false;                   // flush FP32 denormals to zero
    int maxrregcount = 0;               // 0: no register cap
    bool fast_math = false;             // --use_fast_math: approximate exp/log/pow/sin/cos/sqrt (+ ftz, fast division)
    std::string arch;                   // e.g. "sm_103a"
};

struct CompiledProgram {
    std::vector<char> cubin;
    std::string log;
    std::string source;                 // the full program text handed to NVRTC
    std::string options;
    std::string key;
};

// Compile (or fetch from the on-disk cache) the ensemble program for `spec`.
CompiledProgram compile_program(const ProgramSpec &spec);
// "sm_XY[a]" of a device; "sm_103a" when no device is present.
std::string device_arch(int device);
void set_cache_dir(const std::string &dir);

// every kernel launch the library issues is counted (clode_launch_count)
void count_launch();

// Launch description of a built feature simulator's persistent features
// kernel, for the entry point that allocates nothing (noalloc.cu): solver and
// observer parameters and the global time span filled in, every buffer
// pointer left null for the caller's memory and the shared scratch.
struct NoallocFeaturesLaunch {
    void *kernel;          // cudaKernel_t of clode_features_persistent
    int single;            // working precision is float
    unsigned int obs_words;
    int n_par;             // parameter columns the kernel reads from pars
    int device;
    int block;
    unsigned char args[768];  // ArgsT<float> or ArgsT<double>
};
}  // namespace clode

struct clode_sim;

namespace clode {
void noalloc_features_prepare(clode_sim *sim, NoallocFeaturesLaunch *out);
// sets the message clode_last_error() returns on this thread
void set_last_error_message(const char *msg);

// -------------------------------------------------------------- AOT kernels
void launch_f64_to_f32(const double *src, float *dst, size_t n, cudaStream_t s);
void launch_f32_to_f64(const float *src, double *dst, size_t n, cudaStream_t s);
void launch_seed_rng_sequential(unsigned long long *rng, size_t n, int seed, cudaStream_t s);
void launch_seed_rng_random(unsigned long long *rng, size_t n, unsigned long long base, cudaStream_t s);
void launch_fill_f32(float *dst, float v, size_t n, cudaStream_t s);
void launch_fill_f64(double *dst, double v, size_t n, cudaStream_t s);
void launch_fill_i32(int *dst, int v, size_t n, cudaStream_t s);
// Members by decreasing per-member time span (tspan [2 i], [2 i + 1] on the
// device): with scratch == NULL only *scratch_bytes is set
void order_by_span_f32(const float *tspan, size_t n, int *order, void *scratch, size_t *scratch_bytes, cudaStream_t s);
void order_by_span_f64(const double *tspan, size_t n, int *order, void *scratch, size_t *scratch_bytes, cudaStream_t s);
// Members by decreasing count (counts[i] >= 0), same conventions
void order_by_count(const int *counts, size_t n, int *order, void *scratch, size_t *scratch_bytes, cudaStream_t s);
// dst[(i - m0) * nc + c] = src[c * ld + i] for members i in [m0, m0 + nm), c < nc
void launch_regroup_by_member_f32(const float *src, size_t ld, size_t m0, size_t nm, size_t nc, double *dst,
                                  cudaStream_t s);
void launch_regroup_by_member_f64(const double *src, size_t ld, size_t m0, size_t nm, size_t nc, double *dst,
                                  cudaStream_t s);

}  // namespace clode
