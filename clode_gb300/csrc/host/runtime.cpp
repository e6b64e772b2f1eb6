// Host runtime: errors, logging, device selection and the NVRTC program
// builder with its on-disk cache.  Replaces clODE's OpenCLResource layer
// (clode/cpp/OpenCLResource.cpp:40-296): where that layer picks an OpenCL
// platform/device and JIT-builds the kernel source with the device driver,
// this one selects a CUDA device and compiles the ensemble program for its
// architecture with NVRTC, which is loaded at run time (dlopen) so that the
// library itself loads on machines without a GPU driver.
#include "common.hpp"

#include <dlfcn.h>
#include <nvrtc.h>
#include <sys/stat.h>
#include <unistd.h>

#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <mutex>
#include <sstream>

namespace clode {

// ------------------------------------------------------------------ errors
[[noreturn]] void fail(int code, const char *fmt, ...)
{
    char buf[4096];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    throw Error(code, buf);
}

void check_cuda(cudaError_t e, const char *what)
{
    if (e == cudaSuccess)
        return;
    int code = CLODE_ERR_CUDA;
    if (e == cudaErrorMemoryAllocation)
        code = CLODE_ERR_OUT_OF_MEMORY;
    else if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver || e == cudaErrorInvalidDevice)
        code = CLODE_ERR_NO_DEVICE;
    cudaGetLastError();  // clear a sticky launch error so later calls report their own
    fail(code, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
}

// ----------------------------------------------------------------- logging
namespace {
std::mutex g_log_mu;
int g_log_level = CLODE_LOG_WARN;
std::string g_log_pattern = "[%Y-%m-%d %H:%M:%S.%e] [%n] [%l] %v";
clode_log_sink_fn g_log_sink = nullptr;
const char *kLevelNames[] = {"trace", "debug", "info", "warning", "error", "critical", "off"};

std::string format_line(int level, const std::string &msg)
{
    // the subset of spdlog's pattern flags that clODE users set
    auto now = std::chrono::system_clock::now();
    std::time_t tt = std::chrono::system_clock::to_time_t(now);
    int ms = (int)(std::chrono::duration_cast<std::chrono::milliseconds>(now.time_since_epoch()).count() % 1000);
    std::tm tm;
    localtime_r(&tt, &tm);
    std::string out;
    const std::string &p = g_log_pattern;
    for (size_t i = 0; i < p.size(); ++i) {
        if (p[i] != '%' || i + 1 == p.size()) {
            out += p[i];
            continue;
        }
        char f = p[++i];
        char b[32];
        switch (f) {
        case 'v': out += msg; break;
        case 'l': out += kLevelNames[level]; break;
        case 'L': out += (char)toupper(kLevelNames[level][0]); break;
        case 'n': out += "clode"; break;
        case 'Y': snprintf(b, sizeof b, "%04d", tm.tm_year + 1900); out += b; break;
        case 'm': snprintf(b, sizeof b, "%02d", tm.tm_mon + 1); out += b; break;
        case 'd': snprintf(b, sizeof b, "%02d", tm.tm_mday); out += b; break;
        case 'H': snprintf(b, sizeof b, "%02d", tm.tm_hour); out += b; break;
        case 'M': snprintf(b, sizeof b, "%02d", tm.tm_min); out += b; break;
        case 'S': snprintf(b, sizeof b, "%02d", tm.tm_sec); out += b; break;
        case 'e': snprintf(b, sizeof b, "%03d", ms); out += b; break;
        case '%': out += '%'; break;
        default: out += '%'; out += f; break;
        }
    }
    return out;
}
}  // namespace

void log_msg(int level, const char *fmt, ...)
{
    if (level < g_log_level || level >= CLODE_LOG_OFF)
        return;
    char buf[8192];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    std::lock_guard<std::mutex> lk(g_log_mu);
    std::string line = format_line(level, buf);
    if (g_log_sink) {
        g_log_sink(level, line.c_str());
    } else {
        fprintf(stdout, "%s\n", line.c_str());
        fflush(stdout);
    }
}

int log_level() { return g_log_level; }

namespace {
std::atomic<unsigned long long> g_launches{0};
}

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

// ----------------------------------------------------------------- devices
int device_count_or_zero()
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

void use_device(int device)
{
    int n = device_count_or_zero();
    if (n == 0)
        fail(CLODE_ERR_NO_DEVICE, "no CUDA device is available (this engine has no CPU path)");
    if (device < 0 || device >= n)
        fail(CLODE_ERR_NO_DEVICE, "CUDA device %d does not exist (%d present)", device, n);
    check_cuda(cudaSetDevice(device), "cudaSetDevice");
    check_cuda(cudaFree(nullptr), "CUDA context initialisation");
}

std::string device_arch(int device)
{
    int n = device_count_or_zero();
    if (n == 0 || device < 0 || device >= n)
        return "sm_103a";
    int major = 0, minor = 0;
    check_cuda(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device), "compute capability");
    check_cuda(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device), "compute capability");
    char b[32];
    // architecture-specific targets ("a") for Hopper and Blackwell parts
    snprintf(b, sizeof b, "sm_%d%d%s", major, minor, major >= 9 ? "a" : "");
    return b;
}

// ------------------------------------------------------------------ NVRTC
namespace {
struct Nvrtc {
    void *h = nullptr;
    decltype(&nvrtcCreateProgram) create = nullptr;
    decltype(&nvrtcCompileProgram) compile = nullptr;
    decltype(&nvrtcDestroyProgram) destroy = nullptr;
    decltype(&nvrtcGetCUBINSize) cubin_size = nullptr;
    decltype(&nvrtcGetCUBIN) cubin = nullptr;
    decltype(&nvrtcGetProgramLogSize) log_size = nullptr;
    decltype(&nvrtcGetProgramLog) log = nullptr;
    decltype(&nvrtcGetErrorString) err = nullptr;
    decltype(&nvrtcVersion) version = nullptr;
};

std::mutex g_nvrtc_mu;
Nvrtc g_nvrtc;
std::string g_cache_dir;

const Nvrtc &nvrtc()
{
    std::lock_guard<std::mutex> lk(g_nvrtc_mu);
    if (g_nvrtc.h)
        return g_nvrtc;
    std::vector<std::string> cands;
    if (const char *p = getenv("CLODE_NVRTC_LIBRARY"))
        cands.push_back(p);
    for (const char *env : {"CUDA_HOME", "CUDA_PATH"})
        if (const char *p = getenv(env))
            cands.push_back(std::string(p) + "/lib64/libnvrtc.so.13");
    cands.push_back("libnvrtc.so.13");
    cands.push_back("/usr/local/cuda/lib64/libnvrtc.so.13");
    cands.push_back("libnvrtc.so");
    void *h = nullptr;
    std::string tried;
    for (auto &c : cands) {
        h = dlopen(c.c_str(), RTLD_NOW | RTLD_GLOBAL);
        if (h)
            break;
        tried += " " + c;
    }
    if (!h)
        fail(CLODE_ERR_COMPILE, "cannot load NVRTC (tried:%s); set CLODE_NVRTC_LIBRARY", tried.c_str());
    Nvrtc n;
    n.h = h;
#define CLODE_SYM(field, name)                                                     \
    n.field = (decltype(n.field))dlsym(h, name);                                   \
    if (!n.field)                                                                  \
        fail(CLODE_ERR_COMPILE, "NVRTC library lacks %s", name);
    CLODE_SYM(create, "nvrtcCreateProgram")
    CLODE_SYM(compile, "nvrtcCompileProgram")
    CLODE_SYM(destroy, "nvrtcDestroyProgram")
    CLODE_SYM(cubin_size, "nvrtcGetCUBINSize")
    CLODE_SYM(cubin, "nvrtcGetCUBIN")
    CLODE_SYM(log_size, "nvrtcGetProgramLogSize")
    CLODE_SYM(log, "nvrtcGetProgramLog")
    CLODE_SYM(err, "nvrtcGetErrorString")
    CLODE_SYM(version, "nvrtcVersion")
#undef CLODE_SYM
    g_nvrtc = n;
    return g_nvrtc;
}

#include "device_headers.inc"

uint64_t fnv1a(const std::string &s, uint64_t h = 1469598103934665603ull)
{
    for (unsigned char c : s) {
        h ^= c;
        h *= 1099511628211ull;
    }
    return h;
}

std::string cache_dir()
{
    if (!g_cache_dir.empty())
        return g_cache_dir;
    if (const char *p = getenv("CLODE_GB300_CACHE_DIR"))
        return p;
    if (const char *p = getenv("XDG_CACHE_HOME"))
        return std::string(p) + "/clode_gb300";
    if (const char *p = getenv("HOME"))
        return std::string(p) + "/.cache/clode_gb300";
    return "/tmp/clode_gb300_cache";
}

void mkdirs(const std::string &path)
{
    std::string cur;
    std::stringstream ss(path);
    std::string part;
    if (!path.empty() && path[0] == '/')
        cur = "/";
    while (std::getline(ss, part, '/')) {
        if (part.empty())
            continue;
        cur += part + "/";
        mkdir(cur.c_str(), 0755);
    }
}

bool read_file(const std::string &fn, std::vector<char> &out)
{
    std::ifstream f(fn, std::ios::binary);
    if (!f)
        return false;
    out.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
    return true;
}

void write_file_atomic(const std::string &fn, const char *data, size_t n)
{
    std::string tmp = fn + ".tmp" + std::to_string(getpid());
    {
        std::ofstream f(tmp, std::ios::binary);
        if (!f)
            return;  // the cache is an optimisation only
        f.write(data, (std::streamsize)n);
    }
    rename(tmp.c_str(), fn.c_str());
}
}  // namespace

void set_cache_dir(const std::string &dir) { g_cache_dir = dir; }

CompiledProgram compile_program(const ProgramSpec &spec)
{
    CompiledProgram out;
    out.source = "#include \"clode_prelude.cuh\"\n#line 1 \"" + (spec.rhs_name.empty() ? std::string("rhs.cl") : spec.rhs_name) +
                 "\"\n" + spec.rhs_source + "\n#include \"clode_engine.cuh\"\n";
    std::vector<std::string> opts = {"--gpu-architecture=" + spec.arch, "-default-device",
                                     std::string("--fmad=") + (spec.fmad ? "true" : "false"), "-std=c++17",
                                     "-lineinfo", "--ptxas-options=-v"};
    if (!spec.prec_div)
        opts.push_back("-prec-div=false");
    if (spec.ftz)
        opts.push_back("-ftz=true");
    if (spec.maxrregcount > 0)  // applied per kernel (clode_kernels.cuh CLODE_CAP)
        opts.push_back("-DCLODE_MAXNREG=" + std::to_string(spec.maxrregcount));
    if (spec.fast_math)
        opts.push_back("--use_fast_math");
    for (auto &d : spec.defines)
        opts.push_back(d);
    std::string optline;
    for (auto &o : opts)
        optline += o + " ";
    out.options = optline;

    const Nvrtc &nv = nvrtc();
    int vmaj = 0, vmin = 0;
    nv.version(&vmaj, &vmin);
    uint64_t h = fnv1a(out.source);
    h = fnv1a(optline, h);
    h = fnv1a(std::to_string(vmaj) + "." + std::to_string(vmin), h);
    for (int k = 0; k < kDeviceHeaderCount; ++k) {
        h = fnv1a(kDeviceHeaderNames[k], h);
        h = fnv1a(kDeviceHeaderSources[k], h);
    }
    char key[40];
    snprintf(key, sizeof key, "%016llx", (unsigned long long)h);
    out.key = key;

    std::string dir = cache_dir();
    std::string base = dir + "/" + out.key + "_" + spec.arch;
    std::vector<char> cached, logbuf;
    if (read_file(base + ".cubin", cached) && !cached.empty()) {
        out.cubin.swap(cached);
        if (read_file(base + ".log", logbuf))
            out.log.assign(logbuf.begin(), logbuf.end());
        log_msg(CLODE_LOG_DEBUG, "ensemble program %s loaded from cache", out.key.c_str());
        return out;
    }

    nvrtcProgram prog;
    nvrtcResult r = nv.create(&prog, out.source.c_str(), "clode_program.cu", kDeviceHeaderCount, kDeviceHeaderSources,
                              kDeviceHeaderNames);
    if (r != NVRTC_SUCCESS)
        fail(CLODE_ERR_COMPILE, "nvrtcCreateProgram: %s", nv.err(r));
    std::vector<const char *> copts;
    for (auto &o : opts)
        copts.push_back(o.c_str());
    auto t0 = std::chrono::steady_clock::now();
    r = nv.compile(prog, (int)copts.size(), copts.data());
    double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    size_t lsz = 0;
    nv.log_size(prog, &lsz);
    std::string log(lsz, '\0');
    if (lsz)
        nv.log(prog, &log[0]);
    while (!log.empty() && log.back() == '\0')
        log.pop_back();
    out.log = log;
    if (r != NVRTC_SUCCESS) {
        nv.destroy(&prog);
        log_msg(CLODE_LOG_ERR, "ensemble program build failed:\n%s", log.c_str());
        fail(CLODE_ERR_COMPILE, "ensemble program build failed (%s):\n%s", nv.err(r), log.c_str());
    }
    size_t csz = 0;
    nv.cubin_size(prog, &csz);
    out.cubin.resize(csz);
    nv.cubin(prog, out.cubin.data());
    nv.destroy(&prog);
    log_msg(CLODE_LOG_INFO, "built ensemble program %s for %s in %.2f s", out.key.c_str(), spec.arch.c_str(), secs);
    mkdirs(dir);
    write_file_atomic(base + ".cubin", out.cubin.data(), out.cubin.size());
    write_file_atomic(base + ".log", out.log.data(), out.log.size());
    return out;
}

}  // namespace clode

// ------------------------------------------------------------ logging ABI
extern "C" {

int clode_log_set_level(int level)
{
    if (level < CLODE_LOG_TRACE || level > CLODE_LOG_OFF)
        return CLODE_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(clode::g_log_mu);
    clode::g_log_level = level;
    return CLODE_OK;
}

int clode_log_get_level(void) { return clode::g_log_level; }

unsigned long long clode_launch_count(void) { return clode::g_launches.load(); }

int clode_log_set_pattern(const char *pattern)
{
    if (!pattern)
        return CLODE_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(clode::g_log_mu);
    clode::g_log_pattern = pattern;
    return CLODE_OK;
}

int clode_log_set_sink(clode_log_sink_fn sink)
{
    std::lock_guard<std::mutex> lk(clode::g_log_mu);
    clode::g_log_sink = sink;
    return CLODE_OK;
}

int clode_log_message(int level, const char *message)
{
    if (level < CLODE_LOG_TRACE || level > CLODE_LOG_OFF || !message)
        return CLODE_ERR_INVALID_ARGUMENT;
    clode::log_msg(level, "%s", message);
    return CLODE_OK;
}

}  // extern "C"
