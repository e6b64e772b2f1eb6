// The simulator object behind the C ABI: one ensemble problem, its device
// buffers, its compiled program and its CUDA stream.  It re-implements the
// host logic of clODE's CLODE, CLODEfeatures and CLODEtrajectory classes
// (clode/cpp/CLODE.cpp, CLODEfeatures.cpp, CLODEtrajectory.cpp) over CUDA:
// buffer sizing on nPts changes, precision conversion of host doubles,
// RNG seeding, dt persistence for adaptive continuation, lazy observer
// initialisation and the x0/tspan shifts for continuation runs.
#include "common.hpp"
#include "rng_jump.hpp"
#include "../device/clode_args.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <random>
#include <sstream>

using namespace clode;

namespace {

// stepper name -> define (clode/cpp/steppers.cl:26-43)
const std::map<std::string, std::string> kSteppers = {
    {"euler", "EXPLICIT_EULER"}, {"heun", "EXPLICIT_HEUN"},     {"rk4", "EXPLICIT_RK4"},
    {"bs23", "EXPLICIT_BS23"},   {"dopri5", "EXPLICIT_DOPRI5"}, {"seuler", "STOCHASTIC_EULER"},
};

// observer name -> define (clode/cpp/observers.cl:122-143)
const std::map<std::string, std::string> kObservers = {
    {"basic", "USE_OBSERVER_BASIC"},
    {"basicall", "USE_OBSERVER_BASIC_ALLVAR"},
    {"localmax", "USE_OBSERVER_LOCAL_MAX"},
    {"nhood1", "USE_OBSERVER_NEIGHBORHOOD_1"},
    {"nhood2", "USE_OBSERVER_NEIGHBORHOOD_2"},
    {"thresh2", "USE_OBSERVER_THRESHOLD_2"},
};

std::vector<std::string> split_lines(const char *s)
{
    std::vector<std::string> out;
    if (!s)
        return out;
    std::string cur;
    for (const char *p = s; *p; ++p) {
        if (*p == '\n') {
            out.push_back(cur);
            cur.clear();
        } else {
            cur += *p;
        }
    }
    if (!cur.empty())
        out.push_back(cur);
    return out;
}

// Feature names, in the order the kernels write F: the getObserverInfo_*
// lists of clode/cpp/observers/observer_*.clh
std::vector<std::string> feature_names(const std::string &obs, const std::vector<std::string> &vars,
                                       const std::vector<std::string> &auxs, unsigned int fvar, unsigned int nse)
{
    std::vector<std::string> f;
    auto extent = [&](bool with_range_centre) {
        for (auto &v : vars) {
            f.push_back("max " + v);
            f.push_back("min " + v);
            f.push_back("mean " + v);
            if (with_range_centre) {
                f.push_back("range " + v);
                f.push_back("nhood center " + v);
            }
            f.push_back("max d" + v + "/dt");
            f.push_back("min d" + v + "/dt");
        }
        for (auto &a : auxs) {
            f.push_back("max " + a);
            f.push_back("min " + a);
            f.push_back("mean " + a);
        }
    };
    if (obs == "basic") {
        std::string v = fvar < vars.size() ? vars[fvar] : std::string("");
        f = {"max " + v, "min " + v, "mean " + v, "max d" + v + "/dt", "min d" + v + "/dt", "step count"};
    } else if (obs == "basicall") {
        extent(false);
        f.push_back("step count");
    } else if (obs == "localmax") {
        f = {"max IMI", "min IMI", "mean IMI", "max amplitude", "min amplitude", "mean amplitude"};
        extent(false);
        for (unsigned j = 0; j < nse; ++j) {
            f.push_back("localmax event time " + std::to_string(j));
            f.push_back("localmax event evar " + std::to_string(j));
            f.push_back("localmin event time " + std::to_string(j));
            f.push_back("localmin event evar " + std::to_string(j));
        }
        f.push_back("event count");
        f.push_back("step count");
    } else if (obs == "nhood1") {
        f = {"max period", "min period", "mean period", "max peaks", "min peaks", "mean peaks"};
        extent(false);
        f.push_back("period count");
        f.push_back("step count");
        f.push_back("max dt");
        f.push_back("min dt");
        f.push_back("mean dt");
    } else if (obs == "nhood2") {
        f = {"max period", "min period", "mean period", "max peaks", "min peaks", "mean peaks"};
        extent(true);
        for (unsigned j = 0; j < nse; ++j)
            f.push_back("nhood event time " + std::to_string(j));
        f.push_back("event count");
        f.push_back("step count");
        f.push_back("max dt");
        f.push_back("min dt");
        f.push_back("mean dt");
    } else if (obs == "thresh2") {
        for (const char *g : {"period", "peaks", "upDuration", "downDuration", "duty", "activeDip"}) {
            f.push_back(std::string("max ") + g);
            f.push_back(std::string("min ") + g);
            f.push_back(std::string("mean ") + g);
        }
        extent(false);
        for (unsigned j = 0; j < nse; ++j) {
            f.push_back("up event time " + std::to_string(j));
            f.push_back("down event time " + std::to_string(j));
        }
        f.push_back("event count");
        f.push_back("step count");
        f.push_back("max dt");
        f.push_back("min dt");
        f.push_back("mean dt");
    }
    return f;
}

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    void reserve(size_t b)
    {
        if (b <= bytes && p)
            return;
        release();
        if (b == 0)
            return;
        cudaError_t e = cudaMalloc(&p, b);
        if (e != cudaSuccess) {
            p = nullptr;
            bytes = 0;
            cudaGetLastError();
            fail(CLODE_ERR_OUT_OF_MEMORY, "cannot allocate %.3f GB on the device: %s", b / 1e9, cudaGetErrorString(e));
        }
        bytes = b;
    }
    void release()
    {
        if (p)
            cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <typename T>
    T *as() const { return (T *)p; }
};

thread_local std::string g_last_error;

}  // namespace

struct clode_sim {
    int kind = CLODE_SIM_BASE;
    // problem (ProblemInfo)
    std::string rhs_source, rhs_name;
    int nVar = 0, nPar = 0, nAux = 0, nWiener = 0;
    std::vector<std::string> var_names, par_names, aux_names;
    std::string stepper, observer;
    bool single = true;
    int device = 0;
    clode_solver_params sp = {0.1, 0.5, 1e-6, 1e-3, 1000000u, 1000000u, 1u};
    clode_observer_params op = {0u, 0u, 100u, 0u, 0.0, 0.0, 0.05, 0.2, 0.2, 0.0, 0.0, 0.0};
    double tspan[2] = {0.0, 1000.0};
    bool tspan_per_member = false;
    std::vector<double> tspan_pm;
    long long nPts = 0;
    std::vector<double> pars_host;

    // device state
    int buffers_device = -1;
    bool buffers_single = true;
    DevBuf x0, pars, xf, rng, dt, tf, tspan_dev, odata, F, t, x, dx, aux, nstored, status, stats, stage, work;
    DevBuf ev_t, ev_x, ev_dx, ev_aux, nevents;  // features with storage: event states
    DevBuf order, order_scratch;                // persistent kernels: members by decreasing time span
    DevBuf work_counts, order_work;             // warm-up steps per member; the feature pass's order by them
    // replay of the warm-up pass: record regions, row masks, member lists,
    // rows used per region, finish blocks, fallback list and its length
    DevBuf rec, rec_mask, rec_member, rec_used, fin, fallback, fallback_count;
    DevBuf rec_err;  // set by the replay when a shared-memory stage was not filled in time
    // pre-drawn deviates of stochastic trajectory runs: the deviates, each
    // member's count, the generator's jump matrices
    DevBuf noise, noise_count, noise_mats;

    // program
    bool built = false;
    CompiledProgram prog;
    std::string built_key;
    cudaLibrary_t lib = nullptr;
    int lib_device = -1;
    cudaKernel_t k_transient = nullptr, k_trajectory = nullptr, k_init = nullptr, kp_init = nullptr,
                 k_features = nullptr;
    cudaKernel_t kp_transient = nullptr, kp_trajectory = nullptr, kp_features = nullptr;
    cudaKernel_t kp_init_rec = nullptr, kp_replay = nullptr;  // replay of the warm-up pass
    cudaKernel_t kp_replay_staged = nullptr;                  // ... through shared-memory stages
    cudaKernel_t kp_record_replay = nullptr;                  // recording and replay in one launch
    cudaKernel_t k_noise_count = nullptr, k_noise_draw = nullptr;  // pre-drawn deviates (stochastic stepper)
    unsigned int fin_words = 0, rec_fields = 0;
    int last_grid = 0, last_block = 0;
    unsigned int obs_words = 0;
    unsigned int built_nse = 0;

    // features bookkeeping (CLODEfeatures.cpp:143-177)
    long long F_elements = -1;
    unsigned int odata_words_alloc = 0;
    bool observer_initialized = false;
    // trajectory bookkeeping (CLODEtrajectory.cpp:45-94)
    long long traj_rows = -1, traj_pts = -1, traj_width = -1;
    // stored columns (all when store_subset is false) and the event store
    bool store_subset = false;
    std::vector<int> store_var_ix, store_aux_ix;
    bool want_store = false;  // build the features kernels with storage (CLODE_FEATURE_STORE)
    bool built_store = false;
    std::string built_subset;
    long long ev_rows_alloc = -1, ev_pts = -1, ev_width = -1;
    unsigned int ev_rows = 0;
    bool events_valid = false;

    // engine options
    int schedule = 0;
    int block_size = 128;
    int blocks_per_sm = 0;
    bool fmad = false;
    bool prec_div = true;
    bool ftz = false;
    bool fast_math = false;
    bool fast_exp = false;        // FP32 exp and controller pow of a few ulp (CLODE_FAST_EXP)
    bool paired = true;           // FP32 Runge-Kutta stages two variables per instruction (CLODE_PAIRED)
    bool precise = false;         // precision option (CLODE_PRECISE): compensated time and means,
                                  // compensated error estimate, refined event times
    bool split_attempts = false;  // persistent kernels: one adaptive attempt per loop iteration
    int step_block = 16;          // persistent kernels: steps between warp-wide refill votes
    int maxrregcount = 0;
    double time_budget_ms = 0.0;
    bool fuse_init = false;  // separate initialisation launch, as the reference (CLODEfeatures.cpp:180-259)
    bool collect_stats = true;
    bool order_by_span = true;  // persistent kernels take the longest per-member time spans first
    bool order_valid = false;   // `order` holds the permutation of the current per-member spans
    bool order_by_work = true;  // the feature pass of a two-pass observer takes the members with the
                                // most warm-up steps first (the separate warm-up launch counts them)
    bool record_work = false;   // the next warm-up launch writes work_counts
    bool replay = true;         // two-pass observers: the feature pass replays the warm-up's stored steps
    double replay_mb = 0.0;     // record regions' size in MiB (0: sized to the need, within the free memory)
    int replay_stages = 0;      // shared-memory row stages per replay warp (0: rows read from global memory;
                                // -1: up to 4 that fit)
    double replay_cap_scale = 1.0;  // autotuner trials on a sample: the regions' memory scaled by its fraction
    bool replay_split = false;  // rows of the observer's event fields, the pass's sums taken while recording
    double replay_room = 2.5;   // region room kept for the members in flight, in mean member lengths
    bool replay_fused = false;  // recording and replay in one launch per launch pair
    bool predraw = false;       // stochastic trajectories: deviates drawn by their own launches first
    bool noise_on = false;      // make_args: the launch reads the pre-drawn deviates
    bool last_predrawn = false;
    double last_draw_ms = 0.0;  // the count and draw launches of the last pre-drawn run
    unsigned long long noise_stride = 0;
    unsigned int mats_block = 0;  // candidates per lane and round the jump matrices in noise_mats are for
    unsigned int last_stages = 0;          // stages the last replayed run used
    unsigned int last_regions_per_warp = 0;  // regions each replay warp of the last replayed run took
    unsigned int last_rewarm = 0;          // of last_fallback: members whose warm-up was run again
    double last_rows = 0.0;                // rows the last replayed run recorded (all regions, all launches)
    unsigned int last_reallocs = 0;        // record-region allocations the last replayed run made
    double last_warmup_ms = 0.0;           // the separate warm-up launch of the last integrated features run
    double replay_steps_per_member = 0.0;  // measured by the last replayed run (sizes the next one)
    int last_replay_chunks = 0;            // recording launches of the last replayed run
    unsigned int last_fallback = 0;        // members the last replayed run gave to the plain feature pass
    bool use_work_order = false;  // the next features launch runs members in order_work
    long long range_end = -1;  // autotuner trials: run members [0, range_end) only
    int range_stride = 1;      // ... every range_stride-th of them (persistent kernels)

    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t rev[3] = {nullptr, nullptr, nullptr};  // replayed runs: times of the launch kinds
    double last_record_ms = 0.0, last_replay_ms = 0.0, last_fallback_ms = 0.0;
    double last_ms = 0.0;
    unsigned long long last_stats[CLODE_STAT_COUNT] = {0};

    ~clode_sim()
    {
        if (buffers_device >= 0 || lib) {
            cudaSetDevice(buffers_device >= 0 ? buffers_device : lib_device);
            for (DevBuf *b : all_buffers())
                b->release();
            if (chain_graph)
                cudaGraphExecDestroy(chain_graph);
            if (lib)
                cudaLibraryUnload(lib);
            if (stream)
                cudaStreamDestroy(stream);
            if (ev0)
                cudaEventDestroy(ev0);
            if (ev1)
                cudaEventDestroy(ev1);
            for (cudaEvent_t &e : rev)
                if (e)
                    cudaEventDestroy(e);
            for (cudaEvent_t &e : dl_ev)
                if (e)
                    cudaEventDestroy(e);
        }
    }

    std::vector<DevBuf *> all_buffers()
    {
        return {&x0,  &pars,   &xf,    &rng,    &dt,   &tf,    &tspan_dev, &odata, &F,
                &t,   &x,      &dx,    &aux,    &nstored, &status, &stats, &stage, &work,
                &ev_t, &ev_x, &ev_dx, &ev_aux, &nevents, &order, &order_scratch, &work_counts, &order_work,
                &rec, &rec_mask, &rec_member, &rec_used, &fin, &fallback, &fallback_count, &rec_err,
                &noise, &noise_count, &noise_mats};
    }

    size_t real_size() const { return single ? sizeof(float) : sizeof(double); }
    bool stepper_adaptive() const { return stepper == "bs23" || stepper == "dopri5"; }
    // the builds in which the option "paired" changes the program (CLODE_PAIRED_STAGES)
    bool pairing_applies() const { return single && fmad && stepper == "dopri5" && nVar >= 2 && !precise; }
    bool obs_two_pass() const { return observer == "thresh2" || observer == "nhood2"; }

    // --------------------------------------------------------- set-up --
    void set_problem(const clode_problem *p)
    {
        if (!p || !p->rhs_source)
            fail(CLODE_ERR_INVALID_ARGUMENT, "problem info with an RHS source is required");
        if (p->n_var < 1 || p->n_par < 0 || p->n_aux < 0 || p->n_wiener < 0)
            fail(CLODE_ERR_INVALID_ARGUMENT, "invalid problem sizes nVar=%d nPar=%d nAux=%d nWiener=%d", p->n_var,
                 p->n_par, p->n_aux, p->n_wiener);
        rhs_source = p->rhs_source;
        rhs_name = p->rhs_name ? p->rhs_name : "rhs.cl";
        nVar = p->n_var;
        nPar = p->n_par;
        nAux = p->n_aux;
        nWiener = p->n_wiener;
        var_names = split_lines(p->var_names);
        par_names = split_lines(p->par_names);
        aux_names = split_lines(p->aux_names);
        while ((int)var_names.size() < nVar)
            var_names.push_back("x" + std::to_string(var_names.size()));
        while ((int)aux_names.size() < nAux)
            aux_names.push_back("aux" + std::to_string(aux_names.size()));
        var_names.resize(nVar);
        aux_names.resize(nAux);
        store_subset = false;  // stored columns index the old problem's variables
        store_var_ix.clear();
        store_aux_ix.clear();
        built = false;
    }

    // Stored columns of trajectories and event states.  A negative count
    // keeps every variable (or auxiliary variable); both negative restore
    // the reference layout.  Invalidates the stored arrays of earlier runs.
    void set_store_variables(const int *var_ix, int n_var_ix, const int *aux_ix, int n_aux_ix)
    {
        std::vector<int> v, w;
        if (n_var_ix >= 0) {
            if (n_var_ix > 0 && !var_ix)
                fail(CLODE_ERR_INVALID_ARGUMENT, "variable index list is null");
            for (int k = 0; k < n_var_ix; ++k) {
                if (var_ix[k] < 0 || var_ix[k] >= nVar)
                    fail(CLODE_ERR_INVALID_ARGUMENT, "stored variable index %d is outside [0, %d)", var_ix[k], nVar);
                v.push_back(var_ix[k]);
            }
        } else {
            for (int k = 0; k < nVar; ++k)
                v.push_back(k);
        }
        if (n_aux_ix >= 0) {
            if (n_aux_ix > 0 && !aux_ix)
                fail(CLODE_ERR_INVALID_ARGUMENT, "auxiliary index list is null");
            for (int k = 0; k < n_aux_ix; ++k) {
                if (aux_ix[k] < 0 || aux_ix[k] >= nAux)
                    fail(CLODE_ERR_INVALID_ARGUMENT, "stored auxiliary index %d is outside [0, %d)", aux_ix[k], nAux);
                w.push_back(aux_ix[k]);
            }
        } else {
            for (int k = 0; k < nAux; ++k)
                w.push_back(k);
        }
        store_subset = n_var_ix >= 0 || n_aux_ix >= 0;
        store_var_ix = store_subset ? v : std::vector<int>();
        store_aux_ix = store_subset ? w : std::vector<int>();
        traj_rows = -1;
        events_valid = false;
    }

    void set_stepper(const char *s)
    {
        std::string n = s ? s : "";
        if (kSteppers.count(n))
            stepper = n;
        else
            log_msg(CLODE_LOG_WARN, "Unknown stepper: %s. Stepper method unchanged", n.c_str());
        built = false;
    }

    void set_observer(const char *s)
    {
        std::string n = s ? s : "";
        if (kObservers.count(n))
            observer = n;
        else
            log_msg(CLODE_LOG_WARN, "unknown observer: %s. Observer method unchanged", n.c_str());
        built = false;
    }

    std::vector<std::string> names() const
    {
        return feature_names(observer, var_names, aux_names, op.f_var_ix, op.max_event_timestamps);
    }

    void ensure_stream()
    {
        use_device(device);
        if (!stream || buffers_device != device) {
            if (stream && buffers_device >= 0) {
                cudaSetDevice(buffers_device);
                cudaStreamDestroy(stream);
                cudaEventDestroy(ev0);
                cudaEventDestroy(ev1);
                for (cudaEvent_t &e : rev)
                    if (e) {
                        cudaEventDestroy(e);
                        e = nullptr;
                    }
                cudaSetDevice(device);
            }
            check_cuda(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
            check_cuda(cudaEventCreate(&ev0), "cudaEventCreate");
            check_cuda(cudaEventCreate(&ev1), "cudaEventCreate");
        }
    }

    // Rows the trajectory getters return: max_store, as CLODEtrajectory's
    // getters copy (CLODEtrajectory.cpp:132-200), but never more than the
    // buffers of the last run hold (max_store may have grown since).
    size_t stored_rows() const
    {
        return traj_rows > 0 ? std::min<size_t>(sp.max_store, (size_t)traj_rows - 1) : 0;
    }

    // ------------------------------------------------------------ build --
    static std::string join_ix(const std::vector<int> &v)
    {
        std::string r;
        for (size_t k = 0; k < v.size(); ++k)
            r += (k ? "," : "") + std::to_string(v[k]);
        return r;
    }

    std::string subset_key() const
    {
        return store_subset ? join_ix(store_var_ix) + "/" + join_ix(store_aux_ix) : std::string("all");
    }

    // stored columns per row: x (and dx) and aux
    int store_nv() const { return store_subset ? (int)store_var_ix.size() : nVar; }
    int store_na() const { return store_subset ? (int)store_aux_ix.size() : nAux; }

    ProgramSpec spec() const
    {
        ProgramSpec s;
        s.rhs_source = rhs_source;
        s.rhs_name = rhs_name;
        s.fmad = fmad;
        s.prec_div = prec_div;
        s.ftz = ftz;
        s.maxrregcount = maxrregcount;
        s.fast_math = fast_math;
        s.arch = device_arch(device);
        s.defines = {single ? "-DCLODE_SINGLE_PRECISION" : "-DCLODE_DOUBLE_PRECISION", "-D" + kSteppers.at(stepper),
                     "-DN_PAR=" + std::to_string(nPar), "-DN_VAR=" + std::to_string(nVar),
                     "-DN_AUX=" + std::to_string(nAux), "-DN_WIENER=" + std::to_string(nWiener),
                     std::string("-DCLODE_SPLIT_ATTEMPTS=") + (split_attempts ? "1" : "0"),
                     std::string("-DCLODE_FAST_EXP=") + (fast_exp ? "1" : "0"),
                     std::string("-DCLODE_PAIRED=") + (paired ? "1" : "0"),
                     std::string("-DCLODE_FMAD=") + (fmad ? "1" : "0"),
                     std::string("-DCLODE_FTZ=") + (ftz || fast_math ? "1" : "0"),
                     std::string("-DCLODE_PREC_DIV=") + (prec_div && !fast_math ? "1" : "0"),
                     std::string("-DCLODE_PRECISE=") + (precise ? "1" : "0"),
                     "-DCLODE_STEP_BLOCK=" + std::to_string(step_block)};
        if (kind == CLODE_SIM_FEATURES) {
            s.defines.push_back("-D" + kObservers.at(observer));
            s.defines.push_back("-DN_STORE_EVENTS=" + std::to_string(op.max_event_timestamps));
            if (want_store)
                s.defines.push_back("-DCLODE_FEATURE_STORE=1");
            if (!replay_split)
                s.defines.push_back("-DCLODE_REPLAY_WHOLE_ROWS=1");
        } else {
            s.defines.push_back("-DN_STORE_EVENTS=0");
        }
        if (store_subset) {
            s.defines.push_back("-DCLODE_STORE_NV=" + std::to_string(store_var_ix.size()));
            s.defines.push_back("-DCLODE_STORE_VARS=" + join_ix(store_var_ix));
            s.defines.push_back("-DCLODE_STORE_NA=" + std::to_string(store_aux_ix.size()));
            s.defines.push_back("-DCLODE_STORE_AUX=" + join_ix(store_aux_ix));
        }
        return s;
    }

    void build()
    {
        if (rhs_source.empty())
            fail(CLODE_ERR_STATE, "no problem info set");
        if (!kSteppers.count(stepper))
            fail(CLODE_ERR_INVALID_ARGUMENT, "no valid stepper selected");
        if (kind == CLODE_SIM_FEATURES && !kObservers.count(observer))
            fail(CLODE_ERR_INVALID_ARGUMENT, "no valid observer selected");
        if (kind == CLODE_SIM_FEATURES && nVar > 0 && (op.e_var_ix >= (unsigned)nVar || op.f_var_ix >= (unsigned)nVar))
            fail(CLODE_ERR_INVALID_ARGUMENT, "observer variable index out of range (eVarIx=%u fVarIx=%u nVar=%d)",
                 op.e_var_ix, op.f_var_ix, nVar);
        ProgramSpec s = spec();
        CompiledProgram p = compile_program(s);
        bool have_device = device_count_or_zero() > 0;
        if (have_device) {
            use_device(device);
            cudaLibrary_t nl = nullptr;
            check_cuda(cudaLibraryLoadData(&nl, p.cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0),
                       "loading the ensemble program");
            if (lib) {
                cudaSetDevice(lib_device);
                cudaLibraryUnload(lib);
                cudaSetDevice(device);
            }
            lib = nl;
            lib_device = device;
            check_cuda(cudaLibraryGetKernel(&k_transient, lib, "clode_transient"), "kernel clode_transient");
            check_cuda(cudaLibraryGetKernel(&k_trajectory, lib, "clode_trajectory"), "kernel clode_trajectory");
            check_cuda(cudaLibraryGetKernel(&kp_transient, lib, "clode_transient_persistent"),
                       "kernel clode_transient_persistent");
            check_cuda(cudaLibraryGetKernel(&kp_trajectory, lib, "clode_trajectory_persistent"),
                       "kernel clode_trajectory_persistent");
            k_init = kp_init = k_features = kp_features = nullptr;
            kp_init_rec = kp_replay = kp_replay_staged = kp_record_replay = nullptr;
            k_noise_count = k_noise_draw = nullptr;
            if (stepper == "seuler") {
                check_cuda(cudaLibraryGetKernel(&k_noise_count, lib, "clode_noise_count"), "kernel clode_noise_count");
                check_cuda(cudaLibraryGetKernel(&k_noise_draw, lib, "clode_noise_draw"), "kernel clode_noise_draw");
            }
            obs_words = 0;
            if (kind == CLODE_SIM_FEATURES) {
                check_cuda(cudaLibraryGetKernel(&k_init, lib, "clode_init_observer"), "kernel clode_init_observer");
                check_cuda(cudaLibraryGetKernel(&kp_init, lib, "clode_init_observer_persistent"),
                           "kernel clode_init_observer_persistent");
                check_cuda(cudaLibraryGetKernel(&k_features, lib, "clode_features"), "kernel clode_features");
                check_cuda(cudaLibraryGetKernel(&kp_features, lib, "clode_features_persistent"),
                           "kernel clode_features_persistent");
                void *gp = nullptr;
                size_t gb = 0;
                check_cuda(cudaLibraryGetGlobal(&gp, &gb, lib, "clode_observer_words"), "observer state size");
                check_cuda(cudaMemcpy(&obs_words, gp, sizeof obs_words, cudaMemcpyDeviceToHost), "observer state size");
                fin_words = rec_fields = 0;
                if (!want_store) {
                    check_cuda(cudaLibraryGetKernel(&kp_init_rec, lib, "clode_init_observer_record"),
                               "kernel clode_init_observer_record");
                    check_cuda(cudaLibraryGetKernel(&kp_replay, lib, "clode_features_replay"),
                               "kernel clode_features_replay");
                    check_cuda(cudaLibraryGetKernel(&kp_replay_staged, lib, "clode_features_replay_staged"),
                               "kernel clode_features_replay_staged");
                    check_cuda(cudaLibraryGetKernel(&kp_record_replay, lib, "clode_features_record_replay"),
                               "kernel clode_features_record_replay");
                    check_cuda(cudaLibraryGetGlobal(&gp, &gb, lib, "clode_finish_words"), "finish block size");
                    check_cuda(cudaMemcpy(&fin_words, gp, sizeof fin_words, cudaMemcpyDeviceToHost),
                               "finish block size");
                    check_cuda(cudaLibraryGetGlobal(&gp, &gb, lib, "clode_record_fields"), "record size");
                    check_cuda(cudaMemcpy(&rec_fields, gp, sizeof rec_fields, cudaMemcpyDeviceToHost), "record size");
                }
            }
        }
        prog = p;
        built_key = p.key;
        built_nse = op.max_event_timestamps;
        built_store = want_store;
        built_subset = subset_key();
        built = true;
        log_msg(CLODE_LOG_DEBUG, "program %s ready (%s, %s, %s)", p.key.c_str(), stepper.c_str(),
                kind == CLODE_SIM_FEATURES ? observer.c_str() : "-", single ? "single" : "double");
    }

    // the program was built for the current observer parameters that it compiles in
    bool observer_program_current() const
    {
        return built_nse == op.max_event_timestamps;
    }

    void ensure_built()
    {
        if (!built || lib == nullptr || lib_device != device || (kind == CLODE_SIM_FEATURES && !observer_program_current()) ||
            built_store != want_store || built_subset != subset_key()) {
            if (device_count_or_zero() == 0)
                fail(CLODE_ERR_NO_DEVICE, "no CUDA device is available (this engine has no CPU path)");
            build();
        }
    }

    // ---------------------------------------------------- problem data --
    // The device address of page-locked host memory the caller holds (null
    // for any other memory): kernels read and write it directly, over the
    // host link, without a staging copy.
    static void *pinned_device_ptr(const void *host)
    {
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
            (void)cudaGetLastError();
            return nullptr;
        }
        return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
    }

    void upload(DevBuf &dst, const double *src, size_t n)
    {
        if (n == 0)
            return;
        if (single) {
            // page-locked source: converted straight from host memory
            if (void *d = pinned_device_ptr(src)) {
                launch_f64_to_f32(static_cast<const double *>(d), dst.as<float>(), n, stream);
                check_cuda(cudaStreamSynchronize(stream), "H2D conversion");
                return;
            }
        }
        HostPin pin(const_cast<double *>(src), n * sizeof(double));
        if (single) {
            stage.reserve(n * sizeof(double));
            check_cuda(cudaMemcpyAsync(stage.p, src, n * sizeof(double), cudaMemcpyHostToDevice, stream), "H2D copy");
            launch_f64_to_f32(stage.as<double>(), dst.as<float>(), n, stream);
        } else {
            check_cuda(cudaMemcpyAsync(dst.p, src, n * sizeof(double), cudaMemcpyHostToDevice, stream), "H2D copy");
        }
        check_cuda(cudaStreamSynchronize(stream), "H2D copy");
    }

    // Page-locks a large caller-owned host range while it receives a copy,
    // so the device-to-host transfer runs at the link's rate instead of
    // through the driver's pageable staging.  A range that cannot be
    // registered (or already is) is copied as it is.
    struct HostPin {
        void *p = nullptr;
        HostPin(void *ptr, size_t bytes)
        {
            if (ptr && bytes >= ((size_t)32 << 20)) {
                // memory the caller already page-locked is used as it is
                cudaPointerAttributes at;
                if (cudaPointerGetAttributes(&at, ptr) == cudaSuccess && at.type == cudaMemoryTypeHost)
                    return;
                (void)cudaGetLastError();
                if (cudaHostRegister(ptr, bytes, cudaHostRegisterDefault) == cudaSuccess)
                    p = ptr;
                else
                    (void)cudaGetLastError();
            }
        }
        ~HostPin()
        {
            if (p)
                cudaHostUnregister(p);
        }
        HostPin(const HostPin &) = delete;
        HostPin &operator=(const HostPin &) = delete;
    };

    void download(const DevBuf &src, double *dst, size_t n)
    {
        if (n == 0)
            return;
        const auto w0 = std::chrono::steady_clock::now();
        // page-locked destination: the conversion kernel writes it directly
        void *direct = single ? pinned_device_ptr(dst) : nullptr;
        HostPin pin(direct ? nullptr : dst, n * sizeof(double));
        const auto w1 = std::chrono::steady_clock::now();
        for (cudaEvent_t *e : {&dl_ev[0], &dl_ev[1], &dl_ev[2]})
            if (!*e)
                check_cuda(cudaEventCreate(e), "cudaEventCreate");
        check_cuda(cudaEventRecord(dl_ev[0], stream), "event record");
        check_cuda(cudaEventRecord(dl_ev[2], stream), "event record");
        if (direct) {
            launch_f32_to_f64(src.as<float>(), static_cast<double *>(direct), n, stream);
            check_cuda(cudaEventRecord(dl_ev[2], stream), "event record");
        } else if (single) {
            stage.reserve(n * sizeof(double));
            launch_f32_to_f64(src.as<float>(), stage.as<double>(), n, stream);
            check_cuda(cudaEventRecord(dl_ev[2], stream), "event record");
            check_cuda(cudaMemcpyAsync(dst, stage.p, n * sizeof(double), cudaMemcpyDeviceToHost, stream), "D2H copy");
        } else {
            check_cuda(cudaMemcpyAsync(dst, src.p, n * sizeof(double), cudaMemcpyDeviceToHost, stream), "D2H copy");
        }
        check_cuda(cudaEventRecord(dl_ev[1], stream), "event record");
        check_cuda(cudaStreamSynchronize(stream), "D2H copy");
        float ms = 0.0f, cv = 0.0f;
        check_cuda(cudaEventElapsedTime(&ms, dl_ev[0], dl_ev[1]), "event timing");
        check_cuda(cudaEventElapsedTime(&cv, dl_ev[0], dl_ev[2]), "event timing");
        last_download_ms = ms;
        last_download_convert_ms = cv;
        last_download_pin_ms = std::chrono::duration<double, std::milli>(w1 - w0).count();
        last_download_wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - w0).count();
    }
    cudaEvent_t dl_ev[3] = {nullptr, nullptr, nullptr};
    double last_download_ms = 0.0, last_download_wall_ms = 0.0, last_download_pin_ms = 0.0;
    double last_download_convert_ms = 0.0;

    void fill_real(DevBuf &b, double v, size_t n)
    {
        if (single)
            launch_fill_f32(b.as<float>(), (float)v, n, stream);
        else
            launch_fill_f64(b.as<double>(), v, n, stream);
    }

    // CLODE::setNpts (CLODE.cpp:174-242): resize, dt = sp.dt, random seed
    void set_npts(long long n)
    {
        ensure_stream();
        bool realloc = n != nPts || buffers_device != device || buffers_single != single;
        if (!realloc)
            return;
        if (buffers_device >= 0 && buffers_device != device) {
            cudaSetDevice(buffers_device);
            for (DevBuf *b : all_buffers())
                b->release();
            cudaSetDevice(device);
        }
        nPts = n;
        buffers_device = device;
        buffers_single = single;
        size_t rs = real_size();
        x0.reserve(std::max<size_t>(1, nVar * n) * rs);
        pars.reserve(std::max<size_t>(1, nPar * n) * rs);
        xf.reserve(std::max<size_t>(1, nVar * n) * rs);
        rng.reserve(std::max<size_t>(1, 2 * n) * sizeof(unsigned long long));
        dt.reserve(std::max<size_t>(1, n) * rs);
        tf.reserve(std::max<size_t>(1, n) * rs);
        status.reserve(std::max<size_t>(1, n) * sizeof(int));
        stats.reserve(CLODE_STAT_COUNT * sizeof(unsigned long long));
        work.reserve(64);
        fill_real(dt, sp.dt, n);
        F_elements = -1;
        traj_rows = -1;
        events_valid = false;
        ev_rows_alloc = -1;  // event buffers are re-made for the new size or precision
        order_valid = false;
        observer_initialized = false;
        if (tspan_per_member && (long long)tspan_pm.size() != 2 * n) {
            tspan_per_member = false;
            log_msg(CLODE_LOG_WARN, "ensemble size changed: per-member time spans dropped, using [%g, %g]", tspan[0],
                    tspan[1]);
        }
        seed_rng(false, 0);
        log_msg(CLODE_LOG_DEBUG, "set nPts=%lld", n);
    }

    void set_problem_data(const double *nx0, size_t n_x0, const double *np, size_t n_p)
    {
        if (n_x0 % (size_t)nVar != 0)
            fail(CLODE_ERR_INVALID_ARGUMENT, "Invalid initial condition vector: not a multiple of nVar=%d", nVar);
        long long n = (long long)(n_x0 / nVar);
        if (nPar > 0) {
            if (n_p % (size_t)nPar != 0)
                fail(CLODE_ERR_INVALID_ARGUMENT, "Invalid parameter vector: not a multiple of nPar=%d", nPar);
            if ((long long)(n_p / nPar) != n)
                fail(CLODE_ERR_INVALID_ARGUMENT,
                     "Initial condition and parameter vector dimensions don't match: %lld sets of x0, %zu of pars", n,
                     n_p / nPar);
        } else if (n_p != 0) {
            fail(CLODE_ERR_INVALID_ARGUMENT, "parameters given for a problem with nPar=0");
        }
        if (n > INT32_MAX / 2)
            fail(CLODE_ERR_INVALID_ARGUMENT, "nPts=%lld exceeds the supported maximum %d", n, INT32_MAX / 2);
        set_npts(n);
        set_x0(nx0, n_x0);
        set_pars(np, n_p);
    }

    void set_x0(const double *v, size_t n)
    {
        if ((long long)n != nPts * nVar)
            fail(CLODE_ERR_INVALID_ARGUMENT, "Invalid initial condition vector: expected %lld*%d elements, received %zu",
                 nPts, nVar, n);
        ensure_stream();
        upload(x0, v, n);
    }

    void set_pars(const double *v, size_t n)
    {
        if ((long long)n != nPts * nPar)
            fail(CLODE_ERR_INVALID_ARGUMENT, "Invalid parameter vector: expected %lld*%d elements, received %zu", nPts,
                 nPar, n);
        ensure_stream();
        pars_host.assign(v, v + n);
        upload(pars, v, n);
    }

    void seed_rng(bool use_seed, int seed)
    {
        if (nPts == 0)
            return;
        ensure_stream();
        if (use_seed) {
            launch_seed_rng_sequential(rng.as<unsigned long long>(), 2 * (size_t)nPts, seed, stream);
        } else {
            std::random_device rd;
            unsigned long long base = ((unsigned long long)rd() << 32) ^ rd();
            launch_seed_rng_random(rng.as<unsigned long long>(), 2 * (size_t)nPts, base, stream);
        }
        check_cuda(cudaStreamSynchronize(stream), "RNG seeding");
    }

    // ------------------------------------------------------------ runs --
    template <typename R>
    ArgsT<R> make_args()
    {
        ArgsT<R> a;
        memset(&a, 0, sizeof a);
        a.nPts = (int)nPts;
        a.i_begin = 0;
        a.i_end = (int)(range_end >= 0 ? std::min(range_end, nPts) : nPts);
        a.i_stride = range_stride;
        a.t0 = (R)tspan[0];
        a.t1 = (R)tspan[1];
        a.tspan_pm = tspan_per_member ? tspan_dev.as<R>() : nullptr;
        a.x0 = x0.as<R>();
        a.pars = pars.as<R>();
        a.xf = xf.as<R>();
        a.rng = rng.as<unsigned long long>();
        a.dt = dt.as<R>();
        a.tf = tf.as<R>();
        a.odata = odata.as<unsigned int>();
        a.F = F.as<R>();
        a.t_out = t.as<R>();
        a.x_out = x.as<R>();
        a.dx_out = dx.as<R>();
        a.aux_out = aux.as<R>();
        a.n_stored = nstored.as<int>();
        a.work_out = record_work ? work_counts.as<int>() : nullptr;
        a.ev_t = ev_t.as<R>();
        a.ev_x = ev_x.as<R>();
        a.ev_dx = ev_dx.as<R>();
        a.ev_aux = ev_aux.as<R>();
        a.n_events = nevents.as<int>();
        a.ev_rows = ev_rows;
        a.status = status.as<int>();
        a.stats = collect_stats ? stats.as<unsigned long long>() : nullptr;
        a.work_next = work.as<unsigned int>();
        a.time_budget_ns = (unsigned long long)(time_budget_ms * 1e6);
        if (noise_on) {
            a.noise = noise.as<R>();
            a.noise_stride = noise_stride;
        }
        a.sp.dt = (R)sp.dt;
        a.sp.dtmax = (R)sp.dtmax;
        a.sp.abstol = (R)sp.abstol;
        a.sp.reltol = (R)sp.reltol;
        a.sp.max_steps = sp.max_steps;
        a.sp.max_store = sp.max_store;
        a.sp.nout = sp.nout;
        a.op.eVarIx = op.e_var_ix;
        a.op.fVarIx = op.f_var_ix;
        a.op.maxEventCount = op.max_event_count;
        a.op.maxEventTimestamps = op.max_event_timestamps;
        a.op.minXamp = (R)op.min_x_amp;
        a.op.minIMI = (R)op.min_imi;
        a.op.nHoodRadius = (R)op.nhood_radius;
        a.op.xUpThresh = (R)op.x_up_thresh;
        a.op.xDownThresh = (R)op.x_down_thresh;
        a.op.dxUpThresh = (R)op.dx_up_thresh;
        a.op.dxDownThresh = (R)op.dx_down_thresh;
        a.op.eps_dx = (R)op.eps_dx;
        return a;
    }

    // Members by decreasing time span (stable), so the persistent lanes take
    // the longest members first and the launch does not end on one lane
    // stepping through a long member after the rest have finished (longest
    // processing time first).  Each member's arithmetic is unchanged.
    const int *member_order()
    {
        if (!(schedule == 1 && order_by_span && tspan_per_member) || nPts <= 1)
            return nullptr;
        if (!order_valid) {
            size_t scratch = 0;
            if (single)
                order_by_span_f32(tspan_dev.as<float>(), (size_t)nPts, nullptr, nullptr, &scratch, stream);
            else
                order_by_span_f64(tspan_dev.as<double>(), (size_t)nPts, nullptr, nullptr, &scratch, stream);
            order.reserve((size_t)nPts * sizeof(int));
            order_scratch.reserve(scratch);
            if (single)
                order_by_span_f32(tspan_dev.as<float>(), (size_t)nPts, order.as<int>(), order_scratch.p, &scratch,
                                  stream);
            else
                order_by_span_f64(tspan_dev.as<double>(), (size_t)nPts, order.as<int>(), order_scratch.p, &scratch,
                                  stream);
            order_valid = true;
        }
        return order.as<int>();
    }

    // The feature pass of a two-pass observer integrates exactly the steps
    // its warm-up pass took, which counted them per member: sorting by those
    // counts gives that launch the longest-first order from the work itself
    // (a member held back by a tiny step size starts first instead of last).
    // Enqueued inside the features launch's timing; each member's arithmetic
    // is unchanged.
    const int *work_order()
    {
        size_t scratch = 0;
        order_by_count(work_counts.as<int>(), (size_t)nPts, nullptr, nullptr, &scratch, stream);
        order_work.reserve((size_t)nPts * sizeof(int));
        order_scratch.reserve(scratch);
        order_by_count(work_counts.as<int>(), (size_t)nPts, order_work.as<int>(), order_scratch.p, &scratch, stream);
        return order_work.as<int>();
    }

    // grid schedule: one thread per member.  persistent schedule: as many
    // resident blocks as the SMs hold (or blocks_per_sm per SM), lanes pull
    // members from a counter; never more threads than members.
    void launch(cudaKernel_t kgrid, cudaKernel_t kpersist, int fused_init)
    {
        if (nPts == 0)
            return;
        int sms = 0;
        check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "SM count");
        unsigned int block = (unsigned int)std::max(32, std::min(1024, block_size));
        // Few members (fewer than one block per SM at this block size): shrink
        // the block, in whole warps, until the blocks reach every SM.  Each
        // member still has its own thread; its SM's pipes serve fewer warps.
        long long active = range_end >= 0 ? std::min(range_end, nPts) : nPts;
        if (range_stride > 1)
            active = (active + range_stride - 1) / range_stride;
        if ((long long)block * sms > active) {
            const long long per_sm_members = (active + sms - 1) / std::max(sms, 1);
            const unsigned int b = (unsigned int)std::max<long long>(32, (per_sm_members + 31) / 32 * 32);
            block = std::min(block, b);
        }
        unsigned int grid = (unsigned int)((nPts + block - 1) / block);
        cudaKernel_t k = kgrid;
        if (schedule == 1 && kpersist) {
            k = kpersist;
            int per_sm = blocks_per_sm;
            if (per_sm <= 0) {
                check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *)k, (int)block, 0),
                           "occupancy query");
                per_sm = std::max(per_sm, 1);
            }
            unsigned long long want = (unsigned long long)per_sm * sms;
            grid = (unsigned int)std::min<unsigned long long>(want, grid);
            check_cuda(cudaMemsetAsync(work.p, 0, sizeof(unsigned int), stream), "work counter reset");
            if (time_budget_ms > 0.0)
                launch_fill_i32(status.as<int>(), STATUS_TIME_BUDGET, (size_t)nPts, stream);
        }
        last_grid = (int)grid;
        last_block = (int)block;
        const int *ord = k != kpersist ? nullptr : use_work_order ? work_order() : member_order();
        if (single) {
            ArgsT<float> a = make_args<float>();
            a.fused_init = fused_init;
            a.order = ord;
            void *params[] = {&a};
            check_cuda(cudaLaunchKernel((const void *)k, dim3(grid), dim3(block), params, 0, stream), "kernel launch");
            count_launch();
        } else {
            ArgsT<double> a = make_args<double>();
            a.fused_init = fused_init;
            a.order = ord;
            void *params[] = {&a};
            check_cuda(cudaLaunchKernel((const void *)k, dim3(grid), dim3(block), params, 0, stream), "kernel launch");
            count_launch();
        }
    }

    void begin_run()
    {
        ensure_built();
        ensure_stream();
        if (collect_stats && nPts > 0)
            check_cuda(cudaMemsetAsync(stats.p, 0, CLODE_STAT_COUNT * sizeof(unsigned long long), stream), "stats reset");
        check_cuda(cudaEventRecord(ev0, stream), "event record");
    }

    void end_run(const char *what)
    {
        check_cuda(cudaEventRecord(ev1, stream), "event record");
        check_cuda(cudaStreamSynchronize(stream), what);
        float ms = 0.0f;
        check_cuda(cudaEventElapsedTime(&ms, ev0, ev1), "event timing");
        last_ms = ms;
        memset(last_stats, 0, sizeof last_stats);
        if (collect_stats && nPts > 0)
            check_cuda(cudaMemcpy(last_stats, stats.p, sizeof last_stats, cudaMemcpyDeviceToHost), "stats read");
    }

    void require_problem()
    {
        if (buffers_device < 0)
            fail(CLODE_ERR_STATE, "problem data must be set before running (set_problem_data)");
    }

    void sync_tspan_device()
    {
        order_valid = false;
        if (!tspan_per_member)
            return;
        tspan_dev.reserve(std::max<size_t>(1, tspan_pm.size()) * real_size());
        upload(tspan_dev, tspan_pm.data(), tspan_pm.size());
    }

    void transient()
    {
        require_problem();
        begin_run();
        launch(k_transient, kp_transient, 0);
        end_run("transient");
        log_msg(CLODE_LOG_INFO, "run transient");
    }

    // CLODEfeatures::resizeFeaturesVariables (CLODEfeatures.cpp:143-177)
    void resize_features()
    {
        long long nf = (long long)names().size();
        long long fe = nf * nPts;
        if (fe != F_elements || obs_words != odata_words_alloc) {
            F_elements = fe;
            F.reserve(std::max<long long>(1, fe) * real_size());
            odata.reserve(std::max<size_t>(1, (size_t)obs_words * nPts) * sizeof(unsigned int));
            odata_words_alloc = obs_words;
            observer_initialized = false;
            log_msg(CLODE_LOG_DEBUG, "resize F, odata with nPts=%lld, nF=%lld", nPts, nf);
        }
    }

    void initialize_observer()
    {
        require_problem();
        if (kind != CLODE_SIM_FEATURES)
            fail(CLODE_ERR_STATE, "not a feature simulator");
        begin_run();
        resize_features();
        launch(k_init, kp_init, 0);
        end_run("initializeObserver");
        observer_initialized = true;
        log_msg(CLODE_LOG_DEBUG, "run initializeObserver");
    }

    void features(int reinit)
    {
        require_problem();
        if (kind != CLODE_SIM_FEATURES)
            fail(CLODE_ERR_STATE, "not a feature simulator");
        if (reinit >= 0)
            observer_initialized = reinit == 0;
        want_store = false;
        ensure_built();
        resize_features();
        int fused = 0;
        double init_ms = 0.0;
        unsigned long long init_stats[CLODE_STAT_COUNT] = {0};
        bool by_work = false;
        if (!observer_initialized && replay_usable() && features_replay()) {
            observer_initialized = true;
            log_msg(CLODE_LOG_DEBUG, "run features (replayed warm-up, %d recording launches, %u members by "
                                     "the plain feature pass)", last_replay_chunks, last_fallback);
            return;
        }
        if (!observer_initialized) {
            if (fuse_init) {
                fused = 1;
            } else {
                by_work = schedule == 1 && order_by_work && obs_two_pass() && nPts > 1 && kp_init != nullptr;
                if (by_work)
                    work_counts.reserve((size_t)nPts * sizeof(int));
                record_work = by_work;
                try {
                    initialize_observer();
                } catch (...) {
                    record_work = false;
                    throw;
                }
                record_work = false;
                init_ms = last_ms;
                memcpy(init_stats, last_stats, sizeof init_stats);
            }
        }
        use_work_order = by_work;
        begin_run();
        try {
            launch(k_features, kp_features, fused);
        } catch (...) {
            use_work_order = false;
            throw;
        }
        use_work_order = false;
        end_run("features");
        last_warmup_ms = init_ms;
        // time and counters of the whole call, observer initialisation included
        last_ms += init_ms;
        for (int k = 0; k < CLODE_STAT_COUNT; ++k)
            last_stats[k] += init_stats[k];
        observer_initialized = true;
        log_msg(CLODE_LOG_DEBUG, "run features");
    }


    // ------------------------------------------------ replayed warm-up --
    // A two-pass observer's feature pass integrates the trajectory its
    // warm-up pass already integrated.  With `replay` on, the warm-up launch
    // (clode_init_observer_record) also stores every step of the feature pass
    // in per-warp regions of device memory and the feature pass
    // (clode_features_replay) reads them back instead of integrating again.
    // The map runs in as many recording + replay launch pairs as the regions
    // need.  Members that the observer ends early, or that take no step,
    // run in a plain feature-pass launch at the end; members still running
    // when their warp's region filled run in plain warm-up and feature-pass
    // launches at the end.  Results are those of the separate warm-up and
    // feature launches.
    bool replay_usable() const
    {
        return replay && schedule == 1 && !fuse_init && obs_two_pass() && kp_init_rec && kp_replay && kp_features &&
               kp_init &&
               !want_store && time_budget_ms <= 0.0 && nPts > 0 && fin_words > 0 && rec_fields > 0;
    }

    // persistent grid and block of a kernel, as launch() sizes them
    void persistent_shape(cudaKernel_t k, long long active, unsigned int &grid, unsigned int &block)
    {
        int sms = 0;
        check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "SM count");
        block = (unsigned int)std::max(32, std::min(1024, block_size)) / 32 * 32;
        if ((long long)block * sms > active) {
            const long long per_sm_members = (active + sms - 1) / std::max(sms, 1);
            const unsigned int b = (unsigned int)std::max<long long>(32, (per_sm_members + 31) / 32 * 32);
            block = std::min(block, b);
        }
        int per_sm = blocks_per_sm;
        if (per_sm <= 0) {
            check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *)k, (int)block, 0),
                       "occupancy query");
            per_sm = std::max(per_sm, 1);
        }
        const unsigned long long want = (unsigned long long)per_sm * sms;
        const unsigned long long cover = ((unsigned long long)active + block - 1) / block;
        grid = (unsigned int)std::max<unsigned long long>(1, std::min(want, cover));
    }

    template <typename R>
    void launch_args(cudaKernel_t k, unsigned int grid, unsigned int block, ArgsT<R> &a, size_t smem = 0)
    {
        void *params[] = {&a};
        check_cuda(cudaLaunchKernel((const void *)k, dim3(grid), dim3(block), params, smem, stream),
                   "kernel launch");
        count_launch();
    }

    // Region geometry for `budget` bytes over `warps` warps; false when the
    // budget gives fewer than 64 rows per warp.  Grows the buffers as needed.
    bool replay_regions(double budget, unsigned long long warps, double row_bytes, size_t rs,
                        unsigned long long &rows, unsigned int &members_cap)
    {
        // regions already allocated that hold at least nine tenths of the
        // budget's rows are used as they are: freeing and re-allocating a
        // few hundred GB costs more (the next transfers wait for the unmap)
        // than the rows it would add
        if (rec.p && warps > 0) {
            const double held_rows = (double)rec.bytes / ((double)warps * (double)rec_fields * 32.0 * (double)rs);
            const double want_rows = budget / ((double)warps * (row_bytes + 0.5));
            if (want_rows > held_rows && want_rows <= 1.1 * held_rows)
                budget = held_rows * (double)warps * (row_bytes + 0.5);
        }
        rows = (unsigned long long)(budget / ((double)warps * (row_bytes + 0.5)));
        // a multiple of 16 rows: every region's masks start on a 16-byte
        // boundary, as the replay's bulk L2 prefetches require
        rows = std::min<unsigned long long>(rows, 0xfffffff0ull) & ~15ull;
        if (rows < 64)
            return false;
        members_cap = (unsigned int)std::min<unsigned long long>(rows / 8 + 64, 0x7fffffffull);
        if (rec.bytes < (size_t)(warps * rows * rec_fields * 32ull * rs))
            ++last_reallocs;
        rec.reserve((size_t)(warps * rows * rec_fields * 32ull * rs));
        rec_mask.reserve((size_t)(warps * rows * 2ull * sizeof(unsigned int)) + 16);
        rec_member.reserve((size_t)(warps * members_cap * sizeof(int)));
        return true;
    }

    // Shared-memory stages of the replay for rows of `row_bytes`: the most
    // (up to replay_stages, or 4) whose dynamic shared memory lets the
    // recording launch's blocks per SM all stay resident; 0 (rows read from
    // global memory) when fewer than 2 fit or the option is 0.  The layout
    // per warp (rows, two 128-byte mask slots, S + 2 mbarriers, rounded to
    // 16 bytes) is the replay kernel's stage_bytes.
    unsigned int replay_stage_count(unsigned int grid, unsigned int block, unsigned int row_bytes, size_t &smem)
    {
        smem = 0;
        if (replay_stages == 0 || !kp_replay_staged)
            return 0;
        int sms = 1, per_sm = 0, optin = 0;
        check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "SM count");
        check_cuda(cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, device),
                   "shared memory per SM");
        check_cuda(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device),
                   "shared memory per block");
        const unsigned long long blocks_sm = ((unsigned long long)grid + sms - 1) / std::max(sms, 1);
        const unsigned long long wpb = block / 32;
        const unsigned int want = replay_stages > 0 ? (unsigned int)std::min(replay_stages, 16) : 4u;
        for (unsigned int S = want; S >= 2; --S) {
            const unsigned long long per_warp = ((unsigned long long)S * row_bytes + 256ull + 8ull * (S + 2) + 15ull) &
                                                ~15ull;
            const unsigned long long b = wpb * per_warp;
            // 1 KiB per block is reserved by the system
            if (b <= (unsigned long long)optin && blocks_sm * (b + 1024ull) <= (unsigned long long)per_sm) {
                smem = (size_t)b;
                check_cuda(cudaFuncSetAttribute((const void *)kp_replay_staged,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)smem),
                           "replay shared memory");
                return S;
            }
        }
        return 0;
    }

    // The replay launch's shape for a recording launch of `grid` blocks of
    // `block` threads: the same number of blocks, each of block / k threads
    // whose warps take k regions in turn, for the smallest k (1, 2, 4) whose
    // blocks fit on an SM as many at a time as the recording launch's (the
    // replay's own register cap then never makes its regions wait for a
    // second wave); and its shared-memory stages at that block size.
    void replay_shape(unsigned int grid, unsigned int block, unsigned int row_bytes, unsigned int &k,
                      unsigned int &rblock, unsigned int &stages, size_t &smem)
    {
        int sms = 1;
        check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "SM count");
        const unsigned long long rec_per_sm = ((unsigned long long)grid + sms - 1) / std::max(sms, 1);
        k = 1;
        rblock = block;
        stages = 0;
        smem = 0;
        for (unsigned int kk = 1; kk <= 4; kk *= 2) {
            if (block % (32u * kk) != 0)
                break;
            const unsigned int rb = block / kk;
            size_t sm = 0;
            const unsigned int st = replay_stage_count(grid, rb, row_bytes, sm);
            int per_sm = 0;
            check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                           &per_sm, (const void *)(st >= 2 ? kp_replay_staged : kp_replay), (int)rb, sm),
                       "replay occupancy query");
            k = kk;
            rblock = rb;
            stages = st;
            smem = sm;
            if ((unsigned long long)per_sm >= rec_per_sm)
                return;
        }
    }

    // false (nothing launched) when the memory for the regions is too small
    template <typename R>
    bool replay_run(long long positions)
    {
        const bool fused = replay_fused && kp_record_replay;
        last_reallocs = 0;
        unsigned int grid = 0, block = 0;
        persistent_shape(fused ? kp_record_replay : kp_init_rec, positions, grid, block);
        const unsigned long long warps = (unsigned long long)grid * block / 32;
        const size_t rs = sizeof(R);
        // bytes per warp-wide row: every field of 32 lanes and the two masks
        const double row_bytes = (double)rec_fields * 32.0 * rs + 8.0;
        // the most the regions may take: the replay_mb option, else most of
        // the device memory that is free (counting what the regions hold now)
        double cap;
        if (replay_mb > 0.0) {
            cap = replay_mb * 1048576.0;
        } else {
            size_t fr = 0, tot = 0;
            check_cuda(cudaMemGetInfo(&fr, &tot), "cudaMemGetInfo");
            const double held = (double)(rec.bytes + rec_mask.bytes + rec_member.bytes);
            const double keep = 2.0 * 1073741824.0 + 0.02 * (double)tot;
            cap = std::max(0.0, ((double)fr + held - keep) * 0.8);
        }
        // a trial on a sample gets the sample's share, so that it runs in as
        // many launch pairs (and as many members per lane in each) as the
        // whole ensemble would
        cap *= replay_cap_scale;
        // what `members` members need at `spm` steps each (holes included), plus slack per warp
        auto need_for = [&](long long members, double spm) {
            return (double)members * spm * row_bytes / 32.0 * 1.25 + (double)warps * 256.0 * row_bytes;
        };
        // first launch: sized from the last run's steps per member, else a
        // quarter of what the regions may take (the launches after it are
        // sized from what it measured)
        double budget = replay_steps_per_member > 0.0 ? need_for(positions, replay_steps_per_member)
                                                      : std::max(1073741824.0, 0.25 * cap);
        budget = std::min(budget, cap);
        unsigned long long R_rows = 0;
        unsigned int members_cap = 0;
        if (!replay_regions(budget, warps, row_bytes, rs, R_rows, members_cap)) {
            log_msg(CLODE_LOG_INFO, "replay: %.1f MB of device memory gives fewer than 64 rows per warp; "
                                    "integrating the feature pass", budget / 1e6);
            return false;
        }
        rec_used.reserve((size_t)warps * sizeof(unsigned int));
        fin.reserve((size_t)nPts * fin_words * sizeof(unsigned int));
        fallback.reserve((size_t)nPts * sizeof(int));
        fallback_count.reserve(2 * sizeof(unsigned int));
        rec_err.reserve(sizeof(unsigned int));
        size_t stage_smem = 0;
        unsigned int stages = 0, per_warp = 1, rblock = block;
        if (!fused)
            replay_shape(grid, block, (unsigned int)(rec_fields * 32u * rs), per_warp, rblock, stages, stage_smem);
        // a warp takes no new member once its region is this full: the members
        // it holds then should still fit (replay_room times the average
        // member's steps); a larger room makes longer drains, a smaller one
        // more members cut off by a full region (run again by the plain passes)
        double spm = replay_steps_per_member;
        auto fetch_rows_for = [&](unsigned long long rows) {
            unsigned long long room = rows / 2;
            if (spm > 0.0)
                room = std::min<unsigned long long>(room, (unsigned long long)(replay_room * spm) + 64);
            return rows - room;
        };

        ArgsT<R> a = make_args<R>();
        a.fused_init = 0;
        a.order = member_order();
        a.work_out = nullptr;
        a.rec_used = rec_used.as<unsigned int>();
        a.fin = fin.as<unsigned int>();
        a.fallback = fallback.as<int>();
        a.fallback_count = fallback_count.as<unsigned int>();
        a.rec_stages = stages;
        a.rec_error = rec_err.as<unsigned int>();
        a.rec_regions_per_warp = per_warp;
        auto set_regions = [&]() {
            a.rec = rec.as<R>();
            a.rec_mask = rec_mask.as<unsigned int>();
            a.rec_member = rec_member.as<int>();
            a.rec_rows = R_rows;
            a.rec_fetch_rows = fetch_rows_for(R_rows);
            a.rec_members = members_cap;
        };
        set_regions();
        check_cuda(cudaMemsetAsync(work.p, 0, sizeof(unsigned int), stream), "work counter reset");
        check_cuda(cudaMemsetAsync(fallback_count.p, 0, 2 * sizeof(unsigned int), stream), "fallback counters reset");
        check_cuda(cudaMemsetAsync(rec_err.p, 0, sizeof(unsigned int), stream), "replay error reset");
        last_grid = (int)grid;
        last_block = (int)block;
        std::vector<unsigned int> used(warps);
        double rows_total = 0.0;
        unsigned int taken = 0, before = 0;
        int chunks = 0;
        for (cudaEvent_t &e : rev)
            if (!e)
                check_cuda(cudaEventCreate(&e), "cudaEventCreate");
        last_record_ms = last_replay_ms = last_fallback_ms = 0.0;
        auto elapsed = [&](cudaEvent_t e0, cudaEvent_t e1) {
            float ms = 0.0f;
            check_cuda(cudaEventElapsedTime(&ms, e0, e1), "event timing");
            return (double)ms;
        };
        for (;;) {
            check_cuda(cudaEventRecord(rev[0], stream), "event record");
            if (fused) {
                launch_args(kp_record_replay, grid, block, a);
                check_cuda(cudaEventRecord(rev[1], stream), "event record");
            } else {
                launch_args(kp_init_rec, grid, block, a);
                check_cuda(cudaEventRecord(rev[1], stream), "event record");
                launch_args(stages >= 2 ? kp_replay_staged : kp_replay, grid, rblock, a, stage_smem);
            }
            check_cuda(cudaEventRecord(rev[2], stream), "event record");
            ++chunks;
            check_cuda(cudaMemcpyAsync(&taken, work.p, sizeof taken, cudaMemcpyDeviceToHost, stream),
                       "work counter read");
            check_cuda(cudaMemcpyAsync(used.data(), rec_used.p, warps * sizeof(unsigned int),
                                       cudaMemcpyDeviceToHost, stream), "rows read");
            check_cuda(cudaStreamSynchronize(stream), "replay");
            last_record_ms += elapsed(rev[0], rev[1]);
            last_replay_ms += elapsed(rev[1], rev[2]);
            const long long done = std::min<long long>(taken, positions);
            if (done >= positions) {
                for (unsigned int u : used)
                    rows_total += u;
                break;
            }
            if (taken == before)
                fail(CLODE_ERR_INTERNAL, "replay: a recording launch took no member (%u of %lld)", taken, positions);
            // rows per member of this launch (holes included) estimate the rest
            double rows_used = 0.0;
            for (unsigned int u : used)
                rows_used += u;
            rows_total += rows_used;
            spm = rows_used * 32.0 / (double)(done - std::min<long long>(before, positions)) / 1.25;
            const double need = need_for(positions - done, spm);
            const double have = (double)warps * (double)R_rows * row_bytes;
            if (need > 1.05 * have && have < 0.95 * cap) {
                rec.release();
                rec_mask.release();
                rec_member.release();
                if (!replay_regions(std::min(need, cap), warps, row_bytes, rs, R_rows, members_cap))
                    fail(CLODE_ERR_OUT_OF_MEMORY, "replay: the record regions could not be regrown");
            }
            set_regions();
            before = taken;
        }
        unsigned int counts[2] = {0, 0}, err = 0;
        check_cuda(cudaMemcpyAsync(counts, fallback_count.p, sizeof counts, cudaMemcpyDeviceToHost, stream),
                   "fallback counts read");
        check_cuda(cudaMemcpyAsync(&err, rec_err.p, sizeof err, cudaMemcpyDeviceToHost, stream), "replay error read");
        check_cuda(cudaStreamSynchronize(stream), "replay");
        if (err != 0)
            fail(CLODE_ERR_INTERNAL, "replay: a shared-memory stage was not filled within its wait limit");
        const unsigned int nfb = counts[0], nrw = counts[1];
        // the plain passes over the members of a list: warm-up (when `warm`)
        // and features, persistent, in the list's order
        auto plain_passes = [&](const int *list, unsigned int count, bool warm) {
            ArgsT<R> f = make_args<R>();
            f.fused_init = 0;
            f.order = list;
            f.i_begin = 0;
            f.i_end = (int)count;
            f.i_stride = 1;
            f.work_out = nullptr;
            unsigned int g2 = 0, b2 = 0;
            if (warm) {
                persistent_shape(kp_init, (long long)count, g2, b2);
                check_cuda(cudaMemsetAsync(work.p, 0, sizeof(unsigned int), stream), "work counter reset");
                launch_args(kp_init, g2, b2, f);
            }
            persistent_shape(kp_features, (long long)count, g2, b2);
            check_cuda(cudaMemsetAsync(work.p, 0, sizeof(unsigned int), stream), "work counter reset");
            launch_args(kp_features, g2, b2, f);
        };
        if (nfb + nrw > 0) {
            if (nfb + nrw > (unsigned long long)nPts)
                fail(CLODE_ERR_INTERNAL, "replay: %u + %u fallback members of %lld", nfb, nrw, nPts);
            check_cuda(cudaEventRecord(rev[0], stream), "event record");
            if (nfb > 0)
                plain_passes(fallback.as<int>(), nfb, false);
            if (nrw > 0)
                plain_passes(fallback.as<int>() + (nPts - (long long)nrw), nrw, true);
            check_cuda(cudaEventRecord(rev[1], stream), "event record");
            check_cuda(cudaStreamSynchronize(stream), "replay fallback");
            last_fallback_ms = elapsed(rev[0], rev[1]);
        }
        last_replay_chunks = chunks;
        last_rows = rows_total;
        last_fallback = nfb + nrw;
        last_rewarm = nrw;
        last_stages = stages;
        last_regions_per_warp = per_warp;
        if (spm > 0.0)
            replay_steps_per_member = spm;
        return true;
    }

    // the replayed features run; false (nothing run) when it cannot be
    // given its memory, and the caller integrates the feature pass instead
    bool features_replay()
    {
        begin_run();
        resize_features();
        long long active = range_end >= 0 ? std::min(range_end, nPts) : nPts;
        const long long stride = range_stride > 1 ? range_stride : 1;
        const long long positions = (active + stride - 1) / stride;
        const bool ran = single ? replay_run<float>(positions) : replay_run<double>(positions);
        if (!ran) {
            last_replay_chunks = 0;
            last_fallback = 0;
            last_rewarm = 0;
            last_stages = 0;
            check_cuda(cudaStreamSynchronize(stream), "replay");
            return false;
        }
        end_run("features");
        // average steps per member of this run, to size the next one
        if (collect_stats && positions > 0)
            replay_steps_per_member = (double)last_stats[CLODE_STAT_STEPS] / (double)positions;
        return true;
    }

    // Features with storage: the feature pass of features() that also
    // stores the trajectory rows (as trajectory(): row 0 and every nout-th
    // step, rows up to max_store) and the state at each of the first
    // event_rows observer events of every member.  F, xf, dt, tf and the RNG
    // state come out as from features(); the program is the features
    // program compiled with CLODE_FEATURE_STORE.
    void features_store(int reinit, unsigned int event_rows)
    {
        require_problem();
        if (kind != CLODE_SIM_FEATURES)
            fail(CLODE_ERR_STATE, "not a feature simulator");
        if (sp.nout == 0)
            fail(CLODE_ERR_INVALID_ARGUMENT, "nout must be at least 1");
        if (reinit >= 0)
            observer_initialized = reinit == 0;
        want_store = true;
        ensure_built();
        resize_features();
        resize_trajectory();
        resize_events(event_rows);
        int fused = 0;
        double init_ms = 0.0;
        unsigned long long init_stats[CLODE_STAT_COUNT] = {0};
        bool by_work = false;
        if (!observer_initialized) {
            if (fuse_init) {
                fused = 1;
            } else {
                by_work = schedule == 1 && order_by_work && obs_two_pass() && nPts > 1 && kp_init != nullptr;
                if (by_work)
                    work_counts.reserve((size_t)nPts * sizeof(int));
                record_work = by_work;
                try {
                    initialize_observer();
                } catch (...) {
                    record_work = false;
                    throw;
                }
                record_work = false;
                init_ms = last_ms;
                memcpy(init_stats, last_stats, sizeof init_stats);
            }
        }
        use_work_order = by_work;
        begin_run();
        try {
            launch(k_features, kp_features, fused);
        } catch (...) {
            use_work_order = false;
            throw;
        }
        use_work_order = false;
        end_run("features with storage");
        last_ms += init_ms;
        for (int k = 0; k < CLODE_STAT_COUNT; ++k)
            last_stats[k] += init_stats[k];
        observer_initialized = true;
        events_valid = true;
        log_msg(CLODE_LOG_DEBUG, "run features with storage");
    }

    // CLODEtrajectory::resizeTrajectoryVariables (CLODEtrajectory.cpp:45-94)
    void resize_trajectory()
    {
        long long rows = (long long)sp.max_store + 1;  // the kernel may write row max_store
        const int nv = store_nv(), na = store_na();
        const long long width = 1 + 2 * nv + na;
        if (rows == traj_rows && nPts == traj_pts && width == traj_width)
            return;
        size_t rs = real_size();
        double need = (double)rows * nPts * width * rs;
        size_t free_b = 0, total_b = 0;
        cudaMemGetInfo(&free_b, &total_b);
        if (need > (double)free_b) {
            long long max_rows = (long long)(free_b / ((double)nPts * width * rs));
            log_msg(CLODE_LOG_ERR,
                    "Storage requested exceeds device memory. Try reducing storage to <%lld time points, or reducing nPts.",
                    max_rows);
            fail(CLODE_ERR_OUT_OF_MEMORY, "trajectory storage of %.2f GB exceeds free device memory (%.2f GB)",
                 need / 1e9, free_b / 1e9);
        }
        t.reserve(std::max<size_t>(1, rows * nPts) * rs);
        x.reserve(std::max<size_t>(1, rows * nPts * nv) * rs);
        dx.reserve(std::max<size_t>(1, rows * nPts * nv) * rs);
        aux.reserve(std::max<size_t>(1, rows * nPts * std::max(na, 1)) * rs);
        nstored.reserve(std::max<size_t>(1, nPts) * sizeof(int));
        // rows a run does not reach read as zero after a resize, as in a
        // freshly created buffer, not as whatever the memory held before
        ensure_stream();
        check_cuda(cudaMemsetAsync(t.p, 0, (size_t)rows * nPts * rs, stream), "trajectory clear");
        check_cuda(cudaMemsetAsync(x.p, 0, (size_t)rows * nPts * nv * rs, stream), "trajectory clear");
        check_cuda(cudaMemsetAsync(dx.p, 0, (size_t)rows * nPts * nv * rs, stream), "trajectory clear");
        if (na > 0)
            check_cuda(cudaMemsetAsync(aux.p, 0, (size_t)rows * nPts * na * rs, stream), "trajectory clear");
        check_cuda(cudaMemsetAsync(nstored.p, 0, (size_t)nPts * sizeof(int), stream), "trajectory clear");
        traj_rows = rows;
        traj_pts = nPts;
        traj_width = width;
    }

    // event store of features with storage: ev_rows rows of (t, x, dx, aux)
    void resize_events(unsigned int rows)
    {
        const int nv = store_nv(), na = store_na();
        const long long width = 1 + 2 * nv + na;
        ensure_stream();
        if ((long long)rows != ev_rows_alloc || nPts != ev_pts || width != ev_width) {
            size_t rs = real_size();
            ev_t.reserve(std::max<size_t>(1, (size_t)rows * nPts) * rs);
            ev_x.reserve(std::max<size_t>(1, (size_t)rows * nPts * nv) * rs);
            ev_dx.reserve(std::max<size_t>(1, (size_t)rows * nPts * nv) * rs);
            ev_aux.reserve(std::max<size_t>(1, (size_t)rows * nPts * std::max(na, 1)) * rs);
            nevents.reserve(std::max<size_t>(1, nPts) * sizeof(int));
            ev_rows_alloc = rows;
            ev_pts = nPts;
            ev_width = width;
        }
        // rows a member does not reach read as zero
        size_t rs = real_size();
        check_cuda(cudaMemsetAsync(ev_t.p, 0, (size_t)rows * nPts * rs, stream), "event store clear");
        check_cuda(cudaMemsetAsync(ev_x.p, 0, (size_t)rows * nPts * nv * rs, stream), "event store clear");
        check_cuda(cudaMemsetAsync(ev_dx.p, 0, (size_t)rows * nPts * nv * rs, stream), "event store clear");
        if (na > 0)
            check_cuda(cudaMemsetAsync(ev_aux.p, 0, (size_t)rows * nPts * na * rs, stream), "event store clear");
        ev_rows = rows;
    }

    // The deviates of a stochastic trajectory run, drawn before it (the
    // count and draw launches of clode_kernels.cuh); false (nothing drawn)
    // when their buffer would take more than half the free device memory,
    // and the trajectory launch draws them itself.
    template <typename R>
    bool predraw_run()
    {
        noise_count.reserve((size_t)nPts * sizeof(unsigned int));
        for (cudaEvent_t &e : rev)
            if (!e)
                check_cuda(cudaEventCreate(&e), "cudaEventCreate");
        ArgsT<R> a = make_args<R>();
        a.noise_count = noise_count.as<unsigned int>();
        check_cuda(cudaEventRecord(rev[0], stream), "event record");
        launch_args(k_noise_count, (unsigned int)((nPts + 255) / 256), 256, a);
        std::vector<unsigned int> counts((size_t)nPts);
        check_cuda(cudaMemcpyAsync(counts.data(), noise_count.p, counts.size() * sizeof(unsigned int),
                                   cudaMemcpyDeviceToHost, stream),
                   "deviate counts read");
        check_cuda(cudaStreamSynchronize(stream), "deviate counts");
        unsigned long long most = 0;
        for (unsigned int c : counts)
            most = std::max<unsigned long long>(most, c);
        const unsigned long long pairs = (most + 1) / 2;
        if (pairs == 0)
            return false;
        const unsigned long long stride = (2 * pairs + 3) & ~3ull;
        const double bytes = (double)nPts * (double)stride * (double)sizeof(R);
        size_t fr = 0, tot = 0;
        check_cuda(cudaMemGetInfo(&fr, &tot), "cudaMemGetInfo");
        if (bytes > 0.5 * ((double)fr + (double)noise.bytes)) {
            log_msg(CLODE_LOG_INFO, "pre-drawn deviates: %.1f GB exceed half the free device memory; drawing "
                                    "them in the trajectory launch", bytes / 1e9);
            noise.release();
            return false;
        }
        noise.reserve((size_t)bytes);
        // candidates per lane and round: about 16 rounds for the member that
        // takes the most (4 lanes, 0.785 of the candidates accepted), 32 to 512
        unsigned int block = (unsigned int)std::min<unsigned long long>(
            512, std::max<unsigned long long>(32, (unsigned long long)((double)pairs / (4 * 0.785 * 16)) + 1));
        block = (block + 31) / 32 * 32;
        if (block != mats_block) {
            // lane l starts l blocks (2 draws a candidate) into the stream; a round moves 4 blocks on
            std::vector<uint64_t> m(4 * 256);
            for (int l = 1; l <= 4; ++l) {
                const Gf2Mat j = gf2_jump(2ull * block * (unsigned long long)l);
                memcpy(&m[(size_t)(l - 1) * 256], j.col, sizeof j.col);
            }
            noise_mats.reserve(m.size() * sizeof(uint64_t));
            check_cuda(cudaMemcpyAsync(noise_mats.p, m.data(), m.size() * sizeof(uint64_t), cudaMemcpyHostToDevice,
                                       stream),
                       "jump matrices upload");
            check_cuda(cudaStreamSynchronize(stream), "jump matrices upload");
            mats_block = block;
        }
        a.noise = noise.as<R>();
        a.noise_stride = stride;
        a.noise_mats = noise_mats.as<unsigned long long>();
        a.noise_block = block;
        check_cuda(cudaEventRecord(rev[1], stream), "event record");
        launch_args(k_noise_draw, (unsigned int)((nPts * 4 + 127) / 128), 128, a);
        check_cuda(cudaEventRecord(rev[2], stream), "event record");
        noise_stride = stride;
        return true;
    }

    void trajectory()
    {
        require_problem();
        if (sp.nout == 0)
            fail(CLODE_ERR_INVALID_ARGUMENT, "solver parameter nout must be at least 1");
        ensure_built();
        ensure_stream();
        resize_trajectory();
        begin_run();
        last_predrawn = false;
        if (predraw && k_noise_draw && nWiener > 0 && time_budget_ms <= 0.0 && nPts > 0)
            last_predrawn = single ? predraw_run<float>() : predraw_run<double>();
        noise_on = last_predrawn;
        try {
            launch(k_trajectory, kp_trajectory, 0);
        } catch (...) {
            noise_on = false;
            throw;
        }
        noise_on = false;
        end_run("trajectory");
        last_draw_ms = 0.0;
        if (last_predrawn) {
            float c = 0.0f, d = 0.0f;
            check_cuda(cudaEventElapsedTime(&c, rev[0], rev[1]), "event timing");
            check_cuda(cudaEventElapsedTime(&d, rev[1], rev[2]), "event timing");
            last_draw_ms = (double)c + (double)d;
        }
        log_msg(CLODE_LOG_DEBUG, "run trajectory%s", last_predrawn ? " (pre-drawn deviates)" : "");
    }

    // Chains: a sequence of runs enqueued back to back on the stream with one
    // synchronisation at the end, optionally captured once as a CUDA graph and
    // replayed.  Each op behaves as the API call of the same name (the first
    // features op of an uninitialised observer runs the initialisation in its
    // launch).  A graph is re-captured when the ops, the ensemble, the time
    // span, the options or the observer's initialisation state change.
    cudaGraphExec_t chain_graph = nullptr;
    std::string chain_key;
    unsigned long long chain_kernels = 0;

    void enqueue_op(int op, bool &obs_init)
    {
        switch (op) {
        case CLODE_OP_TRANSIENT:
            launch(k_transient, kp_transient, 0);
            break;
        case CLODE_OP_FEATURES:
            if (kind != CLODE_SIM_FEATURES)
                fail(CLODE_ERR_STATE, "features op on a simulator that is not a feature simulator");
            if (!obs_init && !fuse_init)
                launch(k_init, kp_init, 0);
            launch(k_features, kp_features, obs_init || !fuse_init ? 0 : 1);
            obs_init = true;
            break;
        case CLODE_OP_TRAJECTORY:
            if (sp.nout == 0)
                fail(CLODE_ERR_INVALID_ARGUMENT, "solver parameter nout must be at least 1");
            launch(k_trajectory, kp_trajectory, 0);
            break;
        case CLODE_OP_SHIFT_X0:
            check_cuda(cudaMemcpyAsync(x0.p, xf.p, (size_t)nPts * nVar * real_size(), cudaMemcpyDeviceToDevice,
                                       stream),
                       "shift x0");
            break;
        default:
            fail(CLODE_ERR_INVALID_ARGUMENT, "unknown chain op %d", op);
        }
    }

    void chain(const int *ops, int n, bool use_graph)
    {
        require_problem();
        want_store = false;  // chained features ops run the plain program
        ensure_built();
        ensure_stream();
        for (int k = 0; k < n; ++k) {  // every allocation happens before any capture
            if (ops[k] == CLODE_OP_FEATURES && kind == CLODE_SIM_FEATURES)
                resize_features();
            if (ops[k] == CLODE_OP_TRAJECTORY)
                resize_trajectory();
        }
        member_order();  // uploaded before any capture; replays read it in place
        bool obs_init = observer_initialized;
        if (collect_stats && nPts > 0)
            check_cuda(cudaMemsetAsync(stats.p, 0, CLODE_STAT_COUNT * sizeof(unsigned long long), stream),
                       "stats reset");
        check_cuda(cudaEventRecord(ev0, stream), "event record");
        if (use_graph) {
            std::ostringstream key;
            key << built_key << "|" << nPts << "|" << tspan[0] << "," << tspan[1] << "|" << tspan_per_member << "|"
                << schedule << "," << block_size << "," << blocks_per_sm << "," << time_budget_ms << "," << fuse_init
                << "," << order_by_span
                << "|" << obs_init
                << "|" << collect_stats << "|" << sp.dt << "," << sp.dtmax << "," << sp.abstol << "," << sp.reltol
                << "," << sp.max_steps << "," << sp.max_store << "," << sp.nout << "|" << op.e_var_ix << ","
                << op.f_var_ix << "," << op.max_event_count << "," << op.nhood_radius << "," << op.x_up_thresh << ","
                << op.x_down_thresh << "," << op.dx_up_thresh << "," << op.dx_down_thresh << "," << op.min_x_amp
                << "|";
            for (int k = 0; k < n; ++k)
                key << ops[k] << ",";
            bool fresh_capture = !chain_graph || chain_key != key.str();
            if (fresh_capture) {
                if (chain_graph) {
                    cudaGraphExecDestroy(chain_graph);
                    chain_graph = nullptr;
                }
                unsigned long long before = clode_launch_count();
                // capture between the two timing events: the graph holds the ops only
                check_cuda(cudaStreamSynchronize(stream), "chain capture");
                cudaGraph_t g;
                check_cuda(cudaStreamBeginCapture(stream, cudaStreamCaptureModeRelaxed), "chain capture");
                bool cap_init = obs_init;
                try {
                    for (int k = 0; k < n; ++k)
                        enqueue_op(ops[k], cap_init);
                } catch (...) {
                    cudaStreamEndCapture(stream, &g);
                    if (g)
                        cudaGraphDestroy(g);
                    throw;
                }
                check_cuda(cudaStreamEndCapture(stream, &g), "chain capture");
                check_cuda(cudaGraphInstantiate(&chain_graph, g, 0), "chain graph instantiate");
                cudaGraphDestroy(g);
                chain_key = key.str();
                // the kernels counted while capturing are the ones this first replay runs
                chain_kernels = clode_launch_count() - before;
            } else {
                for (unsigned long long k = 0; k < chain_kernels; ++k)
                    count_launch();
            }
            check_cuda(cudaGraphLaunch(chain_graph, stream), "chain graph launch");
            for (int k = 0; k < n; ++k)
                if (ops[k] == CLODE_OP_FEATURES)
                    obs_init = true;
        } else {
            for (int k = 0; k < n; ++k)
                enqueue_op(ops[k], obs_init);
        }
        end_run("chain");
        observer_initialized = obs_init;
    }

    // Autotuner: for each (register cap, block size) candidate, build the
    // program (later builds come from the on-disk cache) and time the
    // persistent kernel of this simulator's kind on members [0, sample).
    // The sampled members' dt and RNG words are restored after every trial;
    // their other outputs are recomputed by the next run, and the observer is
    // re-initialised.  Keeps the fastest candidate and the persistent schedule.
    void autotune(long long sample, double *best_ms_out)
    {
        require_problem();
        want_store = false;  // tunes (and leaves loaded) the plain program
        long long S = std::min(nPts, sample > 0 ? sample : nPts);
        if (S <= 0)
            fail(CLODE_ERR_STATE, "no members to tune on");
        // a strided sample over the whole ensemble (members 0, k, 2k, ...),
        // so that it sees every part of a parameter map
        const int stride = (int)std::max<long long>(1, nPts / S);
        const int cands[][2] = {{0, 128}, {128, 128}, {96, 128}, {80, 128}, {64, 128}, {96, 64}, {80, 64}};
        size_t rs = real_size();
        DevBuf save_dt, save_rng;
        save_dt.reserve((size_t)nPts * rs);
        save_rng.reserve((size_t)nPts * 2 * sizeof(unsigned long long));
        ensure_stream();
        auto snapshot = [&](bool restore) {
            auto cp = [&](void *dst, const void *src, size_t b) {
                check_cuda(cudaMemcpyAsync(dst, src, b, cudaMemcpyDeviceToDevice, stream), "autotune copy");
            };
            if (!restore) {
                cp(save_dt.p, dt.p, (size_t)nPts * rs);
                cp(save_rng.p, rng.p, (size_t)nPts * 2 * sizeof(unsigned long long));
            } else {
                cp(dt.p, save_dt.p, (size_t)nPts * rs);
                cp(rng.p, save_rng.p, (size_t)nPts * 2 * sizeof(unsigned long long));
            }
        };
        snapshot(false);
        // one timed run of the sample, then its dt and RNG words restored
        auto run_trial = [&]() {
            if (kind == CLODE_SIM_FEATURES && !fuse_init && (ensure_built(), replay_usable()) && features_replay()) {
                // the path features() takes for this configuration
                snapshot(true);
                check_cuda(cudaStreamSynchronize(stream), "autotune restore");
                return;
            }
            if (kind == CLODE_SIM_FEATURES) {
                resize_features();
                begin_run();
                if (fuse_init) {
                    launch(k_features, kp_features, 1);
                } else {
                    launch(k_init, kp_init, 0);
                    launch(k_features, kp_features, 0);
                }
            } else if (kind == CLODE_SIM_TRAJECTORY) {
                resize_trajectory();
                begin_run();
                launch(k_trajectory, kp_trajectory, 0);
            } else {
                begin_run();
                launch(k_transient, kp_transient, 0);
            }
            end_run("autotune trial");
            snapshot(true);
            check_cuda(cudaStreamSynchronize(stream), "autotune restore");
        };
        // trials run on the strided sample; the full range is restored on any exit
        struct SampleRange {
            clode_sim *sim;
            SampleRange(clode_sim *s, int stride) : sim(s)
            {
                sim->range_end = sim->nPts;
                sim->range_stride = stride;
                sim->replay_cap_scale = (double)((sim->nPts + stride - 1) / stride) / (double)sim->nPts;
            }
            ~SampleRange()
            {
                sim->range_end = -1;
                sim->range_stride = 1;
                sim->replay_cap_scale = 1.0;
            }
        } sample_range(this, stride);
        double best = 1e300;
        int best_regs = maxrregcount, best_block = block_size;
        schedule = 1;
        ensure_built();
        run_trial();  // untimed: buffers (and the replay's regions) allocated before the timed trials
        // register cap and block size for each stepping variant (adaptive
        // steppers: whole steps or one attempt per iteration) and, where they
        // apply (FP32 Dormand-Prince builds with contraction), paired or
        // scalar stage sums: the best cap differs between them, and whether
        // pairing pays depends on the model (it costs register moves and
        // longer dependent chains that a cheap right-hand side does not hide)
        const bool adaptive = stepper_adaptive();
        bool best_split = split_attempts;
        bool best_paired = paired;
        const bool pair_choice = pairing_applies();
        for (int pv = 0; pv < (pair_choice ? 2 : 1); ++pv) {
            const bool pd = pair_choice ? pv == 0 : paired;
            if (pd != paired) {
                paired = pd;
                built = false;
            }
            for (int variant = 0; variant < (adaptive ? 2 : 1); ++variant) {
                const bool sa = adaptive ? variant == 1 : split_attempts;
                if (sa != split_attempts) {
                    split_attempts = sa;
                    built = false;
                }
                for (auto &cd : cands) {
                    if (maxrregcount != cd[0]) {
                        maxrregcount = cd[0];
                        built = false;
                    }
                    block_size = cd[1];
                    ensure_built();
                    run_trial();
                    log_msg(CLODE_LOG_INFO, "autotune: paired=%d split_attempts=%d maxrregcount=%d block=%d: %.3f ms",
                            (int)pd, (int)sa, cd[0], cd[1], last_ms);
                    if (last_ms < best) {
                        best = last_ms;
                        best_regs = cd[0];
                        best_block = cd[1];
                        best_split = sa;
                        best_paired = pd;
                    }
                }
            }
        }
        if (maxrregcount != best_regs || split_attempts != best_split || paired != best_paired) {
            maxrregcount = best_regs;
            split_attempts = best_split;
            paired = best_paired;
            built = false;
        }
        block_size = best_block;
        // replayed or integrated feature pass (two-pass observers, separate passes)
        if (kind == CLODE_SIM_FEATURES && obs_two_pass() && !fuse_init) {
            ensure_built();
            const bool base_replay = replay;
            replay = !base_replay;
            try {
                run_trial();
            } catch (...) {
                replay = base_replay;
                throw;
            }
            log_msg(CLODE_LOG_INFO, "autotune: replay=%d: %.3f ms", (int)replay, last_ms);
            if (last_ms < best)
                best = last_ms;
            else
                replay = base_replay;
            // the replay's row layout (a rebuild) and its launch layout
            if (replay) {
                const bool base_split = replay_split;
                replay_split = !base_split;
                built = false;
                try {
                    ensure_built();
                    run_trial();
                } catch (...) {
                    replay_split = base_split;
                    built = false;
                    throw;
                }
                log_msg(CLODE_LOG_INFO, "autotune: replay_split=%d: %.3f ms", (int)replay_split, last_ms);
                if (last_ms < best) {
                    best = last_ms;
                } else {
                    replay_split = base_split;
                    built = false;
                    ensure_built();
                }
                const bool base_fused = replay_fused;
                replay_fused = !base_fused;
                run_trial();
                log_msg(CLODE_LOG_INFO, "autotune: replay_fused=%d: %.3f ms", (int)replay_fused, last_ms);
                if (last_ms < best)
                    best = last_ms;
                else
                    replay_fused = base_fused;
            }
        }
        // fused or separate observer initialisation (two-pass observers)
        if (kind == CLODE_SIM_FEATURES && obs_two_pass()) {
            ensure_built();
            const bool base_fuse = fuse_init;
            fuse_init = !base_fuse;
            try {
                run_trial();
            } catch (...) {
                fuse_init = base_fuse;
                throw;
            }
            log_msg(CLODE_LOG_INFO, "autotune: fuse_init=%d: %.3f ms", (int)fuse_init, last_ms);
            if (last_ms < best)
                best = last_ms;
            else
                fuse_init = base_fuse;
        }
        observer_initialized = false;
        ensure_built();
        if (best_ms_out)
            *best_ms_out = best;
    }

    void shift_x0()
    {
        require_problem();
        ensure_stream();
        check_cuda(cudaMemcpyAsync(x0.p, xf.p, (size_t)nPts * nVar * real_size(), cudaMemcpyDeviceToDevice, stream),
                   "shift x0");
        check_cuda(cudaStreamSynchronize(stream), "shift x0");
    }

    void shift_tspan()
    {
        if (tspan_per_member) {
            for (size_t i = 0; i + 1 < tspan_pm.size(); i += 2) {
                double a = tspan_pm[i], b = tspan_pm[i + 1];
                tspan_pm[i] = b;
                tspan_pm[i + 1] = b + (b - a);
            }
            ensure_stream();
            sync_tspan_device();
        } else {
            double a = tspan[0], b = tspan[1];
            tspan[0] = b;
            tspan[1] = b + (b - a);
        }
    }

    // --------------------------------------------------------- getters --
    size_t array_len(int which) const
    {
        switch (which) {
        case CLODE_ARRAY_X0:
        case CLODE_ARRAY_XF: return (size_t)nPts * nVar;
        case CLODE_ARRAY_DT:
        case CLODE_ARRAY_TF: return (size_t)nPts;
        case CLODE_ARRAY_PARS: return pars_host.size();
        case CLODE_ARRAY_TSPAN: return tspan_per_member ? tspan_pm.size() : 2;
        case CLODE_ARRAY_F: return F_elements > 0 ? (size_t)F_elements : 0;
        case CLODE_ARRAY_T: return traj_rows > 0 ? stored_rows() * nPts : 0;
        case CLODE_ARRAY_X:
        case CLODE_ARRAY_DX: return traj_rows > 0 ? stored_rows() * nPts * store_nv() : 0;
        case CLODE_ARRAY_AUX: return traj_rows > 0 ? (store_na() > 0 ? stored_rows() * nPts * store_na() : 1) : 0;
        case CLODE_ARRAY_EVENT_T: return events_valid ? (size_t)ev_rows * nPts : 0;
        case CLODE_ARRAY_EVENT_X:
        case CLODE_ARRAY_EVENT_DX: return events_valid ? (size_t)ev_rows * nPts * store_nv() : 0;
        case CLODE_ARRAY_EVENT_AUX: return events_valid ? (size_t)ev_rows * nPts * store_na() : 0;
        }
        fail(CLODE_ERR_INVALID_ARGUMENT, "unknown array id %d", which);
    }

    void get(int which, double *out, size_t n)
    {
        if (which == CLODE_ARRAY_PARS) {
            std::copy(pars_host.begin(), pars_host.begin() + n, out);
            return;
        }
        if (which == CLODE_ARRAY_TSPAN) {
            if (tspan_per_member)
                std::copy(tspan_pm.begin(), tspan_pm.begin() + n, out);
            else
                std::copy(tspan, tspan + n, out);
            return;
        }
        if (n == 0)
            return;
        ensure_stream();
        DevBuf *src = nullptr;
        switch (which) {
        case CLODE_ARRAY_X0: src = &x0; break;
        case CLODE_ARRAY_XF: src = &xf; break;
        case CLODE_ARRAY_DT: src = &dt; break;
        case CLODE_ARRAY_TF: src = &tf; break;
        case CLODE_ARRAY_F: src = &F; break;
        case CLODE_ARRAY_T: src = &t; break;
        case CLODE_ARRAY_X: src = &x; break;
        case CLODE_ARRAY_DX: src = &dx; break;
        case CLODE_ARRAY_AUX:
            if (store_na() == 0) {
                out[0] = 0.0;
                return;
            }
            src = &aux;
            break;
        case CLODE_ARRAY_EVENT_T: src = &ev_t; break;
        case CLODE_ARRAY_EVENT_X: src = &ev_x; break;
        case CLODE_ARRAY_EVENT_DX: src = &ev_dx; break;
        case CLODE_ARRAY_EVENT_AUX: src = &ev_aux; break;
        }
        download(*src, out, n);
    }

    // Rows [0, rows) of members [first, first + count) of the last
    // trajectory (events == false) or of the last run's event states
    // (events == true), regrouped member-major on the device (one transpose
    // per stored array, see launch_regroup_by_member_*) and copied out in
    // chunks of at most 256 MB of staging.  Null outputs are skipped.
    void get_by_member(bool events, long long first, long long count, long long rows, double *t_out, double *x_out,
                       double *dx_out, double *aux_out, int *counts_out)
    {
        if (events ? !events_valid : traj_rows <= 0)
            fail(CLODE_ERR_INVALID_ARGUMENT, events ? "no run has stored event states" : "no trajectory has been run");
        if (first < 0 || count < 0 || first + count > nPts)
            fail(CLODE_ERR_INVALID_ARGUMENT, "members [%lld, %lld) are outside [0, %lld)", first, first + count,
                 nPts);
        const size_t max_rows = events ? (size_t)ev_rows : stored_rows();
        if (rows < 0 || rows > (long long)max_rows)
            fail(CLODE_ERR_INVALID_ARGUMENT, "rows = %lld is outside [0, %zu] (rows of the stored run)", rows,
                 max_rows);
        if (!count)
            return;
        ensure_stream();
        if (counts_out)
            check_cuda(cudaMemcpyAsync(counts_out, (events ? nevents : nstored).as<int>() + first,
                                       (size_t)count * sizeof(int), cudaMemcpyDeviceToHost, stream),
                       "D2H copy");
        struct Part {
            const DevBuf *src;
            double *out;
            size_t width;
        } parts[4] = {{events ? &ev_t : &t, t_out, 1},
                      {events ? &ev_x : &x, x_out, (size_t)store_nv()},
                      {events ? &ev_dx : &dx, dx_out, (size_t)store_nv()},
                      {events ? &ev_aux : &aux, aux_out, (size_t)store_na()}};
        const size_t stage_max = (size_t)256 << 20;
        for (const Part &p : parts) {
            if (!p.out || p.width == 0 || rows == 0)
                continue;
            const size_t nc = (size_t)rows * p.width, per_member = nc * sizeof(double);
            const size_t chunk = std::max<size_t>(1, std::min<size_t>((size_t)count, stage_max / per_member));
            stage.reserve(chunk * per_member);
            HostPin pin(p.out, (size_t)count * per_member);
            for (size_t m = 0; m < (size_t)count; m += chunk) {
                const size_t nm = std::min<size_t>(chunk, (size_t)count - m);
                if (single)
                    launch_regroup_by_member_f32(p.src->as<float>(), (size_t)nPts, (size_t)first + m, nm, nc,
                                                 stage.as<double>(), stream);
                else
                    launch_regroup_by_member_f64(p.src->as<double>(), (size_t)nPts, (size_t)first + m, nm, nc,
                                                 stage.as<double>(), stream);
                check_cuda(cudaMemcpyAsync(p.out + m * nc, stage.p, nm * per_member, cudaMemcpyDeviceToHost, stream),
                           "D2H copy");
            }
            check_cuda(cudaStreamSynchronize(stream), "D2H copy");  // before the range is unpinned
        }
        check_cuda(cudaStreamSynchronize(stream), "D2H copy");
    }

    std::string status_report() const
    {
        std::ostringstream s;
        s << "------------------\n   " << rhs_name << "\n   nVar=" << nVar << "\n   nPar=" << nPar
          << "\n   nAux=" << nAux << "\n   nWiener=" << nWiener << "\nUsing " << (single ? "single" : "double")
          << " precision.\nUsing stepper: " << stepper << "\n";
        if (kind == CLODE_SIM_FEATURES)
            s << "Using observer: " << observer << "\n";
        return s.str();
    }
};

// ==================================================================== C ABI
namespace {

int set_error(int code, const std::string &msg)
{
    g_last_error = msg;
    log_msg(CLODE_LOG_DEBUG, "error %d: %s", code, msg.c_str());
    return code;
}

template <typename F>
int guard(F &&f)
{
    try {
        f();
        g_last_error.clear();
        return CLODE_OK;
    } catch (const Error &e) {
        return set_error(e.code, e.what());
    } catch (const std::bad_alloc &) {
        return set_error(CLODE_ERR_OUT_OF_MEMORY, "host allocation failed");
    } catch (const std::exception &e) {
        return set_error(CLODE_ERR_INTERNAL, e.what());
    }
}

void need(const void *p, const char *what)
{
    if (!p)
        fail(CLODE_ERR_INVALID_ARGUMENT, "%s must not be NULL", what);
}

void copy_string(const std::string &s, char *buf, size_t cap, size_t *n)
{
    if (n)
        *n = s.size();
    if (buf && cap) {
        size_t k = std::min(cap - 1, s.size());
        memcpy(buf, s.data(), k);
        buf[k] = 0;
    }
}

std::string join(const std::vector<std::string> &v)
{
    std::string s;
    for (size_t i = 0; i < v.size(); ++i) {
        if (i)
            s += "\n";
        s += v[i];
    }
    return s;
}

}  // namespace

extern "C" {

const char *clode_last_error(void) { return g_last_error.c_str(); }

int clode_version(void) { return CLODE_GB300_VERSION; }

int clode_device_count(int *count)
{
    return guard([&] {
        need(count, "count");
        *count = device_count_or_zero();
    });
}

int clode_device_query(int ordinal, clode_device_info *out)
{
    return guard([&] {
        need(out, "out");
        int n = device_count_or_zero();
        if (ordinal < 0 || ordinal >= n)
            fail(CLODE_ERR_NO_DEVICE, "CUDA device %d does not exist (%d present)", ordinal, n);
        cudaDeviceProp p;
        check_cuda(cudaGetDeviceProperties(&p, ordinal), "cudaGetDeviceProperties");
        memset(out, 0, sizeof *out);
        snprintf(out->name, sizeof out->name, "%s", p.name);
        snprintf(out->vendor, sizeof out->vendor, "NVIDIA Corporation");
        int rt = 0, drv = 0;
        cudaRuntimeGetVersion(&rt);
        cudaDriverGetVersion(&drv);
        snprintf(out->version, sizeof out->version, "CUDA %d.%d (driver %d.%d)", rt / 1000, (rt % 1000) / 10,
                 drv / 1000, (drv % 1000) / 10);
        out->ordinal = ordinal;
        out->compute_units = p.multiProcessorCount;
        out->cc_major = p.major;
        out->cc_minor = p.minor;
        int khz = 0;
        cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, ordinal);
        out->max_clock_mhz = khz / 1000;
        out->max_work_group_size = p.maxThreadsPerBlock;
        out->double_support = 1;
        out->device_memory_size = p.totalGlobalMem;
        out->max_memory_alloc_size = p.totalGlobalMem;
    });
}

int clode_set_cache_dir(const char *dir)
{
    return guard([&] { set_cache_dir(dir ? dir : ""); });
}

int clode_sim_create(int kind, const clode_problem *prob, const char *stepper, const char *observer,
                     const clode_observer_params *op, int single_precision, int device, clode_sim **out)
{
    return guard([&] {
        need(out, "out");
        *out = nullptr;
        if (kind < CLODE_SIM_BASE || kind > CLODE_SIM_TRAJECTORY)
            fail(CLODE_ERR_INVALID_ARGUMENT, "unknown simulator kind %d", kind);
        std::unique_ptr<clode_sim> s(new clode_sim());
        s->kind = kind;
        s->set_problem(prob);
        s->set_stepper(stepper);
        if (s->stepper.empty())
            fail(CLODE_ERR_INVALID_ARGUMENT, "Unknown stepper: %s", stepper ? stepper : "(null)");
        s->single = single_precision != 0;
        s->device = device;
        if (kind == CLODE_SIM_FEATURES) {
            if (op)
                s->op = *op;
            s->set_observer(observer);
            if (s->observer.empty())
                fail(CLODE_ERR_INVALID_ARGUMENT, "unknown observer: %s", observer ? observer : "(null)");
        }
        *out = s.release();
    });
}

int clode_sim_destroy(clode_sim *sim)
{
    return guard([&] { delete sim; });
}

#define SIM_GUARD(body)                 \
    return guard([&] {                  \
        need(sim, "sim");               \
        body;                           \
    })

int clode_sim_set_problem_info(clode_sim *sim, const clode_problem *prob) { SIM_GUARD(sim->set_problem(prob)); }
int clode_sim_set_stepper(clode_sim *sim, const char *stepper) { SIM_GUARD(sim->set_stepper(stepper)); }
int clode_sim_set_precision(clode_sim *sim, int single_precision)
{
    SIM_GUARD({
        if ((single_precision != 0) != sim->single) {
            sim->single = single_precision != 0;
            sim->built = false;
            sim->nPts = -1;  // device buffers are re-made at the next set_problem_data
        }
    });
}
int clode_sim_set_device(clode_sim *sim, int device)
{
    SIM_GUARD({
        if (device != sim->device) {
            sim->device = device;
            sim->built = false;
            sim->nPts = -1;
        }
    });
}
int clode_sim_set_observer(clode_sim *sim, const char *observer)
{
    SIM_GUARD({
        if (sim->kind != CLODE_SIM_FEATURES)
            fail(CLODE_ERR_STATE, "not a feature simulator");
        sim->set_observer(observer);
    });
}
int clode_sim_build(clode_sim *sim)
{
    SIM_GUARD({
        sim->want_store = false;  // the plain program (CLODE::buildCL); features_store builds its own
        sim->build();
    });
}

int clode_sim_set_problem_data(clode_sim *sim, const double *x0, size_t n_x0, const double *pars, size_t n_pars)
{
    SIM_GUARD({
        if (n_x0)
            need(x0, "x0");
        if (n_pars)
            need(pars, "pars");
        sim->set_problem_data(x0, n_x0, pars, n_pars);
    });
}
int clode_sim_set_x0(clode_sim *sim, const double *x0, size_t n)
{
    SIM_GUARD({
        if (n)
            need(x0, "x0");
        sim->set_x0(x0, n);
    });
}
int clode_sim_set_pars(clode_sim *sim, const double *pars, size_t n)
{
    SIM_GUARD({
        if (n)
            need(pars, "pars");
        sim->set_pars(pars, n);
    });
}
int clode_sim_set_tspan(clode_sim *sim, const double *tspan2)
{
    SIM_GUARD({
        need(tspan2, "tspan");
        sim->tspan[0] = tspan2[0];
        sim->tspan[1] = tspan2[1];
        sim->tspan_per_member = false;
    });
}
int clode_sim_set_tspan_per_member(clode_sim *sim, const double *tspan, size_t n)
{
    SIM_GUARD({
        if ((long long)n != 2 * sim->nPts || sim->nPts <= 0)
            fail(CLODE_ERR_INVALID_ARGUMENT, "per-member tspan needs 2*nPts=%lld values, received %zu",
                 2 * sim->nPts, n);
        need(tspan, "tspan");
        sim->tspan_pm.assign(tspan, tspan + n);
        sim->tspan_per_member = true;
        sim->ensure_stream();
        sim->sync_tspan_device();
    });
}
int clode_sim_set_solver_params(clode_sim *sim, const clode_solver_params *sp)
{
    SIM_GUARD({
        need(sp, "solver params");
        sim->sp = *sp;  // device dt is reset only when nPts changes (CLODE.cpp:377-402)
    });
}
int clode_sim_get_solver_params(clode_sim *sim, clode_solver_params *sp)
{
    SIM_GUARD({
        need(sp, "solver params");
        *sp = sim->sp;
    });
}
int clode_sim_set_observer_params(clode_sim *sim, const clode_observer_params *op)
{
    SIM_GUARD({
        need(op, "observer params");
        sim->op = *op;
    });
}
int clode_sim_get_observer_params(clode_sim *sim, clode_observer_params *op)
{
    SIM_GUARD({
        need(op, "observer params");
        *op = sim->op;
    });
}
int clode_sim_seed_rng(clode_sim *sim, int use_seed, int seed) { SIM_GUARD(sim->seed_rng(use_seed != 0, seed)); }

int clode_rng_jump(unsigned long long s0, unsigned long long s1, unsigned long long steps, unsigned long long *out_s0,
                   unsigned long long *out_s1)
{
    if (!out_s0 || !out_s1)
        return set_error(CLODE_ERR_INVALID_ARGUMENT, "clode_rng_jump: null output");
    uint64_t a = s0, b = s1;
    gf2_apply(gf2_jump(steps), a, b);
    *out_s0 = a;
    *out_s1 = b;
    return CLODE_OK;
}
int clode_sim_transient(clode_sim *sim) { SIM_GUARD(sim->transient()); }
int clode_sim_initialize_observer(clode_sim *sim) { SIM_GUARD(sim->initialize_observer()); }
int clode_sim_features(clode_sim *sim, int reinitialize) { SIM_GUARD(sim->features(reinitialize)); }
int clode_sim_is_observer_initialized(clode_sim *sim, int *initialized)
{
    SIM_GUARD({
        need(initialized, "initialized");
        *initialized = sim->observer_initialized ? 1 : 0;
    });
}
int clode_sim_trajectory(clode_sim *sim) { SIM_GUARD(sim->trajectory()); }
int clode_sim_autotune(clode_sim *sim, long long sample, double *best_ms) { SIM_GUARD(sim->autotune(sample, best_ms)); }
int clode_sim_chain(clode_sim *sim, const int *ops, int n_ops, int use_graph)
{
    SIM_GUARD({
        if (n_ops < 0 || (n_ops > 0 && !ops))
            fail(CLODE_ERR_INVALID_ARGUMENT, "invalid op list");
        sim->chain(ops, n_ops, use_graph != 0);
    });
}
int clode_sim_shift_tspan(clode_sim *sim) { SIM_GUARD(sim->shift_tspan()); }
int clode_sim_shift_x0(clode_sim *sim) { SIM_GUARD(sim->shift_x0()); }

int clode_sim_get_sizes(clode_sim *sim, clode_sizes *out)
{
    SIM_GUARD({
        need(out, "out");
        out->n_pts = std::max<long long>(0, sim->nPts);
        out->n_var = sim->nVar;
        out->n_par = sim->nPar;
        out->n_aux = sim->nAux;
        out->n_wiener = sim->nWiener;
        out->n_features = sim->kind == CLODE_SIM_FEATURES ? (long long)sim->names().size() : 0;
        out->max_store = sim->sp.max_store;
        out->t_elements = (long long)sim->array_len(CLODE_ARRAY_T);
        out->x_elements = (long long)sim->array_len(CLODE_ARRAY_X);
        out->aux_elements = (long long)sim->array_len(CLODE_ARRAY_AUX);
        out->n_store_var = sim->store_nv();
        out->n_store_aux = sim->store_na();
        out->event_rows = sim->events_valid ? sim->ev_rows : 0;
    });
}

int clode_sim_get(clode_sim *sim, int which, double *out, size_t capacity, size_t *n)
{
    SIM_GUARD({
        size_t len = sim->nPts < 0 ? 0 : sim->array_len(which);
        if (n)
            *n = len;
        if (!out)
            return;
        if (capacity < len)
            fail(CLODE_ERR_INVALID_ARGUMENT, "output capacity %zu is smaller than the array (%zu)", capacity, len);
        sim->get(which, out, len);
    });
}

int clode_sim_get_n_stored(clode_sim *sim, int *out, size_t capacity, size_t *n)
{
    SIM_GUARD({
        size_t len = sim->traj_rows > 0 ? (size_t)sim->nPts : 0;
        if (n)
            *n = len;
        if (!out || !len)
            return;
        if (capacity < len)
            fail(CLODE_ERR_INVALID_ARGUMENT, "output capacity %zu is smaller than nPts (%zu)", capacity, len);
        sim->ensure_stream();
        check_cuda(cudaMemcpy(out, sim->nstored.p, len * sizeof(int), cudaMemcpyDeviceToHost), "D2H copy");
    });
}

int clode_sim_get_trajectory_by_member(clode_sim *sim, long long first, long long count, long long rows,
                                       double *t_out, double *x_out, double *dx_out, double *aux_out,
                                       int *n_stored_out)
{
    SIM_GUARD({ sim->get_by_member(false, first, count, rows, t_out, x_out, dx_out, aux_out, n_stored_out); });
}

int clode_sim_get_events_by_member(clode_sim *sim, long long first, long long count, long long rows, double *t_out,
                                   double *x_out, double *dx_out, double *aux_out, int *n_events_out)
{
    SIM_GUARD({ sim->get_by_member(true, first, count, rows, t_out, x_out, dx_out, aux_out, n_events_out); });
}

int clode_sim_features_store(clode_sim *sim, int initialize_observer, unsigned int event_rows)
{
    SIM_GUARD(sim->features_store(initialize_observer, event_rows));
}

int clode_sim_set_store_variables(clode_sim *sim, const int *var_ix, int n_var_ix, const int *aux_ix, int n_aux_ix)
{
    SIM_GUARD(sim->set_store_variables(var_ix, n_var_ix, aux_ix, n_aux_ix));
}

int clode_sim_get_n_events(clode_sim *sim, int *out, size_t capacity, size_t *n)
{
    SIM_GUARD({
        size_t len = sim->events_valid ? (size_t)sim->nPts : 0;
        if (n)
            *n = len;
        if (!out || !len)
            return;
        if (capacity < len)
            fail(CLODE_ERR_INVALID_ARGUMENT, "output capacity %zu is smaller than nPts (%zu)", capacity, len);
        sim->ensure_stream();
        check_cuda(cudaMemcpy(out, sim->nevents.p, len * sizeof(int), cudaMemcpyDeviceToHost), "D2H copy");
    });
}

int clode_sim_get_status(clode_sim *sim, int *out, size_t capacity, size_t *n)
{
    SIM_GUARD({
        size_t len = sim->nPts > 0 ? (size_t)sim->nPts : 0;
        if (n)
            *n = len;
        if (!out || !len)
            return;
        if (capacity < len)
            fail(CLODE_ERR_INVALID_ARGUMENT, "output capacity %zu is smaller than nPts (%zu)", capacity, len);
        sim->ensure_stream();
        check_cuda(cudaMemcpy(out, sim->status.p, len * sizeof(int), cudaMemcpyDeviceToHost), "D2H copy");
    });
}

int clode_sim_get_rng_state(clode_sim *sim, unsigned long long *out, size_t capacity, size_t *n)
{
    SIM_GUARD({
        size_t len = sim->nPts > 0 ? 2 * (size_t)sim->nPts : 0;
        if (n)
            *n = len;
        if (!out || !len)
            return;
        if (capacity < len)
            fail(CLODE_ERR_INVALID_ARGUMENT, "output capacity %zu is smaller than 2*nPts (%zu)", capacity, len);
        sim->ensure_stream();
        check_cuda(cudaMemcpy(out, sim->rng.p, len * sizeof(unsigned long long), cudaMemcpyDeviceToHost), "D2H copy");
    });
}

int clode_sim_set_rng_state(clode_sim *sim, const unsigned long long *state, size_t n)
{
    SIM_GUARD({
        if (sim->nPts <= 0 || n != 2 * (size_t)sim->nPts)
            fail(CLODE_ERR_INVALID_ARGUMENT, "RNG state needs 2*nPts=%lld words, received %zu", 2 * sim->nPts, n);
        need(state, "state");
        // (0, 0) is xoroshiro128+'s fixed point: the polar method would draw
        // rejected candidates from it forever (clode/cpp/clODE_random.cl:88-114)
        const long long np = sim->nPts;
        for (long long i = 0; i < np; ++i)
            if (state[i] == 0 && state[np + i] == 0)
                fail(CLODE_ERR_INVALID_ARGUMENT,
                     "member %lld: the all-zero RNG state is the generator's fixed point and never yields a normal", i);
        sim->ensure_stream();
        check_cuda(cudaMemcpy(sim->rng.p, state, n * sizeof(unsigned long long), cudaMemcpyHostToDevice), "H2D copy");
    });
}

int clode_sim_get_stats(clode_sim *sim, unsigned long long *out)
{
    SIM_GUARD({
        need(out, "out");
        memcpy(out, sim->last_stats, sizeof sim->last_stats);
    });
}

int clode_sim_last_kernel_ms(clode_sim *sim, double *ms)
{
    SIM_GUARD({
        need(ms, "ms");
        *ms = sim->last_ms;
    });
}

int clode_sim_get_string(clode_sim *sim, int which, char *buf, size_t capacity, size_t *n)
{
    SIM_GUARD({
        std::string s;
        switch (which) {
        case CLODE_STRING_PROGRAM:
            s = sim->built ? "// options: " + sim->prog.options + "\n" + sim->prog.source : std::string();
            break;
        case CLODE_STRING_FEATURE_NAMES: s = join(sim->names()); break;
        case CLODE_STRING_AVAILABLE_STEPPERS: {
            std::vector<std::string> v;
            for (auto &kv : kSteppers)
                v.push_back(kv.first);
            s = join(v);
            break;
        }
        case CLODE_STRING_AVAILABLE_OBSERVERS: {
            std::vector<std::string> v;
            for (auto &kv : kObservers)
                v.push_back(kv.first);
            s = join(v);
            break;
        }
        case CLODE_STRING_OBSERVER_NAME: s = sim->observer; break;
        case CLODE_STRING_STEPPER: s = sim->stepper; break;
        case CLODE_STRING_STATUS_REPORT: s = sim->status_report(); break;
        case CLODE_STRING_BUILD_LOG: s = sim->prog.log; break;
        default: fail(CLODE_ERR_INVALID_ARGUMENT, "unknown string id %d", which);
        }
        copy_string(s, buf, capacity, n);
    });
}

int clode_sim_set_option(clode_sim *sim, const char *key, double value)
{
    SIM_GUARD({
        need(key, "key");
        std::string k = key;
        if (k == "schedule") {
            sim->schedule = (int)value;
        } else if (k == "block_size") {
            if (value < 32 || value > 1024)
                fail(CLODE_ERR_INVALID_ARGUMENT, "block_size must be in [32, 1024]");
            sim->block_size = (int)value;
        } else if (k == "blocks_per_sm") {
            sim->blocks_per_sm = (int)value;
        } else if (k == "fmad") {
            bool v = value != 0.0;
            if (v != sim->fmad) {
                sim->fmad = v;
                sim->built = false;
            }
        } else if (k == "prec_div" || k == "ftz" || k == "fast_math" || k == "fast_exp" || k == "paired" ||
                   k == "split_attempts") {
            bool v = value != 0.0;
            bool &field = k == "prec_div"    ? sim->prec_div
                          : k == "ftz"       ? sim->ftz
                          : k == "fast_math" ? sim->fast_math
                          : k == "fast_exp"  ? sim->fast_exp
                          : k == "paired"    ? sim->paired
                                             : sim->split_attempts;
            if (v != field) {
                field = v;
                sim->built = false;
            }
        } else if (k == "step_block") {
            int v = (int)value;
            if (v < 1 || v > 1024)
                fail(CLODE_ERR_INVALID_ARGUMENT, "step_block must be in [1, 1024]");
            if (v != sim->step_block) {
                sim->step_block = v;
                sim->built = false;
            }
        } else if (k == "maxrregcount") {
            int v = (int)value;
            if (v != 0 && (v < 32 || v > 255))
                fail(CLODE_ERR_INVALID_ARGUMENT, "maxrregcount must be 0 or in [32, 255]");
            if (v != sim->maxrregcount) {
                sim->maxrregcount = v;
                sim->built = false;
            }
        } else if (k == "time_budget_ms") {
            sim->time_budget_ms = value;
        } else if (k == "fuse_init") {
            sim->fuse_init = value != 0.0;
        } else if (k == "collect_stats") {
            sim->collect_stats = value != 0.0;
        } else if (k == "order_by_span") {
            sim->order_by_span = value != 0.0;
        } else if (k == "order_by_work") {
            sim->order_by_work = value != 0.0;
        } else if (k == "precise") {
            if ((value != 0.0) != sim->precise) {
                sim->precise = value != 0.0;
                sim->built = false;
            }
        } else if (k == "replay") {
            sim->replay = value != 0.0;
            if (!sim->replay) {
                // the record regions are only used by the replay
                sim->rec.release();
                sim->rec_mask.release();
                sim->rec_member.release();
            }
        } else if (k == "replay_split") {
            if ((value != 0.0) != sim->replay_split) {
                sim->replay_split = value != 0.0;
                sim->built = false;
            }
        } else if (k == "predraw") {
            sim->predraw = value != 0.0;
            if (!sim->predraw) {
                sim->noise.release();
                sim->noise_count.release();
            }
        } else if (k == "replay_room") {
            if (!(value >= 0.0 && value <= 100.0))
                fail(CLODE_ERR_INVALID_ARGUMENT, "replay_room must be in [0, 100]");
            sim->replay_room = value;
        } else if (k == "replay_fused") {
            sim->replay_fused = value != 0.0;
        } else if (k == "replay_stages") {
            if (value < -1.0 || value > 16.0)
                fail(CLODE_ERR_INVALID_ARGUMENT, "replay_stages must be -1 (automatic) or 0 .. 16");
            sim->replay_stages = (int)value;
        } else if (k == "replay_mb") {
            if (value < 0.0)
                fail(CLODE_ERR_INVALID_ARGUMENT, "replay_mb must be >= 0");
            sim->replay_mb = value;
        } else {
            fail(CLODE_ERR_INVALID_ARGUMENT, "unknown option '%s'", key);
        }
    });
}

int clode_sim_get_option(clode_sim *sim, const char *key, double *value)
{
    SIM_GUARD({
        need(key, "key");
        need(value, "value");
        std::string k = key;
        if (k == "schedule") *value = sim->schedule;
        else if (k == "block_size") *value = sim->block_size;
        else if (k == "blocks_per_sm") *value = sim->blocks_per_sm;
        else if (k == "fmad") *value = sim->fmad;
        else if (k == "prec_div") *value = sim->prec_div;
        else if (k == "ftz") *value = sim->ftz;
        else if (k == "fast_math") *value = sim->fast_math;
        else if (k == "fast_exp") *value = sim->fast_exp;
        else if (k == "paired") *value = sim->paired;
        else if (k == "split_attempts") *value = sim->split_attempts;
        else if (k == "step_block") *value = sim->step_block;
        else if (k == "maxrregcount") *value = sim->maxrregcount;
        else if (k == "time_budget_ms") *value = sim->time_budget_ms;
        else if (k == "fuse_init") *value = sim->fuse_init;
        else if (k == "collect_stats") *value = sim->collect_stats;
        else if (k == "order_by_span") *value = sim->order_by_span;
        else if (k == "order_by_work") *value = sim->order_by_work;
        else if (k == "precise") *value = sim->precise;
        else if (k == "replay") *value = sim->replay;
        else if (k == "replay_mb") *value = sim->replay_mb;
        else if (k == "replay_stages") *value = sim->replay_stages;
        else if (k == "replay_split") *value = sim->replay_split;
        else if (k == "replay_fused") *value = sim->replay_fused;
        else if (k == "replay_room") *value = sim->replay_room;
        else if (k == "predraw") *value = sim->predraw;
        else if (k == "predrawn") *value = sim->last_predrawn;
        else if (k == "predraw_ms") *value = sim->last_draw_ms;
        else if (k == "replay_stages_used") *value = sim->last_stages;
        else if (k == "replay_regions_per_warp") *value = sim->last_regions_per_warp;
        else if (k == "replay_rewarm") *value = sim->last_rewarm;
        else if (k == "replay_rows") *value = sim->last_rows;
        else if (k == "replay_reallocs") *value = sim->last_reallocs;
        else if (k == "download_ms") *value = sim->last_download_ms;
        else if (k == "download_wall_ms") *value = sim->last_download_wall_ms;
        else if (k == "download_pin_ms") *value = sim->last_download_pin_ms;
        else if (k == "download_convert_ms") *value = sim->last_download_convert_ms;
        else if (k == "replay_row_bytes")  // one warp-wide row: every stored field of 32 lanes and the two masks
            *value = sim->rec_fields ? (double)sim->rec_fields * 32.0 * (double)sim->real_size() + 8.0 : 0.0;
        else if (k == "warmup_ms") *value = sim->last_warmup_ms;
        else if (k == "replay_chunks") *value = sim->last_replay_chunks;
        else if (k == "replay_fallback") *value = sim->last_fallback;
        else if (k == "replay_record_ms") *value = sim->last_record_ms;
        else if (k == "replay_replay_ms") *value = sim->last_replay_ms;
        else if (k == "replay_fallback_ms") *value = sim->last_fallback_ms;
        else if (k == "last_grid") *value = sim->last_grid;
        else if (k == "last_block") *value = sim->last_block;
        else fail(CLODE_ERR_INVALID_ARGUMENT, "unknown option '%s'", key);
    });
}

int clode_sim_kernel_info(clode_sim *sim, const char *kernel, int *registers, int *max_threads)
{
    SIM_GUARD({
        need(kernel, "kernel");
        sim->ensure_built();
        std::string k = kernel;
        cudaKernel_t kk = k == "transient" ? sim->k_transient
                          : k == "trajectory" ? sim->k_trajectory
                          : k == "init_observer" ? sim->k_init
                          : k == "features" ? sim->k_features
                          : k == "transient_persistent" ? sim->kp_transient
                          : k == "trajectory_persistent" ? sim->kp_trajectory
                          : k == "features_persistent" ? sim->kp_features : nullptr;
        if (!kk)
            fail(CLODE_ERR_INVALID_ARGUMENT, "no kernel '%s' in this program", kernel);
        cudaFuncAttributes fa;
        check_cuda(cudaFuncGetAttributes(&fa, (const void *)kk), "cudaFuncGetAttributes");
        if (registers)
            *registers = fa.numRegs;
        if (max_threads)
            *max_threads = fa.maxThreadsPerBlock;
    });
}

}  // extern "C"

// ------------------------------------------ for the no-allocation entry point
namespace clode {

static_assert(sizeof(ArgsT<double>) <= sizeof(((NoallocFeaturesLaunch *)nullptr)->args), "argument block size");

void set_last_error_message(const char *msg) { g_last_error = msg ? msg : ""; }

void noalloc_features_prepare(clode_sim *sim, NoallocFeaturesLaunch *out)
{
    if (!sim)
        fail(CLODE_ERR_INVALID_ARGUMENT, "sim must not be NULL");
    if (sim->kind != CLODE_SIM_FEATURES)
        fail(CLODE_ERR_STATE, "not a feature simulator");
    if (!sim->built || !sim->lib || !sim->kp_features)
        fail(CLODE_ERR_NOT_BUILT, "the feature simulator must be built (clode_sim_build) on its device first");
    if (!sim->observer_program_current())
        fail(CLODE_ERR_NOT_BUILT, "observer parameters changed the program: rebuild with clode_sim_build");
    if (sim->built_store)
        fail(CLODE_ERR_NOT_BUILT, "the loaded program stores trajectories (features_store ran last): rebuild the plain "
                                  "program with clode_sim_build");
    memset(out, 0, sizeof *out);
    out->kernel = (void *)sim->kp_features;
    out->single = sim->single ? 1 : 0;
    out->obs_words = sim->obs_words;
    out->n_par = sim->nPar;
    out->device = sim->lib_device;
    out->block = std::max(32, std::min(1024, sim->block_size));
    if (sim->single) {
        ArgsT<float> a = sim->make_args<float>();
        ArgsT<float> clean;
        memset(&clean, 0, sizeof clean);
        clean.t0 = a.t0;
        clean.t1 = a.t1;
        clean.sp = a.sp;
        clean.op = a.op;
        memcpy(out->args, &clean, sizeof clean);
    } else {
        ArgsT<double> a = sim->make_args<double>();
        ArgsT<double> clean;
        memset(&clean, 0, sizeof clean);
        clean.t0 = a.t0;
        clean.t1 = a.t1;
        clean.sp = a.sp;
        clean.op = a.op;
        memcpy(out->args, &clean, sizeof clean);
    }
}

}  // namespace clode
