/*
 * clode_gb300 — C ABI of the GB300 ensemble ODE/SDE engine.
 *
 * This is the boundary a host language binds (ctypes, cgo, JNI, N-API ...).
 * It replaces the OpenCL resource/program layer and the three simulator
 * classes of clODE (clode/cpp/OpenCLResource.hpp:73-125, clode/cpp/CLODE.hpp:93-189,
 * clode/cpp/CLODEfeatures.hpp:23-76, clode/cpp/CLODEtrajectory.hpp:21-52) that
 * clODE's pybind11 module clode_cpp_wrapper exposes (clode/cpp/CLODEpython.cpp:35-381).
 * Each entry point below names the reference member function it stands in for.
 *
 * Conventions
 *  - Every function returns CLODE_OK (0) or a CLODE_ERR_* code; the message of
 *    the last error on the calling thread is returned by clode_last_error().
 *  - Host arrays are double, SoA column-major exactly as clODE's host side
 *    takes them: x0[j*nPts + i], pars[j*nPts + i] (clode/cpp/CLODE.cpp:245-350),
 *    features F[k*nPts + i], trajectories [store*nPts*n + j*nPts + i].
 *    Single-precision simulators convert on the device.
 *  - Calls on one simulator are synchronous (every run ends with a stream
 *    synchronize, as the reference ends every launch with finish()) and not
 *    thread-safe; different simulators may be driven from different threads.
 *  - Size mismatches in set_x0 / set_pars / set_problem_data are reported as
 *    CLODE_ERR_INVALID_ARGUMENT (the reference logs and ignores them,
 *    clode/cpp/CLODE.cpp:247-271,309-349); nothing is changed in that case.
 *  - No entry point falls back to the CPU: without a usable CUDA device, run
 *    calls fail with CLODE_ERR_NO_DEVICE.
 */
#ifndef CLODE_GB300_H
#define CLODE_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CLODE_GB300_VERSION 100

enum clode_status {
    CLODE_OK = 0,
    CLODE_ERR_INVALID_ARGUMENT = 1,
    CLODE_ERR_CUDA = 2,
    CLODE_ERR_COMPILE = 3,
    CLODE_ERR_NOT_BUILT = 4,
    CLODE_ERR_NO_DEVICE = 5,
    CLODE_ERR_OUT_OF_MEMORY = 6,
    CLODE_ERR_STATE = 7,
    CLODE_ERR_INTERNAL = 8
};

/* simulator kinds: CLODE, CLODEfeatures, CLODEtrajectory */
enum clode_sim_kind { CLODE_SIM_BASE = 0, CLODE_SIM_FEATURES = 1, CLODE_SIM_TRAJECTORY = 2 };

/* arrays readable with clode_sim_get() */
enum clode_array {
    CLODE_ARRAY_X0 = 0,     /* CLODE::getX0       clode/cpp/CLODE.cpp:517   */
    CLODE_ARRAY_XF = 1,     /* CLODE::getXf       clode/cpp/CLODE.cpp:534   */
    CLODE_ARRAY_DT = 2,     /* CLODE::getDt       clode/cpp/CLODE.cpp:551   */
    CLODE_ARRAY_TF = 3,     /* CLODE::getTf       clode/cpp/CLODE.cpp:568   */
    CLODE_ARRAY_PARS = 4,   /* CLODE::getPars     clode/cpp/CLODE.hpp:180   */
    CLODE_ARRAY_TSPAN = 5,  /* CLODE::getTspan    clode/cpp/CLODE.hpp:178 (2 values, or 2*nPts per member) */
    CLODE_ARRAY_F = 6,      /* CLODEfeatures::getF         clode/cpp/CLODEfeatures.cpp:261 */
    CLODE_ARRAY_T = 7,      /* CLODEtrajectory::getT       clode/cpp/CLODEtrajectory.cpp:132 */
    CLODE_ARRAY_X = 8,      /* CLODEtrajectory::getX       clode/cpp/CLODEtrajectory.cpp:149 */
    CLODE_ARRAY_DX = 9,     /* CLODEtrajectory::getDx      clode/cpp/CLODEtrajectory.cpp:166 */
    CLODE_ARRAY_AUX = 10,   /* CLODEtrajectory::getAux     clode/cpp/CLODEtrajectory.cpp:183 */
    /* event states of clode_sim_features_store(), [k*nPts*w + j*nPts + i]
     * (the t_event/x_event/dx_event/aux_event buffers of the reference's
     * unused clode/cpp/odedriver.cl:27-30) */
    CLODE_ARRAY_EVENT_T = 11,
    CLODE_ARRAY_EVENT_X = 12,
    CLODE_ARRAY_EVENT_DX = 13,
    CLODE_ARRAY_EVENT_AUX = 14
};

/* strings readable with clode_sim_get_string() */
enum clode_string {
    CLODE_STRING_PROGRAM = 0,             /* CLODE::getProgramString          CLODE.hpp:187 */
    CLODE_STRING_FEATURE_NAMES = 1,       /* CLODEfeatures::getFeatureNames   CLODEfeatures.hpp:74, '\n'-separated */
    CLODE_STRING_AVAILABLE_STEPPERS = 2,  /* CLODE::getAvailableSteppers      CLODE.hpp:185 */
    CLODE_STRING_AVAILABLE_OBSERVERS = 3, /* CLODEfeatures::getAvailableObservers CLODEfeatures.hpp:75 */
    CLODE_STRING_OBSERVER_NAME = 4,       /* CLODEfeatures::getObserverName   CLODEfeatures.hpp:71 */
    CLODE_STRING_STEPPER = 5,
    CLODE_STRING_STATUS_REPORT = 6,       /* CLODE::printStatus text          CLODE.cpp:585-596 */
    CLODE_STRING_BUILD_LOG = 7
};

/* launch-wide counters, clode_sim_get_stats() */
enum clode_stat {
    CLODE_STAT_STEPS = 0,      /* time-loop iterations (accepted steps and hmin failures) */
    CLODE_STAT_REJECTED = 1,   /* rejected adaptive attempts */
    CLODE_STAT_RHS_EVALS = 2,  /* right-hand-side evaluations, all passes */
    CLODE_STAT_EVENTS = 3,     /* observer events */
    CLODE_STAT_COUNT = 8
};

/* per-member status bits, clode_sim_get_status() */
enum clode_member_status {
    CLODE_MEMBER_HMIN_FAIL = 1,
    CLODE_MEMBER_NONFINITE = 2,
    CLODE_MEMBER_MAX_STEPS = 4,
    CLODE_MEMBER_TERMINAL_EVENT = 8,
    CLODE_MEMBER_TIME_BUDGET = 16
};

/* log levels: the values of spdlog::level used by clODE's LogLevel enum
 * (clode/cpp/CLODEpython.cpp:43-51) */
enum clode_log_level {
    CLODE_LOG_TRACE = 0, CLODE_LOG_DEBUG = 1, CLODE_LOG_INFO = 2, CLODE_LOG_WARN = 3,
    CLODE_LOG_ERR = 4, CLODE_LOG_CRITICAL = 5, CLODE_LOG_OFF = 6
};

/* ProblemInfo, clode/cpp/CLODE.hpp:22-91.  rhs_source is the model's getRHS
 * source text (the reference reads it from ProblemInfo::clRHSfilename). */
typedef struct clode_problem {
    const char *rhs_source;
    const char *rhs_name;       /* used in diagnostics only; may be NULL */
    int n_var, n_par, n_aux, n_wiener;
    const char *var_names;      /* '\n'-separated, n_var entries (feature names) */
    const char *par_names;      /* '\n'-separated, may be NULL */
    const char *aux_names;      /* '\n'-separated, n_aux entries */
} clode_problem;

/* SolverParams<double>, clode/cpp/clODE_struct_defs.cl:11-20 */
typedef struct clode_solver_params {
    double dt, dtmax, abstol, reltol;
    unsigned int max_steps, max_store, nout;
} clode_solver_params;

/* ObserverParams<double>, clode/cpp/observers.cl:25-46 */
typedef struct clode_observer_params {
    unsigned int e_var_ix, f_var_ix, max_event_count, max_event_timestamps;
    double min_x_amp, min_imi, nhood_radius, x_up_thresh, x_down_thresh;
    double dx_up_thresh, dx_down_thresh, eps_dx;
} clode_observer_params;

/* DeviceInfo, clode/cpp/OpenCLResource.hpp:33-50 */
typedef struct clode_device_info {
    char name[256];
    char vendor[64];
    char version[64];
    int ordinal;
    int compute_units;            /* SM count */
    int cc_major, cc_minor;
    int max_clock_mhz;
    int max_work_group_size;      /* max threads per block */
    int double_support;
    unsigned long long device_memory_size;
    unsigned long long max_memory_alloc_size;
} clode_device_info;

typedef struct clode_sim clode_sim;

/* ---------------------------------------------------------------- runtime */
/* Message of the last failed call on this thread ("" if none). */
const char *clode_last_error(void);
int clode_version(void);
/* Number of CUDA devices (OpenCLResource::getPlatformAndDevices, OpenCLResource.cpp:130-200). */
int clode_device_count(int *count);
/* DeviceInfo of one device (OpenCLResource::getDeviceInfo / query_opencl, CLODEpython.cpp:134-176). */
int clode_device_query(int ordinal, clode_device_info *out);

/* LoggerSingleton (clode/cpp/CLODEpython.cpp:53-95): level, pattern and an
 * optional sink that receives every formatted message instead of stdout. */
typedef void (*clode_log_sink_fn)(int level, const char *message);
int clode_log_set_level(int level);
int clode_log_get_level(void);
int clode_log_set_pattern(const char *pattern);
int clode_log_set_sink(clode_log_sink_fn sink);
int clode_log_message(int level, const char *message);

/* Directory of the on-disk cache of compiled ensemble programs (NULL: default). */
int clode_set_cache_dir(const char *dir);

/* -------------------------------------------------------------- simulator */
/* CLODE / CLODEfeatures / CLODEtrajectory constructors
 * (CLODE.cpp:13-24, CLODEfeatures.cpp:9-18, CLODEtrajectory.cpp:9-14).
 * observer/op are used by CLODE_SIM_FEATURES only (may be NULL otherwise).
 * device is a CUDA ordinal. */
int clode_sim_create(int kind, const clode_problem *prob, const char *stepper, const char *observer,
                     const clode_observer_params *op, int single_precision, int device, clode_sim **out);
int clode_sim_destroy(clode_sim *sim);

/* setters that require clode_sim_build() afterwards */
int clode_sim_set_problem_info(clode_sim *sim, const clode_problem *prob); /* CLODE::setProblemInfo  CLODE.cpp:43 */
int clode_sim_set_stepper(clode_sim *sim, const char *stepper);           /* CLODE::setStepper      CLODE.cpp:61 */
int clode_sim_set_precision(clode_sim *sim, int single_precision);        /* CLODE::setPrecision    CLODE.cpp:78 */
int clode_sim_set_device(clode_sim *sim, int device);                     /* CLODE::setOpenCL       CLODE.cpp:88 */
int clode_sim_set_observer(clode_sim *sim, const char *observer);         /* CLODEfeatures::setObserver CLODEfeatures.cpp:63 */
/* compile the ensemble program with NVRTC (cached on disk) */
int clode_sim_build(clode_sim *sim);                                      /* CLODE::buildCL         CLODE.cpp:155 */

/* problem data (CLODE.cpp:245-402) */
int clode_sim_set_problem_data(clode_sim *sim, const double *x0, size_t n_x0, const double *pars, size_t n_pars);
int clode_sim_set_x0(clode_sim *sim, const double *x0, size_t n);
int clode_sim_set_pars(clode_sim *sim, const double *pars, size_t n);
int clode_sim_set_tspan(clode_sim *sim, const double *tspan2);
int clode_sim_set_solver_params(clode_sim *sim, const clode_solver_params *sp);
int clode_sim_get_solver_params(clode_sim *sim, clode_solver_params *sp);
/* CLODEfeatures.cpp:78.  max_event_timestamps is compiled into the program: changing it
 * rebuilds it at the next run (clode_sim_features_noalloc then needs clode_sim_build first). */
int clode_sim_set_observer_params(clode_sim *sim, const clode_observer_params *op);
int clode_sim_get_observer_params(clode_sim *sim, clode_observer_params *op);
/* CLODE::seedRNG() / seedRNG(int) (CLODE.cpp:420-465): use_seed = 0 draws a random seed */
int clode_sim_seed_rng(clode_sim *sim, int use_seed, int seed);

/* runs (CLODE.cpp:468-515, CLODEfeatures.cpp:180-259, CLODEtrajectory.cpp:97-130) */
int clode_sim_transient(clode_sim *sim);
int clode_sim_initialize_observer(clode_sim *sim);
/* reinitialize: -1 = features(), 0/1 = features(bool reinitialize_observer) */
int clode_sim_features(clode_sim *sim, int reinitialize);
int clode_sim_is_observer_initialized(clode_sim *sim, int *initialized);
int clode_sim_trajectory(clode_sim *sim);
int clode_sim_shift_tspan(clode_sim *sim);
int clode_sim_shift_x0(clode_sim *sim);

/* sizes: nPts, nFeatures, and element counts of every readable array */
typedef struct clode_sizes {
    long long n_pts, n_var, n_par, n_aux, n_wiener, n_features;
    long long max_store;         /* rows of the trajectory arrays */
    long long t_elements, x_elements, aux_elements;
    long long n_store_var, n_store_aux;  /* stored columns of x/dx and of aux per row */
    long long event_rows;                /* rows of the event arrays (0 before clode_sim_features_store) */
} clode_sizes;
int clode_sim_get_sizes(clode_sim *sim, clode_sizes *out);
/* copy an array to host doubles; *n receives its length. With out == NULL only *n is set. */
int clode_sim_get(clode_sim *sim, int which, double *out, size_t capacity, size_t *n);
int clode_sim_get_n_stored(clode_sim *sim, int *out, size_t capacity, size_t *n); /* CLODEtrajectory::getNstored */
int clode_sim_get_string(clode_sim *sim, int which, char *buf, size_t capacity, size_t *n);

/* ------------------------------------------- additions (no reference counterpart) */
/* Per-member time spans: tspan[2*i], tspan[2*i+1] for member i (n = 2*nPts).
 * Replaces the single global tspan until clode_sim_set_tspan() is called again. */
int clode_sim_set_tspan_per_member(clode_sim *sim, const double *tspan, size_t n);
/* Raw per-member RNG state: 2*nPts u64 words laid out [j*nPts + i] as the
 * kernels read it (clode/cpp/transient.cl:37-39).  Setting it lets a shard of a
 * larger ensemble continue exactly the streams the full ensemble would use.
 * A member whose two words are both zero (the generator's fixed point, from
 * which no normal deviate can ever be accepted) is refused with
 * CLODE_ERR_INVALID_ARGUMENT and nothing is changed. */
int clode_sim_get_rng_state(clode_sim *sim, unsigned long long *out, size_t capacity, size_t *n);
int clode_sim_set_rng_state(clode_sim *sim, const unsigned long long *state, size_t n);
/* The last trajectory regrouped by member, as the per-member arrays that
 * clODE's TrajectorySimulator.get_trajectory slices out of getT/getX/getDx/
 * getAux on the host (clode/trajectory.py:216-264): for members i in
 * [first, first + count) and rows r < rows (rows <= max_store),
 *   t_out[(i - first) * rows + r]
 *   x_out[((i - first) * rows + r) * nVar + j], dx_out likewise,
 *   aux_out[((i - first) * rows + r) * nAux + k],
 *   n_stored_out[i - first] (CLODEtrajectory::getNstored).
 * The regrouping runs on the device; any output may be NULL to skip it. */
int clode_sim_get_trajectory_by_member(clode_sim *sim, long long first, long long count, long long rows,
                                       double *t_out, double *x_out, double *dx_out, double *aux_out,
                                       int *n_stored_out);
/* Features with storage, one pass (the design of the reference's unused
 * unified driver clode/cpp/odedriver.cl:10-162, repaired): the features run
 * of clode_sim_features() (same F, xf, dt, tf, RNG state) that also stores
 * the trajectory rows of that pass exactly as clode_sim_trajectory() stores
 * them (row 0 and every nout-th step, at most max_store + 1 rows; a full
 * buffer ends the storing, not the integration), readable with the
 * CLODE_ARRAY_T..AUX getters, clode_sim_get_n_stored() and
 * clode_sim_get_trajectory_by_member(); and the state (t, x, dx, aux) at
 * each of the first event_rows observer events of every member
 * (CLODE_ARRAY_EVENT_*, clode_sim_get_n_events()).  initialize_observer as
 * in clode_sim_features(). */
int clode_sim_features_store(clode_sim *sim, int initialize_observer, unsigned int event_rows);
/* Events each member met in the feature pass of the last clode_sim_features_store() */
int clode_sim_get_n_events(clode_sim *sim, int *out, size_t capacity, size_t *n);
/* The event states of the last clode_sim_features_store() regrouped by member,
 * as clode_sim_get_trajectory_by_member() does for rows (rows <= event_rows):
 * t_out[(i - first) * rows + k], x_out[((i - first) * rows + k) * n + j], ...,
 * n_events_out[i - first].  Member i's events are its first
 * min(n_events, rows) rows; the rest read zero. */
int clode_sim_get_events_by_member(clode_sim *sim, long long first, long long count, long long rows, double *t_out,
                                   double *x_out, double *dx_out, double *aux_out, int *n_events_out);
/* Stored columns of trajectories and event states: the variables var_ix[0..n_var_ix)
 * and auxiliary variables aux_ix[0..n_aux_ix), in that order (the option
 * clode/cpp/trajectory.cl:3 leaves as a TODO).  A negative count keeps all of
 * them; both negative restore the reference layout.  Takes effect at the next
 * run (the program is rebuilt with the lists compiled in). */
int clode_sim_set_store_variables(clode_sim *sim, const int *var_ix, int n_var_ix, const int *aux_ix, int n_aux_ix);
/* Per-member status bits of the last run (CLODE_MEMBER_*). */
int clode_sim_get_status(clode_sim *sim, int *out, size_t capacity, size_t *n);
/* Launch-wide counters of the last run (CLODE_STAT_*; out has CLODE_STAT_COUNT slots). */
int clode_sim_get_stats(clode_sim *sim, unsigned long long *out);
/* Device time of the last run's kernel launches in milliseconds (CUDA events on the simulator's stream). */
int clode_sim_last_kernel_ms(clode_sim *sim, double *ms);
/* Engine options: "schedule" (0 grid, 1 persistent), "block_size", "blocks_per_sm",
 * "fmad" (0/1: allow contraction of a*b+c; 0 reproduces the reference bit for bit),
 * "prec_div" (1: IEEE division, 0: approximate), "ftz" (1: flush FP32 denormals),
 * "fast_math" (1: approximate exp/log/pow/sin/cos/sqrt, implies prec_div 0 and ftz 1),
 * "fast_exp" (1: the model's FP32 exp within 2.5 ulp by Cody-Waite splitting and the
 * hardware exp2; the step-size controller keeps pow),
 * "paired" (1, the default: FP32 Dormand-Prince stage sums take two state
 * variables per paired FP32 instruction; with fmad 0 the results are bitwise those
 * of paired 0; with fmad 1 the contraction pattern is fixed by the engine),
 * "maxrregcount" (0: no cap, else 32..255 registers per thread),
 * "split_attempts" (adaptive steppers, persistent kernels: 1 = one step attempt per
 * loop iteration, a rejected attempt retried in the next; results are identical),
 * "step_block" (persistent kernels: steps taken between the warp-wide votes that
 * refill lanes, default 16; results are identical),
 * "time_budget_ms" (persistent launches stop taking new members after it),
 * "fuse_init" (0/1, default 0: run the observer initialisation inside the features
 * launch instead of a launch of its own before it; results are identical),
 * "collect_stats" (0/1), "order_by_span" (0/1, default 1: with per-member time
 * spans the persistent lanes take the members in decreasing order of span;
 * results are the same either way), "order_by_work" (0/1, default 1: the
 * feature pass of a two-pass observer takes the members in decreasing order
 * of the steps its separate warm-up launch counted; same results),
 * "replay" (0/1, default 1: with a two-pass observer, the persistent schedule
 * and separate passes, the warm-up launch stores every step of the feature
 * pass in device memory and the feature pass replays them into the observer
 * instead of integrating the trajectory again; results are identical;
 * setting it to 0 frees the device memory of the stored steps),
 * "replay_split" (0, the default: a stored row holds t, x, dx and aux and the
 * replay runs the observer's whole feature-pass update; 1: a row holds only
 * the fields the observer's warm-up-dependent logic reads, and the recording
 * launch takes the rest of the pass (extent, means, step statistics) and
 * leaves it in the member's finish block; not with "precise"; results are
 * identical; a rebuild), "replay_fused" (0, the default; 1: each warp
 * records its region and replays it in one launch per launch pair; results
 * are identical),
 * "predraw" (0/1, default 0; 1: a stochastic trajectory run draws its
 * members' normal deviates in launches of their own before it integrates,
 * four lanes per member, and the trajectory launch reads them; results, RNG
 * words included, are identical; read-only "predrawn": whether the last run
 * did, "predraw_ms": its count and draw launches),
 * "replay_stages" (0, the default: the replay reads each stored row from
 * global memory; 2 .. 16: it copies rows that many ahead into shared memory
 * with bulk copies, one per row, completing on mbarriers; -1: up to 4 that
 * fit; results are identical),
 * "replay_mb" (device memory for the stored steps in MiB; 0, the default:
 * sized from the previous run's steps per member, at most 80 % of the free
 * device memory; the map runs in as many launch pairs as that memory needs),
 * "precise" (0/1, default 0: the precision option, not a parity build:
 * compensated time accumulation, compensated time-weighted means, the
 * adaptive error estimate as a compensated sum, event times refined inside
 * the detecting step in FP64).  Read-only for get_option: "last_grid",
 * "last_block", and of the last replayed run "replay_chunks" (launch pairs),
 * "replay_fallback" (members given to the plain passes), "replay_rewarm" (of
 * those, members whose warm-up a full region cut short), "replay_rows" (rows
 * recorded), "replay_row_bytes" (bytes of one warp-wide row of the built
 * program), "replay_stages_used", "replay_regions_per_warp" (regions each
 * replay warp took: more than one when the replay's blocks fit on an SM
 * fewer at a time than the recording launch's), "replay_reallocs" (record
 * region allocations the last replayed run made), "download_ms",
 * "download_wall_ms", "download_pin_ms", "download_convert_ms" (the last
 * device-to-host transfer of a getter: device time of its conversion and
 * copy, wall time, time spent page-locking the destination, device time of
 * the conversion alone), "warmup_ms" (the separate warm-up launch
 * of the last integrated features run),
 * "replay_record_ms", "replay_replay_ms", "replay_fallback_ms" (device time
 * of each launch kind).
 * Changing a build option (fmad, prec_div, ftz, fast_math, fast_exp, paired,
 * maxrregcount, split_attempts, step_block, precise) recompiles the program at the next run. */
int clode_sim_set_option(clode_sim *sim, const char *key, double value);
int clode_sim_get_option(clode_sim *sim, const char *key, double *value);
/* Chains: ops run back to back on the simulator's stream, one synchronisation
 * at the end; with use_graph the sequence is captured once as a CUDA graph and
 * replayed while the ops, ensemble, time span, parameters and options stay the
 * same.  Each op acts as its API call (a transient -> features chain of the
 * reference's Python API is {TRANSIENT, SHIFT_X0, FEATURES, SHIFT_X0}). */
enum clode_op { CLODE_OP_TRANSIENT = 0, CLODE_OP_FEATURES = 1, CLODE_OP_TRAJECTORY = 2, CLODE_OP_SHIFT_X0 = 3 };
int clode_sim_chain(clode_sim *sim, const int *ops, int n_ops, int use_graph);
/* Autotuner: times the persistent kernel of this simulator's kind on members
 * [0, sample) (sample <= 0: all) for register caps {none, 128, 96, 80, 64} and
 * block sizes {64, 128}, keeps the fastest ("maxrregcount", "block_size",
 * schedule 1) for each value of "split_attempts" (adaptive steppers) and, in
 * FP32 Dormand-Prince builds with fmad 1, of "paired"; keeps the fastest; for
 * two-pass observers (nhood2, thresh2) also times the other values of the replay
 * options and of "fuse_init"; returns the best time.  Numerics options (fmad,
 * prec_div, ftz, fast_math, fast_exp, precise) are not changed; with fmad 1 the
 * choice of "paired" changes how the stage sums are rounded, with fmad 0 nothing
 * it chooses changes a result bit.  The sampled members' dt and
 * RNG state are restored; the observer is re-initialised at the next
 * features run. */
int clode_sim_autotune(clode_sim *sim, long long sample, double *best_ms);
/* Number of kernel launches this library has issued since it was loaded
 * (ensemble kernels and the conversion/seeding kernels alike). */
unsigned long long clode_launch_count(void);
/* The per-member random stream's state (s0, s1) advanced by `steps` draws
 * with the generator's jump matrix (the stream of clode/cpp/clODE_random.cl:
 * 28-44 is linear over GF(2)); the matrices the pre-drawn deviates of a
 * stochastic trajectory run use.  No device work; no reference counterpart. */
int clode_rng_jump(unsigned long long s0, unsigned long long s1, unsigned long long steps,
                   unsigned long long *out_s0, unsigned long long *out_s1);
/* features() for callers that cannot allocate device memory.  No counterpart
 * in the reference.  Some callers may not call cudaMalloc once they are
 * running: services whose device memory is partitioned once at start-up,
 * real-time pipelines that forbid allocation after initialisation (it can
 * block on the driver), plug-ins whose host application owns every device
 * allocation.  The regular path allocates its buffers on first use; this one
 * allocates nothing.  The caller passes every input and output as a device
 * pointer in the simulator's working precision (float if single precision,
 * else double), SoA [j*n_pts + i]: x0 and pars (nVar and nPar columns; pars
 * may be NULL only when nPar is 0), tspan (per member [2i], [2i+1]; NULL =
 * the simulator's tspan), rng (2*n_pts words) and dt (n_pts), read and
 * updated in place, xf (nVar columns), tf, F (nFeatures columns) and
 * optionally status (NULL = not written).  The observer is initialised
 * inside the launch on every call.
 * Scratch (the work counter and the observer state parked per member) lives
 * in one fixed 64 MiB device array compiled into the library: held on every
 * GPU that loads the library until the process exits; n_pts beyond what it
 * holds for the observer (64 MiB / state bytes per member) is rejected with
 * CLODE_ERR_INVALID_ARGUMENT.  The first call on each device looks up the
 * array's device address (in that device's primary context, which must not
 * be reset with cudaDeviceReset afterwards), so make that first call before
 * any stream capture.  The call makes the simulator's device current while it
 * runs and restores the caller's current device before it returns.  The
 * launch is enqueued on `stream` (a cudaStream_t of that device; NULL = the
 * default stream) and the call returns without waiting; every call shares the
 * one array and keeps the last call's contents, so calls that overlap on the
 * GPU race and must be ordered by the caller.  The simulator must be a
 * feature simulator built on its device (clode_sim_build) after its last
 * observer-parameter change and after its last clode_sim_features_store
 * (which loads a program that stores rows). */
int clode_sim_features_noalloc(clode_sim *sim, long long n_pts, const void *x0, const void *pars,
                               const void *tspan, unsigned long long *rng, void *dt, void *xf, void *tf,
                               void *F, int *status, void *stream);
/* Register-file footprint of the built kernels: registers per thread of the features
 * (or transient / trajectory) kernel, as reported by the CUDA driver. */
int clode_sim_kernel_info(clode_sim *sim, const char *kernel, int *registers, int *max_threads);

/* ------------------------------------- learned surrogate (no reference counterpart) */
/* An MLP 2 -> 256 -> 256 -> 256 -> n_heads x n_outputs (ReLU hidden layers),
 * BF16 tensor-core layers with FP32 accumulation, trained on the device.  It
 * learns a feature map from engine-computed points and screens large grids.
 * Inputs x are [n x 2] float rows, targets / predictions [n x n_outputs].
 * n_heads * n_outputs must be 16, 32 or 64. */
typedef struct clode_mlp clode_mlp;
int clode_mlp_create(int n_outputs, int n_heads, int device, unsigned long long seed, clode_mlp **out);
int clode_mlp_destroy(clode_mlp *net);
int clode_mlp_param_count(clode_mlp *net, size_t *n);
/* parameters, float32: W1 [2x256], b1, W2 [256x256], b2, W3 [256x256], b3, Wh [256 x H*K], bh */
int clode_mlp_get_params(clode_mlp *net, float *out, size_t n);
int clode_mlp_set_params(clode_mlp *net, const float *in, size_t n);
/* loss and gradient vector of one batch (every head fits the same targets); no update */
int clode_mlp_gradients(clode_mlp *net, const float *x, const float *y, int n, float *grads, size_t n_grads,
                        float *loss);
/* Adam on mean-square error, `steps` minibatches of `batch` rows of a shuffled copy of
 * (x, y); loss_history (steps floats) may be NULL.  Steps after the first replay a CUDA graph. */
int clode_mlp_train(clode_mlp *net, const float *x, const float *y, long long n, int steps, int batch, float lr,
                    unsigned long long seed, float *loss_history);
/* mean and standard deviation over the heads, [n x n_outputs] each; heads [n x H*K] may be NULL */
int clode_mlp_predict(clode_mlp *net, const float *x, long long n, float *mean, float *spread, float *heads);
/* mean over the heads at every point of an nx x ny grid of inputs
 * x = (-1 + 2 ix / (nx - 1), -1 + 2 iy / (ny - 1)) (0 when the extent is 1),
 * point iy * nx + ix, generated on the device; out[p * K + k] =
 * mean * out_scale[k] + out_offset[k] (scale/offset may be NULL: 1 / 0).
 * The prediction is kept for clode_mlp_screen. */
int clode_mlp_predict_grid(clode_mlp *net, int nx, int ny, const float *out_scale, const float *out_offset,
                           float *out);
/* flags of the last prediction laid out as an nx x ny grid (point iy*nx + ix):
 * bit 0 = head spread above spread_thr[k], bit 1 = jump to a 4-neighbour above jump_thr[k] */
int clode_mlp_screen(clode_mlp *net, int nx, int ny, const float *spread_thr, const float *jump_thr, int *flags);
/* wall time of the last train and predict calls, milliseconds */
int clode_mlp_timings(clode_mlp *net, double *train_ms, double *predict_ms);

#ifdef __cplusplus
}
#endif

#endif /* CLODE_GB300_H */
