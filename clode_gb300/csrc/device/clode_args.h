// Kernel argument block shared by the host runtime (g++/nvcc) and the
// NVRTC-compiled ensemble kernels.  Passed by value to every kernel, so the
// solver and observer parameters sit in the constant bank rather than in
// global memory.  No includes: NVRTC compiles it without system headers.
//
// SolverParams / ObserverParams keep the field order and meaning of
// clode/cpp/clODE_struct_defs.cl:11-20 and clode/cpp/observers.cl:25-46.
#pragma once

namespace clode {

template <typename R>
struct SolverParamsT {
    R dt;
    R dtmax;
    R abstol;
    R reltol;
    unsigned int max_steps;
    unsigned int max_store;
    unsigned int nout;
};

template <typename R>
struct ObserverParamsT {
    unsigned int eVarIx;
    unsigned int fVarIx;
    unsigned int maxEventCount;
    unsigned int maxEventTimestamps;
    R minXamp;
    R minIMI;
    R nHoodRadius;
    R xUpThresh;
    R xDownThresh;
    R dxUpThresh;
    R dxDownThresh;
    R eps_dx;
};

// Per-member status bits (written to ArgsT::status when it is non-null)
enum StatusBits {
    STATUS_HMIN_FAIL = 1,       // an adaptive step hit hmin with error above tolerance
    STATUS_NONFINITE = 2,       // the final state holds a NaN or Inf
    STATUS_MAX_STEPS = 4,       // the loop stopped on max_steps before reaching t1
    STATUS_TERMINAL_EVENT = 8,  // the observer's event limit ended the run
    STATUS_TIME_BUDGET = 16,    // the persistent launch ran out of its time budget
};

// Launch-wide counters (ArgsT::stats, 64-bit, accumulated with atomics)
enum StatsSlots {
    STAT_STEPS = 0,        // accepted steps
    STAT_REJECTED = 1,     // rejected adaptive attempts
    STAT_RHS_EVALS = 2,    // right-hand-side evaluations, all passes
    STAT_EVENTS = 3,       // observer events
    STAT_MEMBERS = 4,      // members finished
    STAT_COUNT = 8
};

template <typename R>
struct ArgsT {
    // ensemble geometry: SoA stride and the member range this launch covers
    int nPts;
    int i_begin;
    int i_end;
    int i_stride;              // persistent kernels: members i_begin, i_begin + i_stride, ... below i_end (<= 1: all)
    int fused_init;            // features: run the observer initialisation in the same launch
    // time span: global [t0, t1] or, when tspan_pm != 0, per member [2*i], [2*i+1]
    R t0;
    R t1;
    const R *tspan_pm;
    // problem data, SoA [j * nPts + i]
    const R *x0;
    const R *pars;
    R *xf;
    unsigned long long *rng;   // [2 * nPts]
    R *dt;                     // [nPts], read at start, written at end
    R *tf;                     // [nPts]
    // observer state, SoA in 32-bit words [w * nPts + i], and features [k * nPts + i]
    unsigned int *odata;
    R *F;
    // trajectory output, [row * nPts * n + j * nPts + i]
    R *t_out;
    R *x_out;
    R *dx_out;
    R *aux_out;
    int *n_stored;
    // features with storage (programs built with CLODE_FEATURE_STORE): the
    // state at each of the first ev_rows observer events of a member,
    // [k * nPts * n + j * nPts + i], and the member's event count
    R *ev_t;
    R *ev_x;
    R *ev_dx;
    R *ev_aux;
    int *n_events;
    unsigned int ev_rows;
    // optional diagnostics (may be null)
    int *status;
    unsigned long long *stats;
    // persistent scheduling: next member to hand out, and a %globaltimer budget in ns (0 = none)
    unsigned int *work_next;
    unsigned long long time_budget_ns;
    // persistent kernels: position k of the range runs member order[k]
    // (null: member k), e.g. the longest time spans first
    const int *order;
    // persistent observer initialisation: each member's warm-up steps (null: not recorded)
    int *work_out;
    // replay of the warm-up pass (two-pass observers): the recording warm-up
    // launch stores every step of the feature pass in per-warp regions of
    // rec_rows rows, [((warp * rec_rows + row) * fields + field) * 32 + lane];
    // per row the lanes with a step and the lanes whose member starts there,
    // rec_mask[2 * (warp * rec_rows + row) + {0, 1}]; the members in the
    // order they start, rec_member[warp * rec_members + k]; rows recorded,
    // rec_used[warp]; the state at the end of each member's feature pass,
    // fin[i * stride + word]; and the members the replay cannot finish
    // (fallback[0 .. *fallback_count)), which the plain feature pass runs.
    R *rec;
    unsigned int *rec_mask;
    int *rec_member;
    unsigned int *rec_used;
    unsigned long long rec_rows;
    unsigned long long rec_fetch_rows;  // a warp takes no new member once this many rows are recorded
    unsigned int rec_members;
    unsigned int *fin;
    int *fallback;
    unsigned int *fallback_count;
    // the replay's shared-memory stages per warp (rows copied ahead by TMA
    // bulk copies; 0: rows read from global memory), and a word the replay
    // sets when a stage was not filled within its wait limit
    unsigned int rec_stages;
    unsigned int *rec_error;
    // regions each replay warp takes in turn (the replay's blocks are the
    // recording launch's, with this many times fewer threads)
    unsigned int rec_regions_per_warp;
    // pre-drawn normal deviates (stochastic stepper): member i's k-th deviate
    // is noise[i * noise_stride + k]; null: the kernels draw them.  Filled by
    // the draw launch from noise_count[i] (the deviates member i's run takes,
    // from the count launch), the generator's jump matrices noise_mats and
    // noise_block candidates per lane and round.
    R *noise;
    unsigned long long noise_stride;
    unsigned int *noise_count;
    const unsigned long long *noise_mats;
    unsigned int noise_block;
    SolverParamsT<R> sp;
    ObserverParamsT<R> op;
};

}  // namespace clode
