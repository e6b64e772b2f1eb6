// Ensemble kernels: transient, trajectory, observer initialisation and
// features, one ensemble member per thread with all of its state in
// registers.  Entry points come in two schedules:
//
//  * grid:       one thread per member of [i_begin, i_end), blocks of
//                blockDim.x threads.  The direct counterpart of the
//                reference's NDRange(nPts) launch (clode/cpp/CLODE.cpp:484).
//  * persistent: a fixed grid (a multiple of the SM count) whose lanes pull
//                members from a global counter one at a time.  A lane whose
//                member finishes early refills itself at the next warp-wide
//                vote (every CLODE_STEP_BLOCK steps), so members of very
//                different lengths (adaptive steps, per-member time spans,
//                terminal events, two-pass observers) keep every lane busy.
//                A two-pass observer's warm-up pass runs as its own launch
//                (clode_init_observer_persistent) or, fused, inside the
//                features launch through the same stepper call as the
//                feature pass.  The host may hand out the members through a
//                permutation (`order`: longest time spans first, or the
//                feature pass by the warm-up's step counts).
//
// Programs built with CLODE_FEATURE_STORE also store, in the feature pass,
// the trajectory rows and the state at observer events (FeatureStore).
//
// Per member, both schedules execute the same arithmetic in the same order,
// so their results are identical whatever order the members are taken in.  Member semantics follow
// clode/cpp/transient.cl:9-77, initializeObserver.cl:9-84, features.cl:10-106
// and trajectory.cl:14-112.
#pragma once

#ifndef CLODE_FEATURE_STORE
#define CLODE_FEATURE_STORE 0
#endif

namespace clode {

typedef ArgsT<realtype> Args;

__device__ __forceinline__ unsigned long long globaltimer_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ realtype member_t0(const Args &a, int i)
{
    return a.tspan_pm ? a.tspan_pm[2ull * i] : a.t0;
}

__device__ __forceinline__ realtype member_t1(const Args &a, int i)
{
    return a.tspan_pm ? a.tspan_pm[2ull * i + 1] : a.t1;
}

__device__ __forceinline__ void load_x0(realtype (&x)[N_VAR], const Args &a, int i)
{
    const unsigned long long n = (unsigned long long)a.nPts;
#pragma unroll
    for (int j = 0; j < N_VAR; ++j)
        x[j] = a.x0[j * n + i];
}

// private copies and the slope at the initial point (transient.cl:20-51)
__device__ __forceinline__ void member_load(Member &m, const Args &a, int i, Counters &c)
{
    const unsigned long long n = (unsigned long long)a.nPts;
    m.t = member_t0(a, i);
    m.dt = a.dt[i];
#pragma unroll
    for (int j = 0; j < N_PAR; ++j)
        m.p[j] = a.pars[j * n + i];
    load_x0(m.x, a, i);
#pragma unroll
    for (int j = 0; j < NW1; ++j)
        m.w[j] = ZERO;
#pragma unroll
    for (int j = 0; j < NA1; ++j)
        m.aux[j] = ZERO;
#if CLODE_STOCHASTIC
    m.r.s0 = a.rng[i];
    m.r.s1 = a.rng[n + i];
    m.r.have_spare = false;
    m.r.spare = ZERO;
    m.sqdt = sqrt(m.dt);
#pragma unroll
    for (int j = 0; j < N_WIENER; ++j)
        m.w[j] = rng_normal(m.r) / m.sqdt;
#endif
    getRHS(m.t, m.x, m.p, m.dx, m.aux, m.w);
    c.rhs += 1;
}

// final state, RNG state, step size and time (transient.cl:64-76).  Only
// the stochastic stepper draws numbers, so the stored RNG state of the other
// steppers is the loaded one and is left untouched in global memory.
__device__ __forceinline__ void member_store(const Member &m, const Args &a, int i)
{
    const unsigned long long n = (unsigned long long)a.nPts;
#pragma unroll
    for (int j = 0; j < N_VAR; ++j)
        a.xf[j * n + i] = m.x[j];
#if CLODE_STOCHASTIC
    a.rng[i] = m.r.s0;
    a.rng[n + i] = m.r.s1;
#endif
    a.dt[i] = m.dt;
    a.tf[i] = m.t;
}

__device__ __forceinline__ int member_status_bits(const Member &m, unsigned int step, const Args &a,
                                                  realtype t1, bool hmin_fail, bool terminal)
{
    int s = 0;
    if (hmin_fail) s |= STATUS_HMIN_FAIL;
    if (terminal) s |= STATUS_TERMINAL_EVENT;
    bool finite = isfinite(m.t);
#pragma unroll
    for (int j = 0; j < N_VAR; ++j)
        finite = finite && isfinite(m.x[j]);
    if (!finite) s |= STATUS_NONFINITE;
    if (!terminal && step >= a.sp.max_steps && m.t <= t1) s |= STATUS_MAX_STEPS;
    return s;
}

// Sum per-thread counters over the warp and add them to the launch totals.
// Must be reached by every lane of the warp.
__device__ __forceinline__ void flush_counters(const Args &a, const Counters &c)
{
    if (!a.stats)
        return;
    unsigned long long v[4] = {c.steps, c.rejected, c.rhs, c.events};
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int off = 16; off > 0; off >>= 1)
            v[k] += __shfl_down_sync(0xffffffffu, v[k], off);
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&a.stats[STAT_STEPS], v[0]);
        atomicAdd(&a.stats[STAT_REJECTED], v[1]);
        atomicAdd(&a.stats[STAT_RHS_EVALS], v[2]);
        atomicAdd(&a.stats[STAT_EVENTS], v[3]);
    }
}

// ------------------------------------------------------------ scheduling --
// Persistent kernels take up to this many steps of a member between the
// warp-wide votes that refill lanes and detect the end of the launch; a lane
// whose member ends inside a block waits for the rest of the block.  Per
// member the steps are exactly those of one step per iteration.
#ifndef CLODE_STEP_BLOCK
#define CLODE_STEP_BLOCK 16
#endif

// Persistent schedule: hand out the next members of [i_begin, i_end) (every
// i_stride-th one when i_stride > 1, as the autotuner samples; through the
// permutation `order` when the host gives one) to the lanes of this warp that
// ask for one, with a single atomic per warp.  Every lane of
// the warp must call it (full-mask vote); lanes with want == false get -1.
// Returns -1 as well once the range is exhausted.
__device__ __forceinline__ int fetch_member(const Args &a, bool want)
{
    const unsigned int lane = threadIdx.x & 31u;
    const unsigned int mask = __ballot_sync(0xffffffffu, want);
    if (mask == 0u)
        return -1;
    const unsigned int leader = __ffs(mask) - 1;
    unsigned int base = 0;
    if (lane == leader)
        base = atomicAdd(a.work_next, (unsigned int)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (!want)
        return -1;
    const long long stride = a.i_stride > 1 ? a.i_stride : 1;
    long long k = (long long)a.i_begin + ((long long)base + __popc(mask & ((1u << lane) - 1u))) * stride;
    if (k >= a.i_end)
        return -1;
    return a.order ? a.order[k] : (int)k;
}

// true when this lane should stop taking new members (time budget spent)
__device__ __forceinline__ bool budget_spent(const Args &a, unsigned long long t_start)
{
    return a.time_budget_ns != 0ull && globaltimer_ns() - t_start > a.time_budget_ns;
}

// ------------------------------------------------------------- transient --
__device__ __forceinline__ void run_transient(const Args &a, int i, Counters &c)
{
    Member m;
    member_load(m, a, i, c);
    const realtype t1 = member_t1(a, i);
    unsigned int step = 0;
    bool hmin_fail = false;
    while (m.t <= t1 && step < a.sp.max_steps) {
        ++step;
        hmin_fail |= step_member(m, a.sp, t1, c) != 0;
    }
    member_store(m, a, i);
    if (a.status)
        a.status[i] = member_status_bits(m, step, a, t1, hmin_fail, false);
}

extern "C" __global__ void clode_transient(const Args a)
{
    Counters c = {0, 0, 0, 0};
    int i = a.i_begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (i < a.i_end)
        run_transient(a, i, c);
    flush_counters(a, c);
}

// transient, persistent schedule: each lane refills itself as its member ends
extern "C" __global__ void clode_transient_persistent(const Args a)
{
    Counters c = {0, 0, 0, 0};
    const unsigned long long t_start = globaltimer_ns();
    bool exhausted = false;
    int i = -1;
    unsigned int step = 0;
    bool hmin_fail = false;
    realtype t1 = ZERO;
    Member m;
    StepCtl sc;
    sc.retry = false;
    for (;;) {
        bool want = i < 0 && !exhausted;
        if (want && budget_spent(a, t_start)) {
            want = false;
            exhausted = true;
        }
        int got = fetch_member(a, want);
        if (want) {
            if (got < 0) {
                exhausted = true;
            } else {
                i = got;
                step = 0;
                hmin_fail = false;
                member_load(m, a, i, c);
                t1 = member_t1(a, i);
            }
        }
        if (__all_sync(0xffffffffu, i < 0))
            break;
        if (i < 0)
            continue;
        bool running = true;
        for (int k = 0; k < CLODE_STEP_BLOCK; ++k) {
            running = sc.retry || (m.t <= t1 && step < a.sp.max_steps);
            if (!running)
                break;
            if (!sc.retry)
                ++step;
            hmin_fail |= step_attempt(m, a.sp, t1, c, sc) == -1;
        }
        if (!running) {
            member_store(m, a, i);
            if (a.status)
                a.status[i] = member_status_bits(m, step, a, t1, hmin_fail, false);
            i = -1;
        }
    }
    flush_counters(a, c);
}

// ------------------------------------------------------------ trajectory --
// Stored columns: every variable and auxiliary variable, or the subsets
// compiled in as index lists CLODE_STORE_VARS / CLODE_STORE_AUX of lengths
// CLODE_STORE_NV / CLODE_STORE_NA (the option clode/cpp/trajectory.cl:3
// leaves as a TODO: "store only a subset of variables (allow bigger nPts)").
// A row is t, the stored x, the stored dx (same indices) and the stored aux.
#ifdef CLODE_STORE_NV
__device__ constexpr int clode_store_var_ix[CLODE_STORE_NV > 0 ? CLODE_STORE_NV : 1] = {CLODE_STORE_VARS};
#define CLODE_STORE_VAR(k) clode_store_var_ix[k]
#else
#define CLODE_STORE_NV N_VAR
#define CLODE_STORE_VAR(k) (k)
#endif
#ifdef CLODE_STORE_NA
__device__ constexpr int clode_store_aux_ix[CLODE_STORE_NA > 0 ? CLODE_STORE_NA : 1] = {CLODE_STORE_AUX};
#define CLODE_STORE_AUXV(k) clode_store_aux_ix[k]
#else
#define CLODE_STORE_NA N_AUX
#define CLODE_STORE_AUXV(k) (k)
#endif

// rows [row * nPts * w + k * nPts + i] (trajectory.cl:63-71, :83-95)
__device__ __forceinline__ void store_state(realtype *t, realtype *x, realtype *dx, realtype *aux,
                                            unsigned long long n, int i, unsigned long long row, const Member &m)
{
    t[row * n + i] = m.t;
#pragma unroll
    for (int k = 0; k < CLODE_STORE_NV; ++k)
        x[(row * CLODE_STORE_NV + k) * n + i] = m.x[CLODE_STORE_VAR(k)];
#pragma unroll
    for (int k = 0; k < CLODE_STORE_NV; ++k)
        dx[(row * CLODE_STORE_NV + k) * n + i] = m.dx[CLODE_STORE_VAR(k)];
#pragma unroll
    for (int k = 0; k < CLODE_STORE_NA; ++k)
        aux[(row * CLODE_STORE_NA + k) * n + i] = m.aux[CLODE_STORE_AUXV(k)];
}

__device__ __forceinline__ void store_row(const Args &a, const Member &m, int i, unsigned long long row)
{
    store_state(a.t_out, a.x_out, a.dx_out, a.aux_out, (unsigned long long)a.nPts, i, row, m);
}

__device__ __forceinline__ void run_trajectory(const Args &a, int i, Counters &c)
{
    Member m;
    member_load(m, a, i, c);
    const realtype t1 = member_t1(a, i);
    unsigned long long row = 0;
    store_row(a, m, i, row);
    unsigned int step = 0;
    unsigned int to_store = a.sp.nout;  // steps until the next stored row (step % nout == 0)
    bool hmin_fail = false;
    while (m.t <= t1 && step < a.sp.max_steps && row < (unsigned long long)a.sp.max_store) {
        ++step;
        hmin_fail |= step_member(m, a.sp, t1, c) != 0;
        if (--to_store == 0) {
            to_store = a.sp.nout;
            ++row;
            store_row(a, m, i, row);
        }
    }
    a.n_stored[i] = (int)row;
    member_store(m, a, i);
    if (a.status)
        a.status[i] = member_status_bits(m, step, a, t1, hmin_fail, false);
}

extern "C" __global__ void clode_trajectory(const Args a)
{
    Counters c = {0, 0, 0, 0};
    int i = a.i_begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (i < a.i_end)
        run_trajectory(a, i, c);
    flush_counters(a, c);
}

// trajectory, persistent schedule
extern "C" __global__ void clode_trajectory_persistent(const Args a)
{
    Counters c = {0, 0, 0, 0};
    const unsigned long long t_start = globaltimer_ns();
    bool exhausted = false;
    int i = -1;
    unsigned int step = 0;
    unsigned int to_store = 0;  // steps until the next stored row (step % nout == 0)
    unsigned long long row = 0;
    bool hmin_fail = false;
    realtype t1 = ZERO;
    Member m;
    StepCtl sc;
    sc.retry = false;
    for (;;) {
        bool want = i < 0 && !exhausted;
        if (want && budget_spent(a, t_start)) {
            want = false;
            exhausted = true;
        }
        int got = fetch_member(a, want);
        if (want) {
            if (got < 0) {
                exhausted = true;
            } else {
                i = got;
                step = 0;
                to_store = a.sp.nout;
                row = 0;
                hmin_fail = false;
                member_load(m, a, i, c);
                t1 = member_t1(a, i);
                store_row(a, m, i, row);
            }
        }
        if (__all_sync(0xffffffffu, i < 0))
            break;
        if (i < 0)
            continue;
        bool running = true;
        for (int k = 0; k < CLODE_STEP_BLOCK; ++k) {
            running = sc.retry || (m.t <= t1 && step < a.sp.max_steps && row < (unsigned long long)a.sp.max_store);
            if (!running)
                break;
            if (!sc.retry)
                ++step;
            const int flag = step_attempt(m, a.sp, t1, c, sc);
            hmin_fail |= flag == -1;
            if (flag != 1 && --to_store == 0) {
                to_store = a.sp.nout;
                ++row;
                store_row(a, m, i, row);
            }
        }
        if (!running) {
            a.n_stored[i] = (int)row;
            member_store(m, a, i);
            if (a.status)
                a.status[i] = member_status_bits(m, step, a, t1, hmin_fail, false);
            i = -1;
        }
    }
    flush_counters(a, c);
}

#if CLODE_HAVE_OBSERVER
// --------------------------------------------------- parked observer state --
static_assert(sizeof(Observer) % 4 == 0, "observer state must be a whole number of 32-bit words");
#define CLODE_OBS_WORDS ((int)(sizeof(Observer) / 4))
// Parked state is member-major, [i * CLODE_OBS_STRIDE + word], each member's
// words rounded up to whole 16-byte vectors: a lane moves its member's state
// in contiguous 16-byte pieces, so every sector it touches is written (or
// read) whole, whatever order the members are taken in.
#define CLODE_OBS_VEC ((CLODE_OBS_WORDS + 3) / 4)
#define CLODE_OBS_STRIDE (4 * CLODE_OBS_VEC)

// read by the host to size the parked-state buffer (words per member, padding included)
extern "C" __device__ const unsigned int clode_observer_words = CLODE_OBS_STRIDE;

__device__ __forceinline__ void park_load(Observer &o, const Args &a, int i)
{
    const uint4 *src = reinterpret_cast<const uint4 *>(a.odata + (unsigned long long)i * CLODE_OBS_STRIDE);
    uint4 v[CLODE_OBS_VEC];
#pragma unroll
    for (int k = 0; k < CLODE_OBS_VEC; ++k)
        v[k] = src[k];
    memcpy(&o, v, sizeof(Observer));
}

__device__ __forceinline__ void park_store(const Observer &o, const Args &a, int i)
{
    uint4 *dst = reinterpret_cast<uint4 *>(a.odata + (unsigned long long)i * CLODE_OBS_STRIDE);
    uint4 v[CLODE_OBS_VEC];
    v[CLODE_OBS_VEC - 1] = make_uint4(0u, 0u, 0u, 0u);
    memcpy(v, &o, sizeof(Observer));
#pragma unroll
    for (int k = 0; k < CLODE_OBS_VEC; ++k)
        dst[k] = v[k];
}

// Observer initialisation for one member (initializeObserver.cl:9-84).
// The member's RNG state and dt are not written back.
__device__ __forceinline__ void init_observer_member(Observer &o, const Args &a, int i, Counters &c)
{
    Member m;
    member_load(m, a, i, c);
    o.init(m.t, m.x, m.dx, m.aux, a.op);
    if (Observer::two_pass) {
        const realtype t1 = member_t1(a, i);
        unsigned int step = 0;
        while (m.t < t1 && step < a.sp.max_steps) {
            ++step;
            step_member(m, a.sp, t1, c);
            o.warmup(m.t, m.x, m.dx, m.aux, a.op);
        }
        // rewind to the initial state (the last noise sample is kept)
        m.t = member_t0(a, i);
        load_x0(m.x, a, i);
        getRHS(m.t, m.x, m.p, m.dx, m.aux, m.w);
        c.rhs += 1;
    }
    o.arm(m.t, m.x, m.dx, m.aux, a.op);
}

extern "C" __global__ void clode_init_observer(const Args a)
{
    Counters c = {0, 0, 0, 0};
    int i = a.i_begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (i < a.i_end) {
        Observer o;
        init_observer_member(o, a, i, c);
        park_store(o, a, i);
    }
    flush_counters(a, c);
}

// Observer initialisation, persistent schedule: lanes refill themselves, and
// every lane runs the same (warm-up) pass, so the observer code never
// diverges between passes.  Not subject to the time budget: every member's
// observer is initialised.
extern "C" __global__ void clode_init_observer_persistent(const Args a)
{
    Counters c = {0, 0, 0, 0};
    bool exhausted = false;
    int i = -1;
    bool fresh = false;
    unsigned int step = 0;
    realtype t1 = ZERO;
    Member m;
    Observer o;
    StepCtl sc;
    sc.retry = false;
    for (;;) {
        const bool want = i < 0 && !exhausted;
        const int got = fetch_member(a, want);
        if (want) {
            if (got < 0) {
                exhausted = true;
            } else {
                i = got;
                fresh = true;
            }
        }
        if (__all_sync(0xffffffffu, i < 0))
            break;
        if (i < 0)
            continue;
        if (fresh) {
            member_load(m, a, i, c);
            o.init(m.t, m.x, m.dx, m.aux, a.op);
            step = 0;
            t1 = member_t1(a, i);
            fresh = false;
        }
        bool running = Observer::two_pass;
        for (int k = 0; k < CLODE_STEP_BLOCK && running; ++k) {
            running = sc.retry || (step < a.sp.max_steps && m.t < t1);
            if (!running)
                break;
            if (!sc.retry)
                ++step;
            if (step_attempt(m, a.sp, t1, c, sc) != 1)
                o.warmup(m.t, m.x, m.dx, m.aux, a.op);
        }
        if (!running) {
            if (Observer::two_pass) {
                // rewind to the initial state (the last noise sample is kept)
                m.t = member_t0(a, i);
                load_x0(m.x, a, i);
                getRHS(m.t, m.x, m.p, m.dx, m.aux, m.w);
                c.rhs += 1;
            }
            o.arm(m.t, m.x, m.dx, m.aux, a.op);
            park_store(o, a, i);
            if (a.work_out)  // the feature pass repeats these steps: the host orders it by them
                a.work_out[i] = (int)step;
            i = -1;
        }
    }
    flush_counters(a, c);
}

#if CLODE_FEATURE_STORE
// Features with storage: the feature pass also stores the trajectory rows
// (row 0 at the start, then every nout-th step, at most max_store + 1 rows,
// as trajectory.cl:63-95) and the state at each of the first ev_rows
// observer events.  This is the design of the reference's unused unified
// driver (clode/cpp/odedriver.cl:10-162, and the "record current state into
// dedicated event buffers" note at features.cl:76), with its defects
// repaired: events are numbered from 0, and a full trajectory buffer stops
// the storing but not the integration, so the features, final state and RNG
// state are those of the features kernel.
struct FeatureStore {
    unsigned long long row;
    unsigned int to_store;  // steps until the next stored row (step % nout == 0)
    unsigned int ev;
    bool on;                // the host gave the row and count buffers (it always does for this build)

    __device__ __forceinline__ void start(const Args &a, const Member &m, int i)
    {
        row = 0;
        to_store = a.sp.nout;
        ev = 0;
        on = a.t_out && a.n_stored && a.n_events;
        if (on)
            store_row(a, m, i, 0);
    }
    __device__ __forceinline__ void after_step(const Args &a, const Member &m, int i)
    {
        if (on && --to_store == 0) {
            to_store = a.sp.nout;
            if (row < (unsigned long long)a.sp.max_store) {
                ++row;
                store_row(a, m, i, row);
            }
        }
    }
    __device__ __forceinline__ void on_event(const Args &a, const Member &m, int i)
    {
        if (on && ev < a.ev_rows && a.ev_t)
            store_state(a.ev_t, a.ev_x, a.ev_dx, a.ev_aux, (unsigned long long)a.nPts, i, ev, m);
        ++ev;
    }
    __device__ __forceinline__ void finish(const Args &a, int i) const
    {
        if (on) {
            a.n_stored[i] = (int)row;
            a.n_events[i] = (int)ev;
        }
    }
};
#endif

// Feature pass for one member (features.cl:10-106)
__device__ __forceinline__ void features_member(Observer &o, const Args &a, int i, Counters &c)
{
    Member m;
    member_load(m, a, i, c);
    const realtype t0 = m.t;
    const realtype t1 = member_t1(a, i);
    unsigned int step = 0;
    bool hmin_fail = false, terminal = false;
#if CLODE_FEATURE_STORE
    FeatureStore fs;
    fs.start(a, m, i);
#endif
    while (m.t <= t1 && step < a.sp.max_steps) {
        ++step;
        hmin_fail |= step_member(m, a.sp, t1, c) != 0;
#if CLODE_FEATURE_STORE
        fs.after_step(a, m, i);
#endif
        o.update(m.t, m.x, m.dx, m.aux, a.op);
        if (o.event(m.t, m.x, m.dx, m.aux, a.op)) {
            c.events++;
#if CLODE_FEATURE_STORE
            fs.on_event(a, m, i);
#endif
            if (o.on_event(m.t, m.x, m.dx, m.aux, a.op)) {
                terminal = true;
                break;
            }
        }
    }
#if CLODE_FEATURE_STORE
    fs.finish(a, i);
#endif
    FOut out = {a.F, (unsigned long long)a.nPts, i, 0};
    o.write(out);
    o.rebase(m.t - t0);
    member_store(m, a, i);
    if (a.status)
        a.status[i] = member_status_bits(m, step, a, t1, hmin_fail, terminal);
}

extern "C" __global__ void clode_features(const Args a)
{
    Counters c = {0, 0, 0, 0};
    int i = a.i_begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (i < a.i_end) {
        Observer o;
        if (a.fused_init)
            init_observer_member(o, a, i, c);
        else
            park_load(o, a, i);
        features_member(o, a, i, c);
        park_store(o, a, i);
    }
    flush_counters(a, c);
}

// Features, persistent schedule.  A lane walks its member through the
// observer's warm-up pass (two-pass observers, when the initialisation is
// fused into this launch) and the feature pass, then takes the next member.
// Both passes go through the same step_attempt call, so lanes in different
// passes stay converged on the expensive part of the loop, and a rejected
// adaptive attempt is retried in the next iteration instead of holding the
// warp for a repeat.
extern "C" __global__ void clode_features_persistent(const Args a)
{
    Counters c = {0, 0, 0, 0};
    const unsigned long long t_start = globaltimer_ns();
    bool exhausted = false;
    int i = -1;
    bool warm = false;    // in the warm-up pass
    bool fresh = false;   // a new member to load
    bool rewind = false;  // warm-up pass ended: reload the member for the feature pass
    unsigned int step = 0;
    bool hmin_fail = false, terminal = false;
    realtype t0 = ZERO, t1 = ZERO;
    Member m;
    Observer o;
    StepCtl sc;
    sc.retry = false;
#if CLODE_FEATURE_STORE
    FeatureStore fs;
#endif
    for (;;) {
        bool want = i < 0 && !exhausted;
        if (want && budget_spent(a, t_start)) {
            want = false;
            exhausted = true;
        }
        int got = fetch_member(a, want);
        if (want) {
            if (got < 0) {
                exhausted = true;
            } else {
                i = got;
                fresh = true;
            }
        }
        if (__all_sync(0xffffffffu, i < 0))
            break;
        if (i < 0)
            continue;
        // one load site for both a new member and the start of its feature
        // pass, so the right-hand side is inlined here once
        if (fresh || rewind) {
            member_load(m, a, i, c);
            step = 0;
            if (fresh) {
                hmin_fail = false;
                terminal = false;
                t0 = m.t;
                t1 = member_t1(a, i);
                if (a.fused_init) {
                    o.init(m.t, m.x, m.dx, m.aux, a.op);
                    warm = Observer::two_pass;
                    if (!warm)  // one-pass: arm on the initial state, the feature pass starts from it
                        o.arm(m.t, m.x, m.dx, m.aux, a.op);
                } else {
                    park_load(o, a, i);
                    warm = false;
                }
            } else {
                // end of the warm-up pass: arm the detector on the initial
                // state (the arm hooks read the state, not its slope), then
                // run the feature pass from the stored state
                o.arm(m.t, m.x, m.dx, m.aux, a.op);
                warm = false;
            }
            fresh = rewind = false;
#if CLODE_FEATURE_STORE
            if (!warm)  // the feature pass starts here
                fs.start(a, m, i);
#endif
        }
        bool running = true;
        for (int k = 0; k < CLODE_STEP_BLOCK && running; ++k) {
            running = sc.retry || (step < a.sp.max_steps && (warm ? m.t < t1 : m.t <= t1));
            if (!running)
                break;
            if (!sc.retry)
                ++step;
            int flag = step_attempt(m, a.sp, t1, c, sc);
            if (flag == 1) {
                // rejected: retried in the next iteration
            } else if (warm) {
                o.warmup(m.t, m.x, m.dx, m.aux, a.op);
            } else {
                hmin_fail |= flag != 0;
#if CLODE_FEATURE_STORE
                fs.after_step(a, m, i);
#endif
                o.update(m.t, m.x, m.dx, m.aux, a.op);
                if (o.event(m.t, m.x, m.dx, m.aux, a.op)) {
                    c.events++;
#if CLODE_FEATURE_STORE
                    fs.on_event(a, m, i);
#endif
                    if (o.on_event(m.t, m.x, m.dx, m.aux, a.op)) {
                        terminal = true;
                        running = false;
                    }
                }
            }
        }
        if (!running) {
            if (warm) {
                rewind = true;
            } else {
#if CLODE_FEATURE_STORE
                fs.finish(a, i);
#endif
                FOut out = {a.F, (unsigned long long)a.nPts, i, 0};
                o.write(out);
                o.rebase(m.t - t0);
                member_store(m, a, i);
                park_store(o, a, i);
                if (a.status)
                    a.status[i] = member_status_bits(m, step, a, t1, hmin_fail, terminal);
                i = -1;
            }
        }
    }
    flush_counters(a, c);
}
#endif  // CLODE_HAVE_OBSERVER

}  // namespace clode
