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

// Register cap of the ensemble kernels (the host's maxrregcount option), set
// per kernel so that the replay kernel can keep its own.
#if defined(CLODE_MAXNREG) && CLODE_MAXNREG > 0
#define CLODE_CAP __maxnreg__(CLODE_MAXNREG)
#else
#define CLODE_CAP
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
    m.tlo = ZERO;
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
    m.noise = a.noise ? a.noise + (unsigned long long)i * a.noise_stride : nullptr;
#pragma unroll
    for (int j = 0; j < N_WIENER; ++j)
        m.w[j] = draw_normal(m) / m.sqdt;
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
    if (!a.noise) {  // with pre-drawn deviates the draw launch stored the final RNG words
        a.rng[i] = m.r.s0;
        a.rng[n + i] = m.r.s1;
    }
#endif
    a.dt[i] = m.dt;
    a.tf[i] = m.t;
}

__device__ __forceinline__ int status_bits(realtype t, const realtype (&x)[N_VAR], unsigned int step, const Args &a,
                                           realtype t1, bool hmin_fail, bool terminal)
{
    int s = 0;
    if (hmin_fail) s |= STATUS_HMIN_FAIL;
    if (terminal) s |= STATUS_TERMINAL_EVENT;
    bool finite = isfinite(t);
#pragma unroll
    for (int j = 0; j < N_VAR; ++j)
        finite = finite && isfinite(x[j]);
    if (!finite) s |= STATUS_NONFINITE;
    if (!terminal && step >= a.sp.max_steps && t <= t1) s |= STATUS_MAX_STEPS;
    return s;
}

__device__ __forceinline__ int member_status_bits(const Member &m, unsigned int step, const Args &a,
                                                  realtype t1, bool hmin_fail, bool terminal)
{
    return status_bits(m.t, m.x, step, a, t1, hmin_fail, terminal);
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
    while (t_le(m, t1) && step < a.sp.max_steps) {
        ++step;
        hmin_fail |= step_member(m, a.sp, t1, c) != 0;
    }
    member_store(m, a, i);
    if (a.status)
        a.status[i] = member_status_bits(m, step, a, t1, hmin_fail, false);
}

extern "C" __global__ void CLODE_CAP clode_transient(const Args a)
{
    Counters c = {0, 0, 0, 0};
    int i = a.i_begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (i < a.i_end)
        run_transient(a, i, c);
    flush_counters(a, c);
}

// transient, persistent schedule: each lane refills itself as its member ends
extern "C" __global__ void CLODE_CAP clode_transient_persistent(const Args a)
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
            running = sc.retry || (t_le(m, t1) && step < a.sp.max_steps);
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
    while (t_le(m, t1) && step < a.sp.max_steps && row < (unsigned long long)a.sp.max_store) {
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

extern "C" __global__ void CLODE_CAP clode_trajectory(const Args a)
{
    Counters c = {0, 0, 0, 0};
    int i = a.i_begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (i < a.i_end)
        run_trajectory(a, i, c);
    flush_counters(a, c);
}

// trajectory, persistent schedule
extern "C" __global__ void CLODE_CAP clode_trajectory_persistent(const Args a)
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
            running = sc.retry || (t_le(m, t1) && step < a.sp.max_steps && row < (unsigned long long)a.sp.max_store);
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

#if CLODE_STOCHASTIC
// ------------------------------------------------- pre-drawn deviates --
// A stochastic trajectory run draws its members' normal deviates in two
// launches before it integrates: the count launch replays each member's
// step loop on time alone (run_trajectory's conditions: t <= t1, max_steps,
// max_store) to find how many deviates the member takes (one per noise
// variable at the start and per step); the draw launch then produces each
// member's deviates in order, with CLODE_NOISE_LANES lanes per member.  The
// member's stream is cut into blocks of noise_block candidates of the polar
// method (two uniforms each); lane l starts at block l (the stream jumped
// ahead by l blocks, a GF(2) matrix of the generator, noise_mats[l - 1]) and
// after each round jumps L blocks on (noise_mats[L - 1]).  A round takes
// two passes over the lane's block: the first counts its accepted
// candidates, a scan over the member's lanes gives each lane the index of
// its first pair, the second writes the pairs the member takes.  The
// deviates and the final RNG words (the stream after the candidate of the
// last pair taken; an unused second deviate of that pair is the reference's
// cache, dropped at the end of a launch) are those of drawing in the
// integration loop.  Rejected candidates cost nothing beyond their own
// draws, and four lanes per member run where one did.
#define CLODE_NOISE_LANES 4

extern "C" __global__ void clode_noise_count(const Args a)
{
    const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (unsigned long long)a.nPts)
        return;
    Member m;
    m.t = member_t0(a, (int)i);
    m.tlo = ZERO;
    const realtype dt = a.dt[i], t1 = member_t1(a, (int)i);
    unsigned int step = 0, to_store = a.sp.nout;
    unsigned long long row = 0;
    while (t_le(m, t1) && step < a.sp.max_steps && row < (unsigned long long)a.sp.max_store) {
        ++step;
        advance_time(m.t, m.tlo, dt);
        if (--to_store == 0) {
            to_store = a.sp.nout;
            ++row;
        }
    }
    a.noise_count[i] = (step + 1u) * (unsigned int)N_WIENER;
}

// the stream state (s0, s1) times a jump matrix (128 columns of two words)
__device__ __forceinline__ void jump_apply(const unsigned long long (*m)[2], unsigned long long &s0,
                                           unsigned long long &s1)
{
    unsigned long long r0 = 0ull, r1 = 0ull;
#pragma unroll 16
    for (int c = 0; c < 64; ++c) {
        const unsigned long long k = 0ull - ((s0 >> c) & 1ull);
        r0 ^= m[c][0] & k;
        r1 ^= m[c][1] & k;
    }
#pragma unroll 16
    for (int c = 0; c < 64; ++c) {
        const unsigned long long k = 0ull - ((s1 >> c) & 1ull);
        r0 ^= m[64 + c][0] & k;
        r1 ^= m[64 + c][1] & k;
    }
    s0 = r0;
    s1 = r1;
}

extern "C" __global__ void clode_noise_draw(const Args a)
{
    constexpr unsigned int L = CLODE_NOISE_LANES;
    __shared__ unsigned long long mats[L][128][2];
    for (unsigned int k = threadIdx.x; k < L * 256u; k += blockDim.x)
        (&mats[0][0][0])[k] = a.noise_mats[k];
    __syncthreads();
    const unsigned long long n = (unsigned long long)a.nPts;
    const unsigned long long i = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) / L;
    const unsigned int l = threadIdx.x % L;  // blockDim.x is a multiple of 32: a member's lanes share a warp
    const bool live = i < n;
    const unsigned int P = live ? (a.noise_count[i] + 1u) / 2u : 0u;  // pairs the member takes
    Rng r;
    r.s0 = live ? a.rng[i] : 0ull;
    r.s1 = live ? a.rng[n + i] : 0ull;
    if (l > 0 && P > 0)
        jump_apply(mats[l - 1], r.s0, r.s1);
    realtype *out = live ? a.noise + i * a.noise_stride : nullptr;
    const unsigned int C = a.noise_block;
    unsigned int done = 0;  // pairs the member's lanes have produced (the same in its lanes)
    while (__any_sync(0xffffffffu, done < P)) {
        const bool need = done < P;
        unsigned int cnt = 0;
        if (need) {
            Rng q = r;
            for (unsigned int c = 0; c < C; ++c) {
                realtype u, v;
                if (polar_candidate(q, u, v) < ONE)
                    ++cnt;
            }
        }
        unsigned int incl = cnt;
#pragma unroll
        for (unsigned int off = 1; off < L; off <<= 1) {
            const unsigned int t = __shfl_up_sync(0xffffffffu, incl, off, L);
            if (l >= off)
                incl += t;
        }
        const unsigned int total = __shfl_sync(0xffffffffu, incl, L - 1, L);
        unsigned int p = done + incl - cnt;  // this lane's first pair
        if (need && p < P) {
            Rng q = r;
            for (unsigned int c = 0; c < C && p < P; ++c) {
                realtype u, v;
                const realtype s = polar_candidate(q, u, v);
                if (s < ONE) {
                    realtype y1, y2;
                    polar_pair(u, v, s, y1, y2);
                    out[2ull * p] = y1;  // the buffer holds 2P deviates per member
                    out[2ull * p + 1] = y2;
                    if (p == P - 1) {
                        a.rng[i] = q.s0;
                        a.rng[n + i] = q.s1;
                    }
                    ++p;
                }
            }
        }
        done += total;
        if (need)
            jump_apply(mats[L - 1], r.s0, r.s1);
    }
}
#endif  // CLODE_STOCHASTIC

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
        while (t_lt(m, t1) && step < a.sp.max_steps) {
            ++step;
            step_member(m, a.sp, t1, c);
            o.warmup(m.t, m.x, m.dx, m.aux, a.op);
        }
        // rewind to the initial state (the last noise sample is kept)
        m.t = member_t0(a, i);
        m.tlo = ZERO;
        load_x0(m.x, a, i);
        getRHS(m.t, m.x, m.p, m.dx, m.aux, m.w);
        c.rhs += 1;
    }
    o.arm(m.t, m.x, m.dx, m.aux, a.op);
}

extern "C" __global__ void CLODE_CAP clode_init_observer(const Args a)
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
extern "C" __global__ void CLODE_CAP clode_init_observer_persistent(const Args a)
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
            running = sc.retry || (step < a.sp.max_steps && t_lt(m, t1));
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
                m.tlo = ZERO;
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
    while (t_le(m, t1) && step < a.sp.max_steps) {
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

extern "C" __global__ void CLODE_CAP clode_features(const Args a)
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
extern "C" __global__ void CLODE_CAP clode_features_persistent(const Args a)
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
            running = sc.retry || (step < a.sp.max_steps && (warm ? t_lt(m, t1) : t_le(m, t1)));
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

#if !CLODE_FEATURE_STORE
// ---------------------------------------------- replay of the warm-up pass --
// A two-pass observer's feature pass integrates exactly the trajectory its
// warm-up pass integrated (the same start, step sizes and noise: the warm-up
// writes neither dt nor the RNG words back, initializeObserver.cl:57-77).
// Instead of integrating it twice, the recording warm-up launch stores every
// step of the feature pass — the warm-up's steps and, when the warm-up ends
// exactly on t1, the steps the feature pass's `t <= t1` loop takes beyond
// it — and the replay launch feeds them to the observer's feature-pass hooks
// without integrating.  Per member the hooks see the values the feature
// pass would compute, in the same order, so the features, final state, step
// size and RNG words are those of the feature pass.
//
// Rows are warp-wide: in iteration `row` of the recording launch every lane
// of a warp with an accepted step stores it in column `lane`, one
// coalesced 32-lane store per field.  The replay launch has one warp per
// region and walks its rows in order, each lane following the members its
// recording lane held.  A row holds, per step, what the observer's
// warm-up-dependent feature-pass logic reads (Observer::rec_store); the
// recording launch takes the rest of the feature pass (FeatureSums: extent,
// means, step statistics) from the same steps and leaves it in the member's
// finish block.  With the precise option (event times interpolated from
// every state variable and slope) a row holds t, x, dx and aux and the
// replay runs the whole update.
#if defined(CLODE_OBS_SPLIT)
#define CLODE_REC_FIELDS (Observer::split_fields)
#else
#define CLODE_REC_FIELDS (1 + 2 * N_VAR + N_AUX)
#endif

// a member's state at the end of its feature pass
struct Finish {
    realtype t, dt;
    realtype x[N_VAR];
    unsigned long long s0, s1;  // RNG words (stochastic stepper)
    unsigned int steps;         // the feature pass's step counter (the status word's max_steps test)
    unsigned int records;       // stored steps
    unsigned int flags;         // FIN_*
    unsigned int pad;
#if defined(CLODE_OBS_SPLIT)
    FeatureSums fs;  // the feature pass's warm-up-independent accumulators
#endif
};
enum { FIN_COMPLETE = 1, FIN_HMIN_FAIL = 2 };
static_assert(sizeof(Finish) % 4 == 0, "finish block must be a whole number of 32-bit words");
#define CLODE_FIN_WORDS ((int)(sizeof(Finish) / 4))
#define CLODE_FIN_VEC ((CLODE_FIN_WORDS + 3) / 4)
#define CLODE_FIN_STRIDE (4 * CLODE_FIN_VEC)

// read by the host to size the finish blocks (words per member, padding included)
extern "C" __device__ const unsigned int clode_finish_words = CLODE_FIN_STRIDE;
// record fields per step, read by the host to size the regions
extern "C" __device__ const unsigned int clode_record_fields = CLODE_REC_FIELDS;

__device__ __forceinline__ void fin_store(const Finish &f, const Args &a, int i)
{
    uint4 *dst = reinterpret_cast<uint4 *>(a.fin + (unsigned long long)i * CLODE_FIN_STRIDE);
    uint4 v[CLODE_FIN_VEC];
    v[CLODE_FIN_VEC - 1] = make_uint4(0u, 0u, 0u, 0u);
    memcpy(v, &f, sizeof(Finish));
#pragma unroll
    for (int k = 0; k < CLODE_FIN_VEC; ++k)
        dst[k] = v[k];
}

__device__ __forceinline__ void fin_load(Finish &f, const Args &a, int i)
{
    const uint4 *src = reinterpret_cast<const uint4 *>(a.fin + (unsigned long long)i * CLODE_FIN_STRIDE);
    uint4 v[CLODE_FIN_VEC];
#pragma unroll
    for (int k = 0; k < CLODE_FIN_VEC; ++k)
        v[k] = src[k];
    memcpy(&f, v, sizeof(Finish));
}

// members the plain feature pass finishes from their parked observer state
// (fallback[0 .. fallback_count[0]))
__device__ __forceinline__ void fallback_push(const Args &a, int i)
{
    a.fallback[atomicAdd(a.fallback_count, 1u)] = i;
}

// members whose warm-up a full region cut short: the plain warm-up and
// feature passes run them again from the start (fallback[nPts - k], k = 1 ..
// fallback_count[1], from the end of the same list)
__device__ __forceinline__ void rewarm_push(const Args &a, int i)
{
    a.fallback[(unsigned int)a.nPts - 1u - atomicAdd(a.fallback_count + 1, 1u)] = i;
}

// Warm-up pass of the two-pass observers (clode_init_observer_persistent's
// member loop, per member the same steps and hooks) that also records the
// feature pass's steps.  All lanes of a warp iterate together (a lane
// without a step leaves a hole in its column), so every row holds one step
// or none per lane.  A warp takes no new member once rec_fetch_rows rows
// are recorded or its member list is nearly full; the host launches again
// for the members left.  When the region is full the warp stops: the
// members it holds then (their steps did not all fit) go, warm-up unfinished,
// to the list that the plain warm-up and feature passes run again, so that
// no launch waits on a member far longer than its region.  A member that
// takes no step goes to the fallback list and the plain feature pass runs it
// from the parked observer state.
__device__ __forceinline__ void record_body(const Args &a)
{
    Counters c = {0, 0, 0, 0};
    const unsigned int lane = threadIdx.x & 31u;
    const unsigned long long warp = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    // a region's rows fit 32 bits (the host keeps rec_rows below 2^32)
    const unsigned int R = (unsigned int)a.rec_rows;
    const unsigned int fetch_rows = (unsigned int)(a.rec_fetch_rows < a.rec_rows ? a.rec_fetch_rows : a.rec_rows);
    // this lane's column of the current row, advanced one row per iteration
    realtype *col = a.rec + warp * R * (CLODE_REC_FIELDS * 32ull) + lane;
    // the region's masks, stored 32 rows at a time: lane k holds row k's of
    // the current group of 32 (valid lanes, lanes that start a member)
    uint2 *const masks = reinterpret_cast<uint2 *>(a.rec_mask + 2ull * warp * R);
    unsigned int mv = 0u, ms = 0u;
    unsigned int row = 0;     // warp-uniform
    unsigned int starts = 0;  // warp-uniform: members started in this region
    bool full = false;        // warp-uniform: the region has no row left
    bool exhausted = false;
    int i = -1;
    bool fresh = false, tail = false, first = false, hmin_fail = false;
    unsigned int step = 0, records = 0;
    realtype t1 = ZERO;
    Member m;
    Observer o;
#if defined(CLODE_OBS_SPLIT)
    FeatureSums fs;
#endif
    StepCtl sc;
    sc.retry = false;
    for (;;) {
        const bool want = i < 0 && !exhausted && row < fetch_rows && starts + 32u <= a.rec_members;
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
        if (fresh) {
            member_load(m, a, i, c);
            o.init(m.t, m.x, m.dx, m.aux, a.op);
#if defined(CLODE_OBS_SPLIT)
            fs.init(m.t);
#endif
            step = 0;
            records = 0;
            t1 = member_t1(a, i);
            fresh = tail = hmin_fail = false;
            first = true;
        }
        bool running = i >= 0;
        for (int k = 0; k < CLODE_STEP_BLOCK; ++k) {
            if (!__any_sync(0xffffffffu, running))
                break;
            if (row >= R) {
                full = true;
                break;
            }
            bool valid = false;
            if (running) {
                // the warm-up pass runs while t < t1; the feature pass while
                // t <= t1, so it may take steps beyond the warm-up's last one
                bool go = sc.retry || (step < a.sp.max_steps && (tail ? t_le(m, t1) : t_lt(m, t1)));
                if (!go && !tail) {
                    tail = true;
                    go = step < a.sp.max_steps && t_le(m, t1);
                }
                running = go;
                if (go) {
                    if (!sc.retry)
                        ++step;
                    const int flag = step_attempt(m, a.sp, t1, c, sc);
                    if (flag != 1) {
                        valid = true;
                        hmin_fail |= flag != 0;
                        if (!tail)
                            o.warmup(m.t, m.x, m.dx, m.aux, a.op);
                    }
                }
            }
            {
                const unsigned int vmask = __ballot_sync(0xffffffffu, valid);
                const unsigned int smask = __ballot_sync(0xffffffffu, valid && first);
                if (valid) {
                    realtype *r = col;
#if defined(CLODE_OBS_SPLIT)
                    Observer::rec_store(r, m.t, m.x, m.dx, m.aux, a.op);
                    fs.update(m.t, m.x, m.dx, m.aux);
#else
                    r[0] = m.t;
#pragma unroll
                    for (int j = 0; j < N_VAR; ++j)
                        r[(1 + j) * 32] = m.x[j];
#pragma unroll
                    for (int j = 0; j < N_VAR; ++j)
                        r[(1 + N_VAR + j) * 32] = m.dx[j];
#pragma unroll
                    for (int j = 0; j < N_AUX; ++j)
                        r[(1 + 2 * N_VAR + j) * 32] = m.aux[j];
#endif
                    ++records;
                    if (first) {
                        a.rec_member[warp * a.rec_members + starts + __popc(smask & ((1u << lane) - 1u))] = i;
                        first = false;
                    }
                }
                if (lane == (row & 31u)) {
                    mv = vmask;
                    ms = smask;
                }
                if ((row & 31u) == 31u)
                    masks[row - 31u + lane] = make_uint2(mv, ms);
                starts += __popc(smask);
                ++row;
                col += CLODE_REC_FIELDS * 32;
            }
        }
        if (i >= 0 && !running) {
            // the finish block is written for every member, so that the replay
            // never reads one left by an earlier run
            const bool replayable = records > 0;
            Finish f;
            f.t = m.t;
            f.dt = m.dt;
#pragma unroll
            for (int j = 0; j < N_VAR; ++j)
                f.x[j] = m.x[j];
            f.s0 = m.r.s0;
            f.s1 = m.r.s1;
            f.steps = step;
            f.records = records;
            f.flags = replayable ? (FIN_COMPLETE | (hmin_fail ? FIN_HMIN_FAIL : 0)) : 0u;
            f.pad = 0;
#if defined(CLODE_OBS_SPLIT)
            f.fs = fs;
#endif
            fin_store(f, a, i);
            if (!replayable)
                fallback_push(a, i);
            // rewind to the initial state and arm (clode_init_observer_persistent)
            m.t = member_t0(a, i);
            m.tlo = ZERO;
            load_x0(m.x, a, i);
            getRHS(m.t, m.x, m.p, m.dx, m.aux, m.w);
            c.rhs += 1;
            o.arm(m.t, m.x, m.dx, m.aux, a.op);
            park_store(o, a, i);
            i = -1;
        }
        if (full) {
            // the members still running are run again by the plain passes;
            // their finish blocks say so, for the rows they did record
            if (i >= 0) {
                Finish f = {};
                fin_store(f, a, i);
                rewarm_push(a, i);
                i = -1;
            }
            break;
        }
    }
    // the masks of the last, partial group of 32 rows
    if (lane < (row & 31u))
        masks[(row & ~31u) + lane] = make_uint2(mv, ms);
    if (lane == 0)
        a.rec_used[warp] = row < R ? row : R;
    flush_counters(a, c);
}

extern "C" __global__ void CLODE_CAP clode_init_observer_record(const Args a)
{
    record_body(a);
}

// L2 prefetch of a contiguous global range (TMA bulk prefetch; 16-byte
// aligned start, size a multiple of 16 bytes)
__device__ __forceinline__ void prefetch_l2(const void *p, unsigned int bytes)
{
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// rows ahead of the replay that are prefetched into L2, in blocks of this
// many rows (the path without shared-memory stages)
#ifndef CLODE_REPLAY_AHEAD
#define CLODE_REPLAY_AHEAD 8
#endif
#define CLODE_REPLAY_PF_ROWS 4

// The replay launch has the recording launch's number of blocks, each
// replay warp taking one or more regions (rec_regions_per_warp, chosen by
// the host so that the replay's blocks fit on an SM as many at a time as
// the recording launch's): its own register cap keeps the observer state
// in registers.
#ifndef CLODE_REPLAY_MAXNREG
#if defined(CLODE_DOUBLE_PRECISION)
#define CLODE_REPLAY_MAXNREG 255
#elif CLODE_PRECISE
#define CLODE_REPLAY_MAXNREG 216
#else
#define CLODE_REPLAY_MAXNREG 128
#endif
#endif

// ---- shared-memory stages of the replay (TMA bulk copies, mbarriers) ----
// Each warp of the replay owns a ring of rec_stages row slots and two slots
// of 16 rows' masks in dynamic shared memory, each slot with an mbarrier
// that counts the bytes of its copy.  Lane 0 issues one bulk copy
// (cp.async.bulk, global -> shared) per row and one per 16 rows of masks;
// all lanes wait on the slot's barrier, read their column and, once the
// warp has read the slot, lane 0 refills it with the row rec_stages ahead.
// Every wait is bounded: after CLODE_STAGE_WAIT_NS the warp records the
// failure in *rec_error, waits (bounded again) for its copies in flight and
// stops.
#ifndef CLODE_STAGE_WAIT_NS
#define CLODE_STAGE_WAIT_NS 2000000000ull
#endif

// bytes of one warp's stages: rows, two mask slots, the barriers
__device__ __forceinline__ unsigned int stage_bytes(unsigned int stages, unsigned int row_bytes)
{
    return (stages * row_bytes + 256u + 8u * (stages + 2u) + 15u) & ~15u;
}

__device__ __forceinline__ unsigned int smem_addr(const void *p)
{
    unsigned long long s;
    asm("cvta.to.shared.u64 %0, %1;" : "=l"(s) : "l"(p));
    return (unsigned int)s;
}

__device__ __forceinline__ void bar_init(unsigned int bar)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
}

// one bulk copy of `bytes` (a multiple of 16; both addresses 16-byte
// aligned) into shared memory, completing on `bar`
__device__ __forceinline__ void bulk_to_smem(unsigned int dst, const void *src, unsigned int bytes, unsigned int bar)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

__device__ __forceinline__ bool bar_test(unsigned int bar, unsigned int parity)
{
    unsigned int done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    return done != 0u;
}

// wait for the phase of `parity` of `bar`; false after CLODE_STAGE_WAIT_NS
__device__ __forceinline__ bool bar_wait(unsigned int bar, unsigned int parity)
{
    if (bar_test(bar, parity))
        return true;
    const unsigned long long t0 = globaltimer_ns();
    for (;;) {
        if (bar_test(bar, parity))
            return true;
        if (globaltimer_ns() - t0 > CLODE_STAGE_WAIT_NS)
            return false;
    }
}

// The observer's feature-pass hooks for one row of a region, for this lane
// (the replay's per-row step, from whichever copy of the row it read).
struct ReplayLane {
    int i;
    unsigned int left, events, starts;
    Observer o;
};

__device__ __forceinline__ void replay_row(ReplayLane &L, const Args &a, unsigned long long warp, unsigned int lane,
                                           unsigned int vmask, unsigned int smask, realtype t,
                                           const realtype (&x)[N_VAR], const realtype (&dx)[N_VAR],
                                           const realtype (&aux)[NA1], Counters &c)
{
    const unsigned long long n = (unsigned long long)a.nPts;
    if ((smask >> lane) & 1u) {
        const int j = a.rec_member[warp * a.rec_members + L.starts + __popc(smask & ((1u << lane) - 1u))];
        const Finish *fj = reinterpret_cast<const Finish *>(a.fin + (unsigned long long)j * CLODE_FIN_STRIDE);
        L.i = -1;
        if (fj->flags & FIN_COMPLETE) {
            L.i = j;
            L.left = fj->records;
            L.events = 0;
            park_load(L.o, a, L.i);
        }
    }
    L.starts += __popc(smask);
    if (L.i < 0 || !((vmask >> lane) & 1u))
        return;
    const int i = L.i;
#if defined(CLODE_OBS_SPLIT)
    L.o.update_split(t, x, dx, aux, a.op);
#else
    L.o.update(t, x, dx, aux, a.op);
#endif
    if (L.o.event(t, x, dx, aux, a.op)) {
        ++L.events;
        if (L.o.on_event(t, x, dx, aux, a.op)) {
            fallback_push(a, i);
            L.i = -1;
            return;
        }
    }
    if (--L.left == 0) {
        Finish f;
        fin_load(f, a, i);
#if defined(CLODE_OBS_SPLIT)
        {
            Observer armed;  // still parked: the replay stores the state only below
            park_load(armed, a, i);
            L.o.merge(armed, f.fs);
        }
#endif
        FOut out = {a.F, n, i, 0};
        L.o.write(out);
        L.o.rebase(f.t - member_t0(a, i));
#pragma unroll
        for (int j = 0; j < N_VAR; ++j)
            a.xf[j * n + i] = f.x[j];
#if CLODE_STOCHASTIC
        a.rng[i] = f.s0;
        a.rng[n + i] = f.s1;
#endif
        a.dt[i] = f.dt;
        a.tf[i] = f.t;
        park_store(L.o, a, i);
        if (a.status)
            a.status[i] = status_bits(f.t, f.x, f.steps, a, member_t1(a, i), (f.flags & FIN_HMIN_FAIL) != 0, false);
        c.events += L.events;
        L.i = -1;
    }
}

// this lane's column of a row (fields of 32 lanes each, from global or shared memory)
__device__ __forceinline__ void column_load(const realtype *r, realtype &t, realtype (&x)[N_VAR],
                                            realtype (&dx)[N_VAR], realtype (&aux)[NA1], const ObserverParams &op)
{
#if defined(CLODE_OBS_SPLIT)
    Observer::rec_load(r, t, x, dx, aux, op);
#else
    t = r[0];
#pragma unroll
    for (int j = 0; j < N_VAR; ++j)
        x[j] = r[(1 + j) * 32];
#pragma unroll
    for (int j = 0; j < N_VAR; ++j)
        dx[j] = r[(1 + N_VAR + j) * 32];
#pragma unroll
    for (int j = 0; j < NA1; ++j)
        aux[j] = j < N_AUX ? r[(1 + 2 * N_VAR + j) * 32] : ZERO;
#endif
}

// Feature pass by replay: one warp per region of the recording launch (the
// same grid), each lane walking its column.  A member starts where its lane
// recorded its first step, with the observer state parked (armed) by the
// recording launch; it ends at its last stored step with the feature pass's
// final state from its finish block.  A member whose observer ends it early
// (its event limit) goes to the fallback list, since the state at that step
// was not stored whole.  clode_features_replay_staged takes the rows
// through the warp's rec_stages (>= 2) shared-memory stages (dynamic shared
// memory of blockDim.x / 32 times stage_bytes); clode_features_replay
// reads them from global memory, the rows a few steps ahead prefetched
// into L2.
template <bool STAGED>
__device__ __forceinline__ void replay_region(const Args &a, const unsigned long long warp, Counters &c)
{
    extern __shared__ __align__(128) unsigned char replay_smem[];
    const unsigned int lane = threadIdx.x & 31u;
    const unsigned long long R = a.rec_rows;
    const unsigned long long rows = a.rec_used[warp];
    const unsigned int row_bytes = CLODE_REC_FIELDS * 32u * (unsigned int)sizeof(realtype);
    const unsigned int S = a.rec_stages;
    ReplayLane L;
    L.i = -1;
    L.left = L.events = L.starts = 0;
    realtype t, x[N_VAR], dx[N_VAR], aux[NA1];
    if (STAGED) {
        unsigned char *base = replay_smem + (threadIdx.x >> 5) * stage_bytes(S, row_bytes);
        const unsigned int s_rows = smem_addr(base);
        const unsigned int s_masks = s_rows + S * row_bytes;
        const unsigned int s_bars = s_masks + 256u;  // S row barriers, then 2 mask barriers
        const unsigned int *masks = reinterpret_cast<const unsigned int *>(base + S * row_bytes);
        const realtype *region = a.rec + warp * R * (CLODE_REC_FIELDS * 32ull);
        const unsigned int *region_masks = a.rec_mask + 2 * warp * R;
        // rows [0, issued) and mask chunks [0, chunks_issued) have been requested
        unsigned long long issued = 0, chunks_issued = 0;
        const unsigned long long chunks = (rows + 15) / 16;
        __syncwarp();  // (a warp's previous region is done with the stages)
        if (lane == 0 && rows > 0) {
            for (unsigned int k = 0; k < S + 2; ++k)
                bar_init(s_bars + 8u * k);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        __syncwarp();
        if (rows > 0) {
            if (lane == 0) {
                for (; issued < rows && issued < S; ++issued)
                    bulk_to_smem(s_rows + (unsigned int)issued * row_bytes, region + issued * (CLODE_REC_FIELDS * 32ull),
                                 row_bytes, s_bars + 8u * (unsigned int)issued);
                for (; chunks_issued < chunks && chunks_issued < 2; ++chunks_issued)
                    bulk_to_smem(s_masks + 128u * (unsigned int)chunks_issued, region_masks + 32 * chunks_issued, 128u,
                                 s_bars + 8u * (S + (unsigned int)chunks_issued));
            }
            issued = rows < S ? rows : S;
            chunks_issued = chunks < 2 ? chunks : 2;
        }
        // a lane that saw a stage not filled in time processes no more rows;
        // the warp checks for that once per 16 rows and leaves together
        bool ok = true;
        unsigned int slot = 0, phase = 0;  // row % S, (row / S) & 1
        unsigned long long row = 0;
        for (; row < rows; ++row) {
            const unsigned long long chunk = row >> 4;
            if ((row & 15) == 0) {
                if (__any_sync(0xffffffffu, !ok))
                    break;
                ok = bar_wait(s_bars + 8u * (S + (unsigned int)(chunk & 1)), (unsigned int)(chunk >> 1) & 1u);
            }
            if (ok)
                ok = bar_wait(s_bars + 8u * slot, phase);
            const unsigned int *mk = masks + 32u * (unsigned int)(chunk & 1) + 2u * (unsigned int)(row & 15);
            const unsigned int vmask = mk[0], smask = mk[1];
            column_load(reinterpret_cast<const realtype *>(base + slot * row_bytes) + lane, t, x, dx, aux, a.op);
            // the warp has read the slot (and, at a chunk's last row, the
            // chunk's masks): refill them
            __syncwarp();
            if (lane == 0) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                if (issued < rows)
                    bulk_to_smem(s_rows + slot * row_bytes, region + issued * (CLODE_REC_FIELDS * 32ull), row_bytes,
                                 s_bars + 8u * slot);
                if ((row & 15) == 15 && chunks_issued < chunks) {
                    const unsigned int ms = (unsigned int)(chunks_issued & 1);
                    bulk_to_smem(s_masks + 128u * ms, region_masks + 32 * chunks_issued, 128u, s_bars + 8u * (S + ms));
                }
            }
            if (issued < rows)
                ++issued;
            if ((row & 15) == 15 && chunks_issued < chunks)
                ++chunks_issued;
            if (++slot == S) {
                slot = 0;
                phase ^= 1u;
            }
            if (ok)
                replay_row(L, a, warp, lane, vmask, smask, t, x, dx, aux, c);
        }
        if (__any_sync(0xffffffffu, !ok)) {
            // a stage that was not filled in time: record it, and wait (bounded)
            // for every copy this warp still has in flight before leaving
            if (lane == 0) {
                atomicOr(a.rec_error, 1u);
                for (unsigned long long r = row; r < issued; ++r)
                    bar_wait(s_bars + 8u * (unsigned int)(r % S), (unsigned int)(r / S) & 1u);
                for (unsigned long long k = row >> 4; k < chunks_issued; ++k)
                    bar_wait(s_bars + 8u * (S + (unsigned int)(k & 1)), (unsigned int)(k >> 1) & 1u);
            }
            __syncwarp();
        }
        // every copy of this region has completed: the barriers are released
        // for the warp's next region
        __syncwarp();
        if (lane == 0 && rows > 0) {
            for (unsigned int k = 0; k < S + 2; ++k)
                asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(s_bars + 8u * k) : "memory");
        }
    } else {
        // the first rows of the region into L2 (R is a multiple of 16, so every
        // region's masks start on a 16-byte boundary)
        if (lane == 0) {
            const unsigned long long first = rows < CLODE_REPLAY_AHEAD ? rows : CLODE_REPLAY_AHEAD;
            if (first > 0) {
                prefetch_l2(a.rec + warp * R * (CLODE_REC_FIELDS * 32ull), (unsigned int)first * row_bytes);
                prefetch_l2(a.rec_mask + 2 * warp * R, (unsigned int)((first * 8 + 15) / 16 * 16));
            }
        }
        for (unsigned long long row = 0; row < rows; ++row) {
            const unsigned long long cell = warp * R + row;
            // keep CLODE_REPLAY_AHEAD rows in flight: every CLODE_REPLAY_PF_ROWS rows,
            // the block that far ahead (within the rows recorded)
            if (lane == 0 && row % CLODE_REPLAY_PF_ROWS == 0) {
                const unsigned long long ahead = row + CLODE_REPLAY_AHEAD;
                if (ahead < rows) {
                    const unsigned long long cnt =
                        rows - ahead < CLODE_REPLAY_PF_ROWS ? rows - ahead : CLODE_REPLAY_PF_ROWS;
                    prefetch_l2(a.rec + (cell + CLODE_REPLAY_AHEAD) * (CLODE_REC_FIELDS * 32ull),
                                (unsigned int)cnt * row_bytes);
                    // the masks: 8 bytes per row, rounded to whole 16-byte pieces
                    const unsigned long long b0 = (2 * (cell + CLODE_REPLAY_AHEAD) * 4) & ~15ull;
                    const unsigned long long b1 = (2 * (cell + CLODE_REPLAY_AHEAD + cnt) * 4 + 15) & ~15ull;
                    prefetch_l2(reinterpret_cast<const char *>(a.rec_mask) + b0, (unsigned int)(b1 - b0));
                }
            }
            // the row's masks and this lane's column are loaded together, before
            // anything depends on them, so a row costs one memory latency (a
            // hole in the column is loaded too, and ignored)
            const unsigned int vmask = a.rec_mask[2 * cell];
            const unsigned int smask = a.rec_mask[2 * cell + 1];
            column_load(a.rec + cell * (CLODE_REC_FIELDS * 32ull) + lane, t, x, dx, aux, a.op);
            replay_row(L, a, warp, lane, vmask, smask, t, x, dx, aux, c);
        }
    }
}

// A replay warp takes rec_regions_per_warp consecutive regions in turn, so
// that a replay block of blockDim.x threads covers the regions of a
// recording block of rec_regions_per_warp times as many: the replay's
// registers are not bound by the recording launch's residency.
template <bool STAGED>
__device__ __forceinline__ void features_replay(const Args &a)
{
    Counters c = {0, 0, 0, 0};
    const unsigned long long w = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned int k = a.rec_regions_per_warp > 0 ? a.rec_regions_per_warp : 1u;
    for (unsigned int j = 0; j < k; ++j)
        replay_region<STAGED>(a, w * k + j, c);
    flush_counters(a, c);
}

extern "C" __global__ void __maxnreg__(CLODE_REPLAY_MAXNREG) clode_features_replay(const Args a)
{
    features_replay<false>(a);
}

extern "C" __global__ void __maxnreg__(CLODE_REPLAY_MAXNREG) clode_features_replay_staged(const Args a)
{
    features_replay<true>(a);
}

// Recording and replay in one launch: each warp records its region, then
// replays it (rows from global memory), so that a warp whose region is done
// replays it while others still record, and a launch pair has one end
// instead of two.  The warp's lanes wrote every row, mask, member list entry
// and finish block it reads: __syncwarp orders those writes before the reads.
extern "C" __global__ void CLODE_CAP clode_features_record_replay(const Args a)
{
    record_body(a);
    __syncwarp();
    Counters c = {0, 0, 0, 0};
    replay_region<false>(a, ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5, c);
    flush_counters(a, c);
}
#endif  // !CLODE_FEATURE_STORE
#endif  // CLODE_HAVE_OBSERVER

}  // namespace clode
