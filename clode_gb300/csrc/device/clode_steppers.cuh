// Time steppers.  Each member's state lives in registers (N_VAR, N_PAR, ...
// are compile-time constants, so every array below is fully unrolled).
//
// Arithmetic follows the reference operation by operation, so that with
// --fmad=false the results are bitwise those of clODE's kernels:
//   Euler / stochastic Euler  clode/cpp/steppers/fixed_explicit_Euler.clh:5-18
//   Heun                      clode/cpp/steppers/fixed_explicit_Trapezoidal.clh:5-23
//   RK4                       clode/cpp/steppers/fixed_explicit_RK4.clh:5-40
//   fixed-step wrapper        clode/cpp/steppers/fixed_explicit_step.clh:9-37
//   BS23                      clode/cpp/steppers/adaptive_bs23.clh:27-63
//   Dormand-Prince 5(4)       clode/cpp/steppers/adaptive_dp45.clh:10-111
//   step-size controller      clode/cpp/steppers/adaptive_explicit_step.clh:4-81
// Tableau entries are written as the same quotients the reference's macros
// expand to; the compiler rounds each quotient once to working precision.
#pragma once

namespace clode {

// ------------------------------------------------------- precise option --
// CLODE_PRECISE = 1 builds the engine's precision option (no counterpart in
// the reference, not for parity): time accumulated as a compensated pair,
// the adaptive controller's error estimate as a compensated dot product,
// compensated time-weighted means and refined event times in the observers.
// The error-free transformations below use explicitly rounded operations,
// which the compiler never contracts or reassociates, so they hold in the
// fmad / fast builds too.
#ifndef CLODE_PRECISE
#define CLODE_PRECISE 0
#endif

// (add_rn and mul_rn come with the RNG, clode_rng.cuh)
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }

// s + e = a + b exactly (Knuth's TwoSum)
__device__ __forceinline__ void two_sum(realtype a, realtype b, realtype &s, realtype &e)
{
    s = add_rn(a, b);
    const realtype bp = sub_rn(s, a);
    e = add_rn(sub_rn(a, sub_rn(s, bp)), sub_rn(b, bp));
}

// compensated sum (hi, lo): adds v with its rounding error kept in lo
struct CSum {
    realtype hi, lo;
    __device__ __forceinline__ void reset() { hi = ZERO; lo = ZERO; }
    __device__ __forceinline__ void add(realtype v)
    {
        realtype s, e;
        two_sum(hi, v, s, e);
        hi = s;
        lo = add_rn(lo, e);
    }
    // adds a * b: the product's rounding error (exact through an fma) joins lo
    __device__ __forceinline__ void add_prod(realtype a, realtype b)
    {
        const realtype p = mul_rn(a, b);
        const realtype pe = fma_rn(a, b, -p);
        realtype s, e;
        two_sum(hi, p, s, e);
        hi = s;
        lo = add_rn(lo, add_rn(e, pe));
    }
    __device__ __forceinline__ realtype value() const { return add_rn(hi, lo); }
};

#define NP1 (N_PAR > 0 ? N_PAR : 1)
#define NA1 (N_AUX > 0 ? N_AUX : 1)
#define NW1 (N_WIENER > 0 ? N_WIENER : 1)

#if defined(STOCHASTIC_EULER)
#define CLODE_STOCHASTIC 1
#else
#define CLODE_STOCHASTIC 0
#endif

struct Member {
    realtype t, dt;
    realtype tlo;  // CLODE_PRECISE: the time is t + tlo, |tlo| <= half an ulp of t
    realtype p[NP1];
    realtype x[N_VAR];
    realtype dx[N_VAR];
    realtype aux[NA1];
    realtype w[NW1];
    Rng r;
#if CLODE_STOCHASTIC
    realtype sqdt;  // sqrt(dt), fixed for the whole launch: the stochastic stepper never changes dt
    const realtype *noise;  // this member's pre-drawn deviates, next first (null: drawn here)
#endif
};

#if CLODE_STOCHASTIC
// the member's next normal deviate: pre-drawn by the draw launch, or drawn
// from its stream here (the same sequence either way)
__device__ __forceinline__ realtype draw_normal(Member &m)
{
    if (m.noise)
        return *m.noise++;
    return rng_normal(m.r);
}
#endif

// per-thread work counters, summed into ArgsT::stats at the end of a member
struct Counters {
    unsigned int steps, rejected, rhs, events;
};

typedef SolverParamsT<realtype> SolverParams;

// the member's time against the end of its span: t < t1 and t <= t1, with
// the compensated time of the precise option
__device__ __forceinline__ bool t_lt(const Member &m, realtype t1)
{
#if CLODE_PRECISE
    return m.t < t1 || (m.t == t1 && m.tlo < ZERO);
#else
    return m.t < t1;
#endif
}

__device__ __forceinline__ bool t_le(const Member &m, realtype t1)
{
#if CLODE_PRECISE
    return m.t < t1 || (m.t == t1 && m.tlo <= ZERO);
#else
    return m.t <= t1;
#endif
}

// t (+ tlo) advanced by dt: naively as the reference (t += dt), or, precise,
// as a compensated pair renormalised so that t is the time rounded to
// working precision
__device__ __forceinline__ void advance_time(realtype &t, realtype &tlo, realtype dt)
{
#if CLODE_PRECISE
    realtype s, e;
    two_sum(t, dt, s, e);
    e = add_rn(e, tlo);
    t = add_rn(s, e);
    tlo = sub_rn(e, sub_rn(t, s));
#else
    t += dt;
#endif
}

#if defined(EXPLICIT_EULER) || defined(STOCHASTIC_EULER) || defined(EXPLICIT_HEUN) || defined(EXPLICIT_RK4)
#define CLODE_FIXED_STEP 1

#if defined(EXPLICIT_EULER) || defined(STOCHASTIC_EULER)
#define CLODE_RHS_PER_STEP 1
#elif defined(EXPLICIT_HEUN)
#define CLODE_RHS_PER_STEP 2
#else
#define CLODE_RHS_PER_STEP 4
#endif

__device__ __forceinline__ void fixed_do_step(realtype &t, realtype &tlo, realtype (&x)[N_VAR],
                                              const realtype (&k1)[N_VAR], const realtype (&p)[NP1],
                                              const realtype dt, realtype (&aux)[NA1], const realtype (&w)[NW1])
{
#if defined(EXPLICIT_EULER) || defined(STOCHASTIC_EULER)
#pragma unroll
    for (int k = 0; k < N_VAR; ++k)
        x[k] += dt * k1[k];
    advance_time(t, tlo, dt);
#elif defined(EXPLICIT_HEUN)
#if CLODE_PRECISE
    realtype tn = t, tnlo = tlo;
    advance_time(tn, tnlo, dt);
#else
    realtype tn = t + dt;
#endif
    realtype xp[N_VAR], k2[N_VAR];
#pragma unroll
    for (int k = 0; k < N_VAR; ++k)
        xp[k] = fma(dt, k1[k], x[k]);
    getRHS(tn, xp, p, k2, aux, w);
#pragma unroll
    for (int k = 0; k < N_VAR; ++k)
        x[k] += dt * RCONST(0.5) * (k1[k] + k2[k]);
    t = tn;
#if CLODE_PRECISE
    tlo = tnlo;
#endif
#else
    realtype xs[N_VAR], k2[N_VAR], k3[N_VAR], k4[N_VAR];
    realtype half = dt * RCONST(0.5);
    realtype tm = t + half;
#if CLODE_PRECISE
    realtype te = t, telo = tlo;
    advance_time(te, telo, dt);
#else
    realtype te = t + dt;
#endif
#pragma unroll
    for (int k = 0; k < N_VAR; ++k)
        xs[k] = x[k] + half * k1[k];
    getRHS(tm, xs, p, k2, aux, w);
#pragma unroll
    for (int k = 0; k < N_VAR; ++k)
        xs[k] = x[k] + half * k2[k];
    getRHS(tm, xs, p, k3, aux, w);
#pragma unroll
    for (int k = 0; k < N_VAR; ++k)
        xs[k] = x[k] + dt * k3[k];
    getRHS(te, xs, p, k4, aux, w);
#pragma unroll
    for (int k = 0; k < N_VAR; ++k)
        x[k] += dt * (k1[k] + RCONST(2.0) * k2[k] + RCONST(2.0) * k3[k] + k4[k]) / RCONST(6.0);
    t = te;
#if CLODE_PRECISE
    tlo = telo;
#endif
#endif
}

// one fixed step; afterwards m.dx holds f(t_new, x_new) with fresh noise
__device__ __forceinline__ int step_member(Member &m, const SolverParams &sp, const realtype t1, Counters &c)
{
    fixed_do_step(m.t, m.tlo, m.x, m.dx, m.p, m.dt, m.aux, m.w);
#if CLODE_STOCHASTIC
#pragma unroll
    for (int j = 0; j < N_WIENER; ++j)
        m.w[j] = draw_normal(m) / m.sqdt;  // randn / sqrt(dt), fixed_explicit_step.clh:29-33
#endif
    getRHS(m.t, m.x, m.p, m.dx, m.aux, m.w);
    c.steps++;
    c.rhs += CLODE_RHS_PER_STEP;
    return 0;
}

// retry state of a step spread over several calls (adaptive steppers only)
struct StepCtl {
    bool retry;
};

// one attempt of a step; a fixed step never asks for a retry
__device__ __forceinline__ int step_attempt(Member &m, const SolverParams &sp, const realtype t1, Counters &c,
                                            StepCtl &s)
{
    s.retry = false;
    return step_member(m, sp, t1, c);
}

#elif defined(EXPLICIT_BS23) || defined(EXPLICIT_DOPRI5)
#define CLODE_FIXED_STEP 0

#if defined(EXPLICIT_BS23)
#define CLODE_ERR_ORDER RCONST(2.0)
#define CLODE_MAX_SHRINK RCONST(0.5)
#define CLODE_MAX_GROW RCONST(5.0)
#define CLODE_RHS_PER_ATTEMPT 3

// returns the effective step tnew - t; x, k1 (FSAL) and t advance in place
__device__ __forceinline__ realtype attempt(realtype &t, realtype (&x)[N_VAR], realtype (&k1)[N_VAR],
                                            const realtype (&p)[NP1], const realtype dt, realtype (&aux)[NA1],
                                            realtype (&err)[N_VAR], const realtype (&w)[NW1])
{
    const realtype b1 = RCONST(2.0) / RCONST(9.0), b2 = RCONST(1.0) / RCONST(3.0), b3 = RCONST(4.0) / RCONST(9.0);
    const realtype e1 = RCONST(-5.0) / RCONST(72.0), e2 = RCONST(1.0) / RCONST(12.0);
    const realtype e3 = RCONST(1.0) / RCONST(9.0), e4 = RCONST(-1.0) / RCONST(8.0);
    realtype tn = t + dt;
    realtype h = tn - t;
    realtype xs[N_VAR], k2[N_VAR], k3[N_VAR], k4[N_VAR];
#pragma unroll
    for (int k = 0; k < N_VAR; ++k)
        xs[k] = x[k] + h * RCONST(0.5) * k1[k];
    getRHS(t + h * RCONST(0.5), xs, p, k2, aux, w);
#pragma unroll
    for (int k = 0; k < N_VAR; ++k)
        xs[k] = x[k] + h * RCONST(0.75) * k2[k];
    getRHS(t + h * RCONST(0.75), xs, p, k3, aux, w);
#pragma unroll
    for (int k = 0; k < N_VAR; ++k)
        x[k] = x[k] + h * (b1 * k1[k] + b2 * k2[k] + b3 * k3[k]);
    getRHS(tn, x, p, k4, aux, w);
#pragma unroll
    for (int k = 0; k < N_VAR; ++k) {
#if CLODE_PRECISE
        CSum cs;
        cs.reset();
        cs.add_prod(e1, k1[k]);
        cs.add_prod(e2, k2[k]);
        cs.add_prod(e3, k3[k]);
        cs.add_prod(e4, k4[k]);
        err[k] = h * cs.value();
#else
        err[k] = h * (e1 * k1[k] + e2 * k2[k] + e3 * k3[k] + e4 * k4[k]);
#endif
        k1[k] = k4[k];
    }
    t = tn;
    return h;
}
#else
#define CLODE_ERR_ORDER RCONST(4.0)
#define CLODE_MAX_SHRINK RCONST(0.1)
#define CLODE_MAX_GROW RCONST(5.0)
#define CLODE_RHS_PER_ATTEMPT 6

// ---------------------------------------------- paired stage arithmetic --
// sm_100 and later add, multiply and fma two FP32 values in one instruction
// (f32x2 operands in a 64-bit register pair).  A Runge-Kutta stage applies
// the same combination to every state variable, so in FP32 builds that
// allow contraction (--fmad=true, CLODE_FMAD = 1) the Dormand-Prince stage
// sums take two variables per instruction (CLODE_PAIRED = 1, the default)
// and an odd last variable alone, in one fixed pattern: c1 * k1, then
// fma(c_i, k_i, s) for each further term, and x + h * s as fma(h, s, x).
// The build that reproduces the reference bit for bit (--fmad=false) keeps
// the scalar stage sums: the device compiler fuses a paired multiply into
// the paired add that uses it even under --fmad=false and in PTX with an
// explicit rounding mode (measured on random operands: x + a * (b * b) in
// paired operations differs from the scalar __fadd_rn / __fmul_rn form in
// 1.4 % of cases, while each paired operation alone matches its scalar form
// bit for bit), so separately rounded paired sums cannot be guaranteed.
#ifndef CLODE_PAIRED
#define CLODE_PAIRED 1
#endif
#ifndef CLODE_FMAD
#define CLODE_FMAD 0
#endif
#ifndef CLODE_FTZ
#define CLODE_FTZ 0
#endif
#if defined(CLODE_SINGLE_PRECISION) && CLODE_PAIRED && CLODE_FMAD && !CLODE_PRECISE && N_VAR >= 2
#define CLODE_PAIRED_STAGES 1

#if CLODE_FTZ
#define CLODE_F32X2 ".rn.ftz.f32x2"
#else
#define CLODE_F32X2 ".rn.f32x2"
#endif

// a * b and a * b + c on two lanes (round to nearest, flushed to zero as the
// scalar operations of the build)
__device__ __forceinline__ float2 pmul(float2 a, float2 b)
{
    float2 r;
    asm("{\n\t.reg .b64 pa, pb, pd;\n\t"
        "mov.b64 pa, {%2, %3};\n\t"
        "mov.b64 pb, {%4, %5};\n\t"
        "mul" CLODE_F32X2 " pd, pa, pb;\n\t"
        "mov.b64 {%0, %1}, pd;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}

__device__ __forceinline__ float2 pfma(float2 a, float2 b, float2 c)
{
    float2 r;
    asm("{\n\t.reg .b64 pa, pb, pc, pd;\n\t"
        "mov.b64 pa, {%2, %3};\n\t"
        "mov.b64 pb, {%4, %5};\n\t"
        "mov.b64 pc, {%6, %7};\n\t"
        "fma" CLODE_F32X2 " pd, pa, pb, pc;\n\t"
        "mov.b64 {%0, %1}, pd;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return r;
}

__device__ __forceinline__ float2 pair_of(const float (&a)[N_VAR], int j) { return make_float2(a[j], a[j + 1]); }
__device__ __forceinline__ float2 pair_bcast(float c) { return make_float2(c, c); }

// the further terms of a stage sum over variables j, j+1
__device__ __forceinline__ float2 pair_terms(int, float2 s) { return s; }
template <typename... R>
__device__ __forceinline__ float2 pair_terms(int j, float2 s, float c, const float (&k)[N_VAR], const R &...rest)
{
    return pair_terms(j, pfma(pair_bcast(c), pair_of(k, j), s), rest...);
}

// the same for a single variable j
__device__ __forceinline__ float single_terms(int, float s) { return s; }
template <typename... R>
__device__ __forceinline__ float single_terms(int j, float s, float c, const float (&k)[N_VAR], const R &...rest)
{
    return single_terms(j, __fmaf_rn(c, k[j], s), rest...);
}

// y = x + h * (c1 * k1 + c2 * k2 + ...) per variable (y may be x)
template <typename... R>
__device__ __forceinline__ void stage_sum(float (&y)[N_VAR], const float (&x)[N_VAR], float h, float c1,
                                          const float (&k1)[N_VAR], const R &...rest)
{
#pragma unroll
    for (int j = 0; j + 1 < N_VAR; j += 2) {
        const float2 s = pair_terms(j, pmul(pair_bcast(c1), pair_of(k1, j)), rest...);
        const float2 v = pfma(pair_bcast(h), s, pair_of(x, j));
        y[j] = v.x;
        y[j + 1] = v.y;
    }
    if (N_VAR & 1) {
        const int j = N_VAR - 1;
        y[j] = __fmaf_rn(h, single_terms(j, __fmul_rn(c1, k1[j]), rest...), x[j]);
    }
}

// y = h * (c1 * k1 + c2 * k2 + ...) per variable
template <typename... R>
__device__ __forceinline__ void scaled_sum(float (&y)[N_VAR], float h, float c1, const float (&k1)[N_VAR],
                                           const R &...rest)
{
#pragma unroll
    for (int j = 0; j + 1 < N_VAR; j += 2) {
        const float2 v = pmul(pair_bcast(h), pair_terms(j, pmul(pair_bcast(c1), pair_of(k1, j)), rest...));
        y[j] = v.x;
        y[j + 1] = v.y;
    }
    if (N_VAR & 1) {
        const int j = N_VAR - 1;
        y[j] = __fmul_rn(h, single_terms(j, __fmul_rn(c1, k1[j]), rest...));
    }
}
#else
#define CLODE_PAIRED_STAGES 0
#endif

__device__ __forceinline__ realtype attempt(realtype &t, realtype (&x)[N_VAR], realtype (&k1)[N_VAR],
                                            const realtype (&p)[NP1], const realtype dt, realtype (&aux)[NA1],
                                            realtype (&err)[N_VAR], const realtype (&w)[NW1])
{
    const realtype a2 = RCONST(1.0) / RCONST(5.0), a3 = RCONST(3.0) / RCONST(10.0);
    const realtype a4 = RCONST(4.0) / RCONST(5.0), a5 = RCONST(8.0) / RCONST(9.0);
    const realtype b21 = RCONST(1.0) / RCONST(5.0);
    const realtype b31 = RCONST(3.0) / RCONST(40.0), b32 = RCONST(9.0) / RCONST(40.0);
    const realtype b41 = RCONST(44.0) / RCONST(45.0), b42 = RCONST(-56.0) / RCONST(15.0);
    const realtype b43 = RCONST(32.0) / RCONST(9.0);
    const realtype b51 = RCONST(19372.0) / RCONST(6561.0), b52 = RCONST(-25360.0) / RCONST(2187.0);
    const realtype b53 = RCONST(64448.0) / RCONST(6561.0), b54 = RCONST(-212.0) / RCONST(729.0);
    const realtype b61 = RCONST(9017.0) / RCONST(3168.0), b62 = RCONST(-355.0) / RCONST(33.0);
    const realtype b63 = RCONST(46732.0) / RCONST(5247.0), b64 = RCONST(49.0) / RCONST(176.0);
    const realtype b65 = RCONST(-5103.0) / RCONST(18656.0);
    const realtype c1 = RCONST(35.0) / RCONST(384.0), c3 = RCONST(500.0) / RCONST(1113.0);
    const realtype c4 = RCONST(125.0) / RCONST(192.0), c5 = RCONST(-2187.0) / RCONST(6784.0);
    const realtype c6 = RCONST(11.0) / RCONST(84.0);
    const realtype e1 = RCONST(71.0) / RCONST(57600.0), e3 = RCONST(-71.0) / RCONST(16695.0);
    const realtype e4 = RCONST(71.0) / RCONST(1920.0), e5 = RCONST(-17253.0) / RCONST(339200.0);
    const realtype e6 = RCONST(22.0) / RCONST(525.0), e7 = RCONST(-1.0) / RCONST(40.0);

    realtype tn = t + dt;
    realtype h = tn - t;
    realtype xs[N_VAR], k2[N_VAR], k3[N_VAR], k4[N_VAR], k5[N_VAR], k6[N_VAR], k7[N_VAR];
#if CLODE_PAIRED_STAGES
    stage_sum(xs, x, h, b21, k1);
    getRHS(t + a2 * h, xs, p, k2, aux, w);
    stage_sum(xs, x, h, b31, k1, b32, k2);
    getRHS(t + a3 * h, xs, p, k3, aux, w);
    stage_sum(xs, x, h, b41, k1, b42, k2, b43, k3);
    getRHS(t + a4 * h, xs, p, k4, aux, w);
    stage_sum(xs, x, h, b51, k1, b52, k2, b53, k3, b54, k4);
    getRHS(t + a5 * h, xs, p, k5, aux, w);
    stage_sum(xs, x, h, b61, k1, b62, k2, b63, k3, b64, k4, b65, k5);
    getRHS(t + h, xs, p, k6, aux, w);
    stage_sum(x, x, h, c1, k1, c3, k3, c4, k4, c5, k5, c6, k6);
    getRHS(tn, x, p, k7, aux, w);
    scaled_sum(err, h, e1, k1, e3, k3, e4, k4, e5, k5, e6, k6, e7, k7);
#pragma unroll
    for (int k = 0; k < N_VAR; ++k)
        k1[k] = k7[k];
#else
#pragma unroll
    for (int k = 0; k < N_VAR; ++k)
        xs[k] = x[k] + h * (b21 * k1[k]);
    getRHS(t + a2 * h, xs, p, k2, aux, w);
#pragma unroll
    for (int k = 0; k < N_VAR; ++k)
        xs[k] = x[k] + h * (b31 * k1[k] + b32 * k2[k]);
    getRHS(t + a3 * h, xs, p, k3, aux, w);
#pragma unroll
    for (int k = 0; k < N_VAR; ++k)
        xs[k] = x[k] + h * (b41 * k1[k] + b42 * k2[k] + b43 * k3[k]);
    getRHS(t + a4 * h, xs, p, k4, aux, w);
#pragma unroll
    for (int k = 0; k < N_VAR; ++k)
        xs[k] = x[k] + h * (b51 * k1[k] + b52 * k2[k] + b53 * k3[k] + b54 * k4[k]);
    getRHS(t + a5 * h, xs, p, k5, aux, w);
#pragma unroll
    for (int k = 0; k < N_VAR; ++k)
        xs[k] = x[k] + h * (b61 * k1[k] + b62 * k2[k] + b63 * k3[k] + b64 * k4[k] + b65 * k5[k]);
    getRHS(t + h, xs, p, k6, aux, w);
#pragma unroll
    for (int k = 0; k < N_VAR; ++k)
        x[k] = x[k] + h * (c1 * k1[k] + c3 * k3[k] + c4 * k4[k] + c5 * k5[k] + c6 * k6[k]);
    getRHS(tn, x, p, k7, aux, w);
#pragma unroll
    for (int k = 0; k < N_VAR; ++k) {
#if CLODE_PRECISE
        CSum cs;
        cs.reset();
        cs.add_prod(e1, k1[k]);
        cs.add_prod(e3, k3[k]);
        cs.add_prod(e4, k4[k]);
        cs.add_prod(e5, k5[k]);
        cs.add_prod(e6, k6[k]);
        cs.add_prod(e7, k7[k]);
        err[k] = h * cs.value();
#else
        err[k] = h * (e1 * k1[k] + e3 * k3[k] + e4 * k4[k] + e5 * k5[k] + e6 * k6[k] + e7 * k7[k]);
#endif
        k1[k] = k7[k];
    }
#endif
    t = tn;
    return h;
}
#endif

// adaptive step with error control; returns -1 when the step fails at hmin
// (the reference ignores that flag and keeps stepping; the caller records it)
__device__ __forceinline__ int step_member(Member &m, const SolverParams &sp, const realtype t1, Counters &c)
{
    const realtype safety = RCONST(0.8);
    const realtype expon = RCONST(1.0) / (CLODE_ERR_ORDER + RCONST(1.0));
    realtype tn, nerr = ZERO;
    realtype err[N_VAR], xn[N_VAR], kn[N_VAR];
    realtype h = m.dt;
    const realtype threshold = sp.abstol / sp.reltol;
    const realtype hmin = RCONST(16.0) * fabs(fabs(nextafter(m.t, RCONST(1.1) * t1)) - m.t);
    bool first_try = true;
    for (;;) {
        tn = m.t;
#pragma unroll
        for (int j = 0; j < N_VAR; ++j) {
            xn[j] = m.x[j];
            kn[j] = m.dx[j];
        }
        h = clamp(h, hmin, sp.dtmax);
        h = attempt(tn, xn, kn, m.p, h, m.aux, err, m.w);
        c.rhs += CLODE_RHS_PER_ATTEMPT;
#pragma unroll
        for (int j = 0; j < N_VAR; ++j)
            err[j] /= fmax(fmax(fabs(m.x[j]), fabs(xn[j])), threshold);
        nerr = ZERO;
#pragma unroll
        for (int j = 0; j < N_VAR; ++j)
            nerr = fmax(fabs(err[j]), nerr);
        if (!(nerr > sp.reltol))
            break;
        c.rejected++;
        if (h <= hmin) {
            m.dt = hmin;
            c.steps++;
            return -1;
        }
        if (first_try) {
            first_try = false;
            h *= fmax(CLODE_MAX_SHRINK, safety * pow(sp.reltol / nerr, expon));
        } else {
            h *= RCONST(0.5);
        }
    }
    if (first_try)
        h *= fmin(CLODE_MAX_GROW, safety * pow(sp.reltol / nerr, expon));
    h = fmin(h, t1 - tn);
    h = clamp(h, hmin, sp.dtmax);
    m.dt = h;
    m.t = tn;
#pragma unroll
    for (int j = 0; j < N_VAR; ++j) {
        m.x[j] = xn[j];
        m.dx[j] = kn[j];
    }
    c.steps++;
    return 0;
}
// The same controller as step_member, one attempt per call, so that in the
// persistent kernels a lane whose attempt is rejected retries in the next
// iteration of the member loop while the other lanes of its warp go on with
// their next steps (no warp-wide repeat of the attempt).  Per member the
// operations and their order are those of step_member.
struct StepCtl {
    realtype h;     // step size of the next attempt (before clamping)
    realtype hmin;  // 16 ulp of t at the start of the step
    bool retry;     // an attempt of this step was rejected
    bool first_try;
};

// returns 0 when the step was accepted, 1 when it was rejected and must be
// retried (state unchanged), -1 when it failed at hmin (as step_member).
// Built with CLODE_SPLIT_ATTEMPTS=0 it runs the whole step (step_member) and
// never asks for a retry; which is faster depends on the model and build.
__device__ __forceinline__ int step_attempt(Member &m, const SolverParams &sp, const realtype t1, Counters &c,
                                            StepCtl &s)
{
#if !CLODE_SPLIT_ATTEMPTS
    s.retry = false;
    return step_member(m, sp, t1, c);
#endif
    const realtype safety = RCONST(0.8);
    const realtype expon = RCONST(1.0) / (CLODE_ERR_ORDER + RCONST(1.0));
    if (!s.retry) {
        s.h = m.dt;
        s.hmin = RCONST(16.0) * fabs(fabs(nextafter(m.t, RCONST(1.1) * t1)) - m.t);
        s.first_try = true;
    }
    const realtype threshold = sp.abstol / sp.reltol;
    realtype tn = m.t, nerr = ZERO;
    realtype err[N_VAR], xn[N_VAR], kn[N_VAR];
#pragma unroll
    for (int j = 0; j < N_VAR; ++j) {
        xn[j] = m.x[j];
        kn[j] = m.dx[j];
    }
    realtype h = clamp(s.h, s.hmin, sp.dtmax);
    h = attempt(tn, xn, kn, m.p, h, m.aux, err, m.w);
    c.rhs += CLODE_RHS_PER_ATTEMPT;
#pragma unroll
    for (int j = 0; j < N_VAR; ++j)
        err[j] /= fmax(fmax(fabs(m.x[j]), fabs(xn[j])), threshold);
#pragma unroll
    for (int j = 0; j < N_VAR; ++j)
        nerr = fmax(fabs(err[j]), nerr);
    if (!(nerr > sp.reltol)) {
        if (s.first_try)
            h *= fmin(CLODE_MAX_GROW, safety * pow(sp.reltol / nerr, expon));
        h = fmin(h, t1 - tn);
        h = clamp(h, s.hmin, sp.dtmax);
        m.dt = h;
        m.t = tn;
#pragma unroll
        for (int j = 0; j < N_VAR; ++j) {
            m.x[j] = xn[j];
            m.dx[j] = kn[j];
        }
        c.steps++;
        s.retry = false;
        return 0;
    }
    c.rejected++;
    if (h <= s.hmin) {
        m.dt = s.hmin;
        c.steps++;
        s.retry = false;
        return -1;
    }
    if (s.first_try) {
        s.first_try = false;
        h *= fmax(CLODE_MAX_SHRINK, safety * pow(sp.reltol / nerr, expon));
    } else {
        h *= RCONST(0.5);
    }
    s.h = h;
    s.retry = true;
    return 1;
}
#ifndef CLODE_SPLIT_ATTEMPTS
#error "CLODE_SPLIT_ATTEMPTS must be defined (0 or 1)"
#endif
#else
#error "no stepper selected: define one of EXPLICIT_EULER, EXPLICIT_HEUN, EXPLICIT_RK4, EXPLICIT_BS23, EXPLICIT_DOPRI5, STOCHASTIC_EULER"
#endif

}  // namespace clode
