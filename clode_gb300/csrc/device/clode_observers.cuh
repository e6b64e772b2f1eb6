// On-the-fly feature observers.  One observer is compiled in per program
// (USE_OBSERVER_*).  Its state is a plain struct held in registers for the
// whole time loop; between launches it is parked in global memory
// member-major in 16-byte vectors ([member * stride + word], see park_store),
// so a lane moves its member's state in whole sectors whichever members its
// warp holds.  That layout is private to this engine; only the
// feature vector F has a public layout (F[k * nPts + i], k in the order of
// the reference's feature-name lists).
//
// Hook semantics and arithmetic follow the reference observers:
//   basic     clode/cpp/observers/observer_basic.clh:21-90
//   basicall  clode/cpp/observers/observer_basic_allVar.clh:35-130
//   localmax  clode/cpp/observers/observer_local_maximum.clh:54-328
//   nhood1    clode/cpp/observers/observer_neighborhood_1.clh:44-364
//   nhood2    clode/cpp/observers/observer_neighborhood_2.clh:50-313
//   thresh2   clode/cpp/observers/observer_threshold_2.clh:63-470
// The reference keeps a 3-step solution buffer as [var * 3 + slot]; here it is
// one array per slot (b0 oldest, b2 newest), which holds the same values.
// The event and feature variables (eVarIx, fVarIx) are runtime values, so
// the buffers are read through unrolled selects that keep them in registers.
#pragma once

namespace clode {

typedef ObserverParamsT<realtype> ObserverParams;

#define NSE1 (N_STORE_EVENTS > 0 ? N_STORE_EVENTS : 1)

template <int N>
__device__ __forceinline__ realtype sel(const realtype (&a)[N], unsigned int ix)
{
    realtype v = a[0];
#pragma unroll
    for (int k = 1; k < N; ++k)
        if (ix == (unsigned int)k)
            v = a[k];
    return v;
}

template <int N>
__device__ __forceinline__ void put(realtype (&a)[N], unsigned int ix, realtype v)
{
#pragma unroll
    for (int k = 0; k < N; ++k)
        if (ix == (unsigned int)k)
            a[k] = v;
}

// running means, clode/cpp/clODE_utilities.cl:167-177
__device__ __forceinline__ realtype mean_time(realtype mean, realtype v, realtype dt, realtype elapsed)
{
    return mean + (v - mean) * dt / elapsed;
}

// Builds with approximate division (prec_div 0: CLODE_PREC_DIV = 0) take the
// step's time weight dt / elapsed once for all of a step's time-weighted
// means, and divide the neighbourhood test's distances by per-member
// reciprocals of the ranges: the same quotients within the approximate
// division's own error, with one division per step instead of one per
// variable.  Builds with IEEE division (the default, and the build that
// reproduces the reference) divide per variable as the reference does.
#ifndef CLODE_PREC_DIV
#define CLODE_PREC_DIV 1
#endif
#define CLODE_SHARED_DIV (!CLODE_PREC_DIV && !CLODE_PRECISE)
#if CLODE_SHARED_DIV
__device__ __forceinline__ realtype mean_weighted(realtype mean, realtype v, realtype w)
{
    return mean + (v - mean) * w;
}
#endif

__device__ __forceinline__ void mean_count(realtype &mean, realtype v, unsigned int n)
{
    if (n == 1)
        mean = v;
    else if (n > 1)
        mean += (v - mean) / (realtype)n;
}

// Event times.  The precise option (CLODE_PRECISE) refines the time of a
// threshold crossing inside the step that detected it and keeps event times
// in FP64, so that periods are differences of FP64 times; otherwise an event
// happens at the step's time, as in the reference.
#if CLODE_PRECISE
typedef double evtime;
#else
typedef realtype evtime;
#endif

// cubic Hermite basis on the step (s in [0, 1]) and its derivative in s
struct Hermite {
    double h00, h10, h01, h11, d00, d10, d01, d11;
    __device__ __forceinline__ void at(double s)
    {
        const double s2 = s * s, s3 = s2 * s;
        h00 = 2.0 * s3 - 3.0 * s2 + 1.0;
        h10 = s3 - 2.0 * s2 + s;
        h01 = -2.0 * s3 + 3.0 * s2;
        h11 = s3 - s2;
        d00 = 6.0 * s2 - 6.0 * s;
        d10 = 3.0 * s2 - 4.0 * s + 1.0;
        d01 = -6.0 * s2 + 6.0 * s;
        d11 = 3.0 * s2 - 2.0 * s;
    }
    // value and s-derivative of the interpolant of (x0, slope d0) -> (x1, d1) over a step h
    __device__ __forceinline__ double f(double x0, double d0, double x1, double d1, double h) const
    {
        return h00 * x0 + h10 * h * d0 + h01 * x1 + h11 * h * d1;
    }
    __device__ __forceinline__ double df(double x0, double d0, double x1, double d1, double h) const
    {
        return d00 * x0 + d10 * h * d0 + d01 * x1 + d11 * h * d1;
    }
};

// Safeguarded Newton (FP64) for the root of g on [0, 1], g(0) and g(1) of
// opposite signs: g(s) and g'(s) come from g(s, dg).  Starts from s0.
template <typename G>
__device__ __forceinline__ double refine_root(G g, double g0, double s0)
{
    double lo = 0.0, hi = 1.0;
    double s = fmin(fmax(s0, 0.0), 1.0);
    const bool neg0 = g0 < 0.0;
#pragma unroll 1
    for (int it = 0; it < 12; ++it) {
        double dg = 0.0;
        const double v = g(s, dg);
        if (v == 0.0)
            return s;
        if ((v < 0.0) == neg0)
            lo = s;
        else
            hi = s;
        double sn = dg != 0.0 ? s - v / dg : 0.5 * (lo + hi);
        if (!(sn > lo && sn < hi))
            sn = 0.5 * (lo + hi);
        if (fabs(sn - s) < 1e-15)
            return sn;
        s = sn;
    }
    return s;
}

// time in (t0, t1] at which the interpolant of one variable reaches `level`
// (x0 on one side of it, x1 on the other)
__device__ __forceinline__ evtime crossing_time(realtype t0, realtype x0, realtype d0, realtype t1, realtype x1,
                                                realtype d1, realtype level)
{
    const double h = (double)t1 - (double)t0;
    const double X0 = x0, X1 = x1, D0 = d0, D1 = d1, L = level;
    const double g0 = X0 - L;
    auto g = [&](double s, double &dg) {
        Hermite H;
        H.at(s);
        dg = H.df(X0, D0, X1, D1, h);
        return H.f(X0, D0, X1, D1, h) - L;
    };
    const double s = refine_root(g, g0, X1 != X0 ? (L - X0) / (X1 - X0) : 0.5);
    return (evtime)((double)t0 + s * h);
}

// first-occurrence arg-extremum of three values, clODE_utilities.cl:49-127
__device__ __forceinline__ int argmax3(realtype a, realtype b, realtype c)
{
    realtype best = -BIG_REAL;
    int ix = 0;
    if (a > best) { best = a; ix = 0; }
    if (b > best) { best = b; ix = 1; }
    if (c > best) { best = c; ix = 2; }
    return ix;
}

__device__ __forceinline__ int argmin3(realtype a, realtype b, realtype c)
{
    realtype best = BIG_REAL;
    int ix = 0;
    if (a < best) { best = a; ix = 0; }
    if (b < best) { best = b; ix = 1; }
    if (c < best) { best = c; ix = 2; }
    return ix;
}

__device__ __forceinline__ realtype pick3(int ix, realtype a, realtype b, realtype c)
{
    return ix == 0 ? a : (ix == 1 ? b : c);
}

// max / min / mean triple over events or periods
struct Stat3 {
    realtype hi, lo, mean;
    __device__ __forceinline__ void reset() { hi = -BIG_REAL; lo = BIG_REAL; mean = ZERO; }
    __device__ __forceinline__ void push(realtype v, unsigned int n)
    {
        hi = fmax(v, hi);
        lo = fmin(v, lo);
        mean_count(mean, v, n);
    }
};

// 3-step solution buffer
struct SolBuf {
    realtype t0, t1, t2;
    realtype x0[N_VAR], x1[N_VAR], x2[N_VAR];
    realtype d0[N_VAR], d1[N_VAR], d2[N_VAR];
    __device__ __forceinline__ void seed(realtype t, const realtype (&x)[N_VAR], const realtype (&dx)[N_VAR])
    {
        t2 = t;
#pragma unroll
        for (int j = 0; j < N_VAR; ++j) {
            x2[j] = x[j];
            d2[j] = dx[j];
        }
    }
    __device__ __forceinline__ void shift(realtype t, const realtype (&x)[N_VAR], const realtype (&dx)[N_VAR])
    {
        t0 = t1; t1 = t2; t2 = t;
#pragma unroll
        for (int j = 0; j < N_VAR; ++j) {
            x0[j] = x1[j]; x1[j] = x2[j]; x2[j] = x[j];
            d0[j] = d1[j]; d1[j] = d2[j]; d2[j] = dx[j];
        }
    }
    __device__ __forceinline__ void rebase(realtype T) { t0 -= T; t1 -= T; t2 -= T; }
};

// whole-trajectory extent of every state variable, its slope and every aux
// The time-weighted means follow the reference's running update; the
// precise option instead keeps the compensated sums of value x step (hi part
// in xmean / amean, low part in xlo / alo) and divides by the elapsed time
// when the means are read (xm, am).
struct Extent {
    realtype xmax[N_VAR], xmin[N_VAR], xmean[N_VAR], dxmax[N_VAR], dxmin[N_VAR];
    realtype amax[NA1], amin[NA1], amean[NA1];
#if CLODE_PRECISE
    realtype xlo[N_VAR], alo[NA1];
    realtype span;  // elapsed time at the last update
#endif
    __device__ __forceinline__ void reset()
    {
#pragma unroll
        for (int j = 0; j < N_VAR; ++j) {
            xmax[j] = -BIG_REAL; xmin[j] = BIG_REAL; xmean[j] = ZERO;
            dxmax[j] = -BIG_REAL; dxmin[j] = BIG_REAL;
        }
#pragma unroll
        for (int j = 0; j < N_AUX; ++j) {
            amax[j] = -BIG_REAL; amin[j] = BIG_REAL; amean[j] = ZERO;
        }
#if CLODE_PRECISE
#pragma unroll
        for (int j = 0; j < N_VAR; ++j)
            xlo[j] = ZERO;
#pragma unroll
        for (int j = 0; j < NA1; ++j)
            alo[j] = ZERO;
        span = ZERO;
#endif
    }
    __device__ __forceinline__ void update(const realtype (&x)[N_VAR], const realtype (&dx)[N_VAR],
                                           const realtype (&aux)[NA1], realtype dt, realtype elapsed)
    {
#if CLODE_SHARED_DIV
        const realtype w = dt / elapsed;
#endif
#pragma unroll
        for (int j = 0; j < N_VAR; ++j) {
            xmax[j] = fmax(x[j], xmax[j]);
            xmin[j] = fmin(x[j], xmin[j]);
#if CLODE_PRECISE
            CSum cs = {xmean[j], xlo[j]};
            cs.add_prod(x[j], dt);
            xmean[j] = cs.hi;
            xlo[j] = cs.lo;
#elif CLODE_SHARED_DIV
            xmean[j] = mean_weighted(xmean[j], x[j], w);
#else
            xmean[j] = mean_time(xmean[j], x[j], dt, elapsed);
#endif
            dxmax[j] = fmax(dx[j], dxmax[j]);
            dxmin[j] = fmin(dx[j], dxmin[j]);
        }
#pragma unroll
        for (int j = 0; j < N_AUX; ++j) {
            amax[j] = fmax(aux[j], amax[j]);
            amin[j] = fmin(aux[j], amin[j]);
#if CLODE_PRECISE
            CSum cs = {amean[j], alo[j]};
            cs.add_prod(aux[j], dt);
            amean[j] = cs.hi;
            alo[j] = cs.lo;
#elif CLODE_SHARED_DIV
            amean[j] = mean_weighted(amean[j], aux[j], w);
#else
            amean[j] = mean_time(amean[j], aux[j], dt, elapsed);
#endif
        }
#if CLODE_PRECISE
        span = elapsed;
#endif
    }
    // the time-weighted means as written to the features
    __device__ __forceinline__ realtype xm(int j) const
    {
#if CLODE_PRECISE
        return span != ZERO ? (realtype)(((double)xmean[j] + (double)xlo[j]) / (double)span) : ZERO;
#else
        return xmean[j];
#endif
    }
    __device__ __forceinline__ realtype am(int j) const
    {
#if CLODE_PRECISE
        return span != ZERO ? (realtype)(((double)amean[j] + (double)alo[j]) / (double)span) : ZERO;
#else
        return amean[j];
#endif
    }
};

// The feature pass's accumulators that do not depend on its warm-up: the
// extent (extrema, time-weighted means, slope and aux extrema) and the step
// statistics, updated per step exactly as the two-pass observers' update()
// does.  The replayed feature pass takes them in the recording launch, from
// the same steps in the same order, and the replay merges them into the
// observer at the member's end (merge_sums), so that the stored rows need
// only the fields the warm-up-dependent logic reads.  Not with the precise
// option, whose event refinement interpolates every state variable.
struct FeatureSums {
    Extent ext;
    Stat3 hstat;
    realtype t_prev, t_start;
    unsigned int steps;
    __device__ __forceinline__ void init(realtype t)
    {
        ext.reset();
        hstat.reset();
        t_prev = t;
        t_start = t;
        steps = 0;
    }
    __device__ __forceinline__ void update(realtype t, const realtype (&x)[N_VAR], const realtype (&dx)[N_VAR],
                                           const realtype (&aux)[NA1])
    {
        ++steps;
        const realtype h = t - t_prev;
        t_prev = t;
        hstat.push(h, steps);
        ext.update(x, dx, aux, h, t - t_start);
    }
};

// the extent and step statistics at the end of a feature pass from the
// armed observer's extent (the warm-up's state extrema, reset values
// elsewhere) and the pass's sums: the state extrema are the larger of the
// two, everything else is the pass's.  The armed extent is read again from
// the parked state at the member's end, so that the replay holds no extent
// in registers while it runs.
__device__ __forceinline__ void merge_sums(Extent &ext, Stat3 &hstat, const Extent &armed, const FeatureSums &s)
{
#pragma unroll
    for (int j = 0; j < N_VAR; ++j) {
        ext.xmax[j] = fmax(s.ext.xmax[j], armed.xmax[j]);
        ext.xmin[j] = fmin(s.ext.xmin[j], armed.xmin[j]);
        ext.xmean[j] = s.ext.xmean[j];
        ext.dxmax[j] = s.ext.dxmax[j];
        ext.dxmin[j] = s.ext.dxmin[j];
    }
#pragma unroll
    for (int j = 0; j < NA1; ++j) {
        ext.amax[j] = s.ext.amax[j];
        ext.amin[j] = s.ext.amin[j];
        ext.amean[j] = s.ext.amean[j];
    }
    hstat = s.hstat;
}

// feature writer: F[k * nPts + i]
struct FOut {
    realtype *F;
    unsigned long long stride;
    int i;
    int k;
    __device__ __forceinline__ void operator()(realtype v)
    {
        F[(unsigned long long)k * stride + i] = v;
        ++k;
    }
};

#define CLODE_HOOK_ARGS realtype t, const realtype (&x)[N_VAR], const realtype (&dx)[N_VAR], \
                        const realtype (&aux)[NA1], const ObserverParams &op

#if defined(USE_OBSERVER_BASIC)
#define CLODE_HAVE_OBSERVER 1
struct Observer {
    static constexpr bool two_pass = false;
    realtype xmax, xmin, xmean, dxmax, dxmin, t_last, t_start;
    unsigned int steps;

    __device__ __forceinline__ void init(CLODE_HOOK_ARGS)
    {
        xmax = -BIG_REAL; xmin = BIG_REAL; xmean = ZERO; dxmax = -BIG_REAL; dxmin = BIG_REAL;
        t_last = t; t_start = t; steps = 0;
    }
    __device__ __forceinline__ void warmup(CLODE_HOOK_ARGS) {}
    __device__ __forceinline__ void arm(CLODE_HOOK_ARGS) {}
    __device__ __forceinline__ void update(CLODE_HOOK_ARGS)
    {
        ++steps;
        realtype h = t - t_last;
        t_last = t;
        realtype elapsed = t - t_start;
        realtype xf = sel(x, op.fVarIx), df = sel(dx, op.fVarIx);
        xmax = fmax(xf, xmax);
        xmin = fmin(xf, xmin);
        xmean = mean_time(xmean, xf, h, elapsed);
        dxmax = fmax(df, dxmax);
        dxmin = fmin(df, dxmin);
    }
    __device__ __forceinline__ bool event(CLODE_HOOK_ARGS) { return false; }
    __device__ __forceinline__ bool on_event(CLODE_HOOK_ARGS) { return false; }
    __device__ __forceinline__ void write(FOut &o) const
    {
        o(xmax); o(xmin); o(xmean); o(dxmax); o(dxmin); o((realtype)steps);
    }
    __device__ __forceinline__ void rebase(realtype T) { t_start -= T; }
};

#elif defined(USE_OBSERVER_BASIC_ALLVAR)
#define CLODE_HAVE_OBSERVER 1
struct Observer {
    static constexpr bool two_pass = false;
    Extent ext;
    realtype t_last, t_start;
    unsigned int steps;

    __device__ __forceinline__ void init(CLODE_HOOK_ARGS)
    {
        ext.reset();
        t_last = t; t_start = t; steps = 0;
    }
    __device__ __forceinline__ void warmup(CLODE_HOOK_ARGS) {}
    __device__ __forceinline__ void arm(CLODE_HOOK_ARGS) {}
    __device__ __forceinline__ void update(CLODE_HOOK_ARGS)
    {
        ++steps;
        realtype h = t - t_last;
        t_last = t;
        ext.update(x, dx, aux, h, t - t_start);
    }
    __device__ __forceinline__ bool event(CLODE_HOOK_ARGS) { return false; }
    __device__ __forceinline__ bool on_event(CLODE_HOOK_ARGS) { return false; }
    __device__ __forceinline__ void write(FOut &o) const
    {
#pragma unroll
        for (int j = 0; j < N_VAR; ++j) {
            o(ext.xmax[j]); o(ext.xmin[j]); o(ext.xm(j)); o(ext.dxmax[j]); o(ext.dxmin[j]);
        }
#pragma unroll
        for (int j = 0; j < N_AUX; ++j) {
            o(ext.amax[j]); o(ext.amin[j]); o(ext.am(j));
        }
        o((realtype)steps);
    }
    __device__ __forceinline__ void rebase(realtype T) { t_start -= T; }
};

#elif defined(USE_OBSERVER_LOCAL_MAX)
#define CLODE_HAVE_OBSERVER 1
struct Observer {
    static constexpr bool two_pass = false;
    SolBuf b;
    Extent ext;
    realtype tmax_list[NSE1], xmax_list[NSE1], tmin_list[NSE1], xmin_list[NSE1];
    Stat3 imi, amp;
    realtype t_start, t_last_max, t_last_min, x_last_min;
    unsigned int events, steps;

    __device__ __forceinline__ void init(CLODE_HOOK_ARGS)
    {
        b.seed(t, x, dx);
        ext.reset();
#pragma unroll
        for (int j = 0; j < NSE1; ++j)
            tmax_list[j] = xmax_list[j] = tmin_list[j] = xmin_list[j] = ZERO;
        imi.reset();
        amp.reset();
        t_start = t; t_last_max = ZERO; t_last_min = ZERO; x_last_min = BIG_REAL;
        events = 0; steps = 0;
    }
    __device__ __forceinline__ void warmup(CLODE_HOOK_ARGS) {}
    __device__ __forceinline__ void arm(CLODE_HOOK_ARGS) {}
    __device__ __forceinline__ void update(CLODE_HOOK_ARGS)
    {
        ++steps;
        b.shift(t, x, dx);
        realtype h = b.t2 - b.t1;
        ext.update(x, dx, aux, h, t - t_start);
        if (steps < 2)
            return;
        const unsigned int f = op.fVarIx;
        if (sel(b.d1, f) < ZERO && sel(b.d2, f) > ZERO) {
            realtype a0 = sel(b.x0, f), a1 = sel(b.x1, f), a2 = sel(b.x2, f);
            int ix = argmin3(a0, a1, a2);
            t_last_min = pick3(ix, b.t0, b.t1, b.t2);
            x_last_min = pick3(ix, a0, a1, a2);
            // A minimum before the first maximum (events == 0) is not stored:
            // the reference's unsigned index events-1 points outside the list.
            if (events > 0 && events <= N_STORE_EVENTS) {
                put(tmin_list, events - 1, t_last_min);
                put(xmin_list, events - 1, x_last_min);
            }
        }
    }
    __device__ __forceinline__ bool event(CLODE_HOOK_ARGS)
    {
        if (steps < 2)
            return false;
        return sel(b.d1, op.fVarIx) > ZERO && sel(b.d2, op.fVarIx) < ZERO;
    }
    __device__ __forceinline__ bool on_event(CLODE_HOOK_ARGS)
    {
        const unsigned int f = op.fVarIx;
        realtype a0 = sel(b.x0, f), a1 = sel(b.x1, f), a2 = sel(b.x2, f);
        int ix = argmax3(a0, a1, a2);
        realtype tpk = pick3(ix, b.t0, b.t1, b.t2), xpk = pick3(ix, a0, a1, a2);
        ++events;
        if (events > 1) {
            imi.push(tpk - t_last_max, events - 1);
            amp.push(xpk - x_last_min, events - 1);
        }
        t_last_max = tpk;
        if (events <= N_STORE_EVENTS) {
            put(tmax_list, events - 1, tpk);
            put(xmax_list, events - 1, xpk);
        }
        return events == op.maxEventCount;
    }
    __device__ __forceinline__ void write(FOut &o) const
    {
        bool two = events > 1;
        o(two ? imi.hi : ZERO); o(two ? imi.lo : ZERO); o(two ? imi.mean : ZERO);
        o(two ? amp.hi : ZERO); o(two ? amp.lo : ZERO); o(two ? amp.mean : ZERO);
#pragma unroll
        for (int j = 0; j < N_VAR; ++j) {
            o(ext.xmax[j]); o(ext.xmin[j]); o(ext.xm(j)); o(ext.dxmax[j]); o(ext.dxmin[j]);
        }
#pragma unroll
        for (int j = 0; j < N_AUX; ++j) {
            o(ext.amax[j]); o(ext.amin[j]); o(ext.am(j));
        }
#pragma unroll
        for (int j = 0; j < N_STORE_EVENTS; ++j) {
            o(tmax_list[j]); o(xmax_list[j]); o(tmin_list[j]); o(xmin_list[j]);
        }
        o((realtype)events);
        o((realtype)steps);
    }
    __device__ __forceinline__ void rebase(realtype T)
    {
        t_start -= T;
        t_last_max = t_last_max - T;
        t_last_min = t_last_min - T;
        b.rebase(T);
    }
};

#elif defined(USE_OBSERVER_NEIGHBORHOOD_1)
#define CLODE_HAVE_OBSERVER 1
struct Observer {
    static constexpr bool two_pass = false;
    SolBuf b;
    realtype c[N_VAR];  // neighbourhood centre
    Extent ext;
    Stat3 npk, period, hstat;
    realtype t_start, t_last_event, norm_now, norm_prev;
    unsigned int peaks_now, events, steps, have_c, inside;

    __device__ __forceinline__ void init(CLODE_HOOK_ARGS)
    {
        b.seed(t, x, dx);
        ext.reset();
        npk.reset(); period.reset(); hstat.reset();
        // never read before being set; cleared so the parked state is defined
#pragma unroll
        for (int j = 0; j < N_VAR; ++j)
            c[j] = ZERO;
        t_start = t; t_last_event = ZERO; norm_now = ZERO; norm_prev = ZERO;
        peaks_now = 0; events = 0; steps = 0; have_c = 0; inside = 0;
    }
    __device__ __forceinline__ void warmup(CLODE_HOOK_ARGS) {}
    __device__ __forceinline__ void arm(CLODE_HOOK_ARGS) {}
    __device__ __forceinline__ void update(CLODE_HOOK_ARGS)
    {
        ++steps;
        b.shift(t, x, dx);
        realtype h = b.t2 - b.t1;
        hstat.push(h, steps);
        // per-step (not time-weighted) means in this observer
#pragma unroll
        for (int j = 0; j < N_VAR; ++j) {
            ext.xmax[j] = fmax(x[j], ext.xmax[j]);
            ext.xmin[j] = fmin(x[j], ext.xmin[j]);
            mean_count(ext.xmean[j], x[j], steps);
            ext.dxmax[j] = fmax(dx[j], ext.dxmax[j]);
            ext.dxmin[j] = fmin(dx[j], ext.dxmin[j]);
        }
#pragma unroll
        for (int j = 0; j < N_AUX; ++j) {
            ext.amax[j] = fmax(aux[j], ext.amax[j]);
            ext.amin[j] = fmin(aux[j], ext.amin[j]);
            mean_count(ext.amean[j], aux[j], steps);
        }
        if (steps > 1) {
            const unsigned int e = op.eVarIx, f = op.fVarIx;
            if (!have_c) {
                if (sel(b.d1, e) <= ZERO && sel(b.d2, e) > ZERO) {
                    int ix = argmin3(sel(b.x0, e), sel(b.x1, e), sel(b.x2, e));
                    t_last_event = pick3(ix, b.t0, b.t1, b.t2);
                    have_c = 1;
#pragma unroll
                    for (int j = 0; j < N_VAR; ++j)
                        c[j] = pick3(ix, b.x0[j], b.x1[j], b.x2[j]);
                }
            } else if (sel(b.d1, f) >= ZERO && sel(b.d2, f) < ZERO) {
                peaks_now++;
            }
        }
    }
    __device__ __forceinline__ bool event(CLODE_HOOK_ARGS)
    {
        if (steps < 2 || !have_c)
            return false;
        const unsigned int f = op.fVarIx;
        if (sel(ext.xmax, f) - sel(ext.xmin, f) < op.minXamp)
            return false;
        unsigned int was_inside = inside;
        norm_prev = norm_now;
        realtype acc = ZERO;
#pragma unroll
        for (int j = 0; j < N_VAR; ++j) {
            realtype d = fabs(x[j] - c[j]) / (ext.xmax[j] - ext.xmin[j]);
            acc += d * d;
        }
        norm_now = sqrt(acc);
        inside = norm_now <= op.nHoodRadius;
        return inside && !was_inside;
    }
    __device__ __forceinline__ bool on_event(CLODE_HOOK_ARGS)
    {
        ++events;
        if (events > 1) {
            npk.push((realtype)peaks_now, events - 1);
            period.push(t - t_last_event, events - 1);
        }
        t_last_event = t;
        peaks_now = 0;
        return events >= op.maxEventCount;
    }
    __device__ __forceinline__ void write(FOut &o) const
    {
        bool two = events > 1;
        o(two ? period.hi : ZERO); o(two ? period.lo : ZERO); o(two ? period.mean : ZERO);
        o(two ? npk.hi : ZERO); o(two ? npk.lo : ZERO); o(two ? npk.mean : ZERO);
#pragma unroll
        for (int j = 0; j < N_VAR; ++j) {
            o(ext.xmax[j]); o(ext.xmin[j]); o(ext.xmean[j]); o(ext.dxmax[j]); o(ext.dxmin[j]);
        }
#pragma unroll
        for (int j = 0; j < N_AUX; ++j) {
            o(ext.amax[j]); o(ext.amin[j]); o(ext.amean[j]);
        }
        o((realtype)(events - 1u));  // "period count", unsigned as in the reference
        o((realtype)steps);
        o(hstat.hi); o(hstat.lo); o(hstat.mean);
    }
    __device__ __forceinline__ void rebase(realtype T)
    {
        t_start -= T;
        t_last_event -= T;
        b.rebase(T);
    }
};

#elif defined(USE_OBSERVER_NEIGHBORHOOD_2)
#define CLODE_HAVE_OBSERVER 1
struct Observer {
    static constexpr bool two_pass = true;
    SolBuf b;
    realtype c[N_VAR];  // neighbourhood centre
    Extent ext;
    realtype xrange[N_VAR];
#if CLODE_SHARED_DIV
    realtype xrange_inv[N_VAR];  // 1 / xrange (approximate-division builds)
#endif
    realtype tex_list[NSE1];
    Stat3 npk, period, hstat;
    realtype t_start, x_thresh;
    evtime t_last_event, t_ev;  // t_ev: the refined time of the current event (precise option)
    unsigned int peaks_now, have_c, inside, events, steps;

    __device__ __forceinline__ void init(CLODE_HOOK_ARGS)
    {
        b.seed(t, x, dx);
        ext.reset();
#pragma unroll
        for (int j = 0; j < N_VAR; ++j) {
            c[j] = x[j];
            xrange[j] = ZERO;
#if CLODE_SHARED_DIV
            xrange_inv[j] = ZERO;
#endif
        }
#pragma unroll
        for (int j = 0; j < NSE1; ++j)
            tex_list[j] = ZERO;
        npk.reset(); period.reset(); hstat.reset();
        t_start = t; t_last_event = ZERO; t_ev = ZERO; x_thresh = ZERO;
        peaks_now = 0; have_c = 0; inside = 0; events = 0; steps = 0;
    }
    // first pass: extent of every state variable
    __device__ __forceinline__ void warmup(CLODE_HOOK_ARGS)
    {
#pragma unroll
        for (int j = 0; j < N_VAR; ++j) {
            ext.xmax[j] = fmax(x[j], ext.xmax[j]);
            ext.xmin[j] = fmin(x[j], ext.xmin[j]);
        }
    }
    __device__ __forceinline__ void arm(CLODE_HOOK_ARGS)
    {
#pragma unroll
        for (int j = 0; j < N_VAR; ++j) {
            xrange[j] = ext.xmax[j] - ext.xmin[j];
#if CLODE_SHARED_DIV
            xrange_inv[j] = ONE / xrange[j];
#endif
        }
        x_thresh = sel(ext.xmin, op.eVarIx) + op.xDownThresh * sel(xrange, op.eVarIx);
    }
    __device__ __forceinline__ void update(CLODE_HOOK_ARGS)
    {
        ++steps;
        b.shift(t, x, dx);
        realtype h = b.t2 - b.t1;
        hstat.push(h, steps);
        ext.update(x, dx, aux, h, t - t_start);
        update_events(op);
    }
#if !CLODE_PRECISE && !defined(CLODE_REPLAY_WHOLE_ROWS)
#define CLODE_OBS_SPLIT 1
    // the replayed feature pass: rows of t, every state variable and the
    // slope of fVar (the centre, ball and peak tests); the extent and step
    // statistics come from the recording launch's FeatureSums
    static constexpr int split_fields = 1 + N_VAR + 1;
    __device__ __forceinline__ static void rec_store(realtype *r, CLODE_HOOK_ARGS)
    {
        r[0] = t;
#pragma unroll
        for (int j = 0; j < N_VAR; ++j)
            r[(1 + j) * 32] = x[j];
        r[(1 + N_VAR) * 32] = sel(dx, op.fVarIx);
    }
    __device__ __forceinline__ static void rec_load(const realtype *r, realtype &t, realtype (&x)[N_VAR],
                                                    realtype (&dx)[N_VAR], realtype (&aux)[NA1],
                                                    const ObserverParams &op)
    {
        t = r[0];
#pragma unroll
        for (int j = 0; j < N_VAR; ++j) {
            x[j] = r[(1 + j) * 32];
            dx[j] = ZERO;
        }
        put(dx, op.fVarIx, r[(1 + N_VAR) * 32]);
#pragma unroll
        for (int j = 0; j < NA1; ++j)
            aux[j] = ZERO;
    }
    __device__ __forceinline__ void update_split(CLODE_HOOK_ARGS)
    {
        ++steps;
        b.shift(t, x, dx);
        update_events(op);
    }
    __device__ __forceinline__ void merge(const Observer &armed, const FeatureSums &s)
    {
        merge_sums(ext, hstat, armed.ext, s);
    }
#endif
    // the warm-up-dependent part of update: centre, then peaks between exits
    __device__ __forceinline__ void update_events(const ObserverParams &op)
    {
        if (steps < 2)
            return;
        if (have_c) {
            if (sel(b.d1, op.fVarIx) >= ZERO && sel(b.d2, op.fVarIx) < ZERO)
                peaks_now++;
            return;
        }
        // centre: first downward crossing of the event variable's threshold
        if (sel(b.x1, op.eVarIx) > x_thresh && sel(b.x2, op.eVarIx) < x_thresh) {
            have_c = 1;
            inside = 1;
#pragma unroll
            for (int j = 0; j < N_VAR; ++j)
                c[j] = b.x2[j];
        }
    }
    // event: exit from the L2 ball around c in range-normalised coordinates
    __device__ __forceinline__ bool event(CLODE_HOOK_ARGS)
    {
        if (steps < 2 || !have_c)
            return false;
        realtype acc = ZERO;
#pragma unroll
        for (int j = 0; j < N_VAR; ++j) {
#if CLODE_SHARED_DIV
            realtype d = (x[j] - c[j]) * xrange_inv[j];
#else
            realtype d = (x[j] - c[j]) / xrange[j];
#endif
            acc += d * d;
        }
        unsigned int was_inside = inside;
        inside = sqrt(acc) < op.nHoodRadius;
        const bool exit = was_inside && !inside;
#if CLODE_PRECISE
        if (exit) {
            // the time in this step at which the interpolated state leaves the ball
            const double h = (double)b.t2 - (double)b.t1, r = op.nHoodRadius;
            auto g = [&](double s, double &dg) {
                Hermite H;
                H.at(s);
                double v = -r * r;
                dg = 0.0;
#pragma unroll
                for (int j = 0; j < N_VAR; ++j) {
                    const double R = xrange[j];
                    const double u = (H.f(b.x1[j], b.d1[j], b.x2[j], b.d2[j], h) - (double)c[j]) / R;
                    v += u * u;
                    dg += 2.0 * u * H.df(b.x1[j], b.d1[j], b.x2[j], b.d2[j], h) / R;
                }
                return v;
            };
            double dg0 = 0.0, dg1 = 0.0;
            const double g0 = g(0.0, dg0);
            const double g1 = g(1.0, dg1);
            const double s = refine_root(g, g0, g1 != g0 ? -g0 / (g1 - g0) : 0.5);
            t_ev = (double)b.t1 + s * h;
        }
#endif
        return exit;
    }
    __device__ __forceinline__ bool on_event(CLODE_HOOK_ARGS)
    {
#if CLODE_PRECISE
        const evtime te = t_ev;
#else
        const evtime te = t;
#endif
        ++events;
        if (events > 1) {
            npk.push((realtype)peaks_now, events - 1);
            period.push((realtype)(te - t_last_event), events - 1);
        }
        t_last_event = te;
        peaks_now = 0;
        if (events <= N_STORE_EVENTS)
            put(tex_list, events - 1, (realtype)te);
        return events == op.maxEventCount;
    }
    __device__ __forceinline__ void write(FOut &o) const
    {
        bool two = events > 1;
        o(two ? period.hi : ZERO); o(two ? period.lo : ZERO); o(two ? period.mean : ZERO);
        o(two ? npk.hi : ZERO); o(two ? npk.lo : ZERO); o(two ? npk.mean : ZERO);
#pragma unroll
        for (int j = 0; j < N_VAR; ++j) {
            o(ext.xmax[j]); o(ext.xmin[j]); o(ext.xm(j)); o(xrange[j]); o(c[j]);
            o(ext.dxmax[j]); o(ext.dxmin[j]);
        }
#pragma unroll
        for (int j = 0; j < N_AUX; ++j) {
            o(ext.amax[j]); o(ext.amin[j]); o(ext.am(j));
        }
#pragma unroll
        for (int j = 0; j < N_STORE_EVENTS; ++j)
            o(tex_list[j]);
        o((realtype)events);
        o((realtype)steps);
        o(hstat.hi); o(hstat.lo); o(hstat.mean);
    }
    __device__ __forceinline__ void rebase(realtype T)
    {
        t_start -= T;
        t_last_event -= T;
        b.rebase(T);
    }
};

#elif defined(USE_OBSERVER_THRESHOLD_2)
#define CLODE_HAVE_OBSERVER 1
struct Observer {
    static constexpr bool two_pass = true;
    SolBuf b;
    Extent ext;
    realtype tup_list[NSE1], tdown_list[NSE1];
    Stat3 npk, period, updur, downdur, duty, dip, hstat;
    realtype down_mean;
    realtype gxmax, gxmin, gdxmax, gdxmin, x_up, x_down, dx_up, dx_down;
    realtype t_start, t_last_max, t_last_min, x_last_min;
    evtime t_last_event, t_down, t_ev;  // t_ev: the refined time of the current event (precise option)
    unsigned int peaks_now, steps, events, is_up;

    __device__ __forceinline__ void init(CLODE_HOOK_ARGS)
    {
        b.seed(t, x, dx);
        ext.reset();
#pragma unroll
        for (int j = 0; j < NSE1; ++j)
            tup_list[j] = tdown_list[j] = ZERO;
        npk.reset(); period.reset(); updur.reset(); downdur.reset(); duty.reset(); dip.reset(); hstat.reset();
        down_mean = ZERO;
        gxmax = -BIG_REAL; gxmin = BIG_REAL; gdxmax = -BIG_REAL; gdxmin = BIG_REAL;
        x_up = ZERO; x_down = ZERO; dx_up = ZERO; dx_down = ZERO;
        t_start = t; t_last_event = ZERO; t_down = ZERO; t_ev = ZERO; t_last_max = ZERO; t_last_min = ZERO;
        x_last_min = BIG_REAL;
        is_up = 0; peaks_now = 0; steps = 0; events = 0;
    }
    // first pass: extent of the event variable and of its slope
    __device__ __forceinline__ void warmup(CLODE_HOOK_ARGS)
    {
        realtype xe = sel(x, op.eVarIx), de = sel(dx, op.eVarIx);
        gxmax = fmax(gxmax, xe);
        gxmin = fmin(gxmin, xe);
        gdxmax = fmax(gdxmax, de);
        gdxmin = fmin(gdxmin, de);
    }
    __device__ __forceinline__ void arm(CLODE_HOOK_ARGS)
    {
        realtype amp = gxmax - gxmin;
        x_up = gxmin + op.xUpThresh * amp;
        x_down = op.xDownThresh > ZERO ? gxmin + op.xDownThresh * amp : x_up;
        dx_up = op.dxUpThresh * gdxmax;
        dx_down = op.dxDownThresh > ZERO ? op.dxDownThresh * gdxmin : gdxmin;
        is_up = sel(x, op.eVarIx) > x_up ? 1 : 0;
    }
    __device__ __forceinline__ void update(CLODE_HOOK_ARGS)
    {
        ++steps;
        b.shift(t, x, dx);
        realtype h = b.t2 - b.t1;
        hstat.push(h, steps);
        ext.update(x, dx, aux, h, t - t_start);
        update_events(t, x, dx, h, op);
    }
#if !CLODE_PRECISE && !defined(CLODE_REPLAY_WHOLE_ROWS)
#define CLODE_OBS_SPLIT 1
    // the replayed feature pass: rows of t and the state and slope of eVar
    // and fVar; the extent and step statistics come from the recording
    // launch's FeatureSums
    static constexpr int split_fields = 5;
    __device__ __forceinline__ static void rec_store(realtype *r, CLODE_HOOK_ARGS)
    {
        r[0] = t;
        r[32] = sel(x, op.eVarIx);
        r[64] = sel(x, op.fVarIx);
        r[96] = sel(dx, op.eVarIx);
        r[128] = sel(dx, op.fVarIx);
    }
    __device__ __forceinline__ static void rec_load(const realtype *r, realtype &t, realtype (&x)[N_VAR],
                                                    realtype (&dx)[N_VAR], realtype (&aux)[NA1],
                                                    const ObserverParams &op)
    {
        t = r[0];
#pragma unroll
        for (int j = 0; j < N_VAR; ++j)
            x[j] = dx[j] = ZERO;
        put(x, op.eVarIx, r[32]);
        put(x, op.fVarIx, r[64]);
        put(dx, op.eVarIx, r[96]);
        put(dx, op.fVarIx, r[128]);
#pragma unroll
        for (int j = 0; j < NA1; ++j)
            aux[j] = ZERO;
    }
    __device__ __forceinline__ void update_split(CLODE_HOOK_ARGS)
    {
        ++steps;
        b.shift(t, x, dx);
        update_events(t, x, dx, b.t2 - b.t1, op);
    }
    __device__ __forceinline__ void merge(const Observer &armed, const FeatureSums &s)
    {
        merge_sums(ext, hstat, armed.ext, s);
    }
#endif
    // the warm-up-dependent part of update: peaks and troughs of fVar, the
    // downward crossing of eVar and the mean of fVar since it
    __device__ __forceinline__ void update_events(realtype t, const realtype (&x)[N_VAR],
                                                  const realtype (&dx)[N_VAR], realtype h, const ObserverParams &op)
    {
        if (steps > 1) {
            const unsigned int f = op.fVarIx, e = op.eVarIx;
            realtype a0 = sel(b.x0, f), a1 = sel(b.x1, f), a2 = sel(b.x2, f);
            realtype df1 = sel(b.d1, f), df2 = sel(b.d2, f);
            if (df1 > ZERO && df2 < ZERO) {
                int ix = argmax3(a0, a1, a2);
                peaks_now++;
                t_last_max = pick3(ix, b.t0, b.t1, b.t2);
            }
            if (df1 < ZERO && df2 > ZERO) {
                int ix = argmin3(a0, a1, a2);
                x_last_min = pick3(ix, a0, a1, a2);
                t_last_min = pick3(ix, b.t0, b.t1, b.t2);
            }
            if (is_up) {
                if (sel(x, e) <= x_down && sel(dx, e) >= dx_down) {
#if CLODE_PRECISE
                    const realtype xp = sel(b.x1, e);
                    t_down = xp > x_down ? crossing_time(b.t1, xp, sel(b.d1, e), b.t2, sel(b.x2, e), sel(b.d2, e), x_down)
                                         : (evtime)t;
#else
                    t_down = t;
#endif
                    is_up = 0;
                    if (events > 0 && events <= N_STORE_EVENTS)
                        put(tdown_list, events - 1, (realtype)t_down);
                    down_mean = sel(x, f);
                }
            } else {
                realtype since_down = (realtype)(t - t_down);
                if (since_down > ZERO)
                    down_mean = mean_time(down_mean, sel(x, f), h, since_down);
            }
        }
    }
    __device__ __forceinline__ bool event(CLODE_HOOK_ARGS)
    {
        if (steps < 2)
            return false;
        if (gxmax - gxmin < op.minXamp)
            return false;
        if (is_up)
            return false;
        const bool up = sel(x, op.eVarIx) > x_up && sel(dx, op.eVarIx) > dx_up;
#if CLODE_PRECISE
        if (up) {
            const unsigned int e = op.eVarIx;
            const realtype xp = sel(b.x1, e);
            t_ev = xp <= x_up ? crossing_time(b.t1, xp, sel(b.d1, e), b.t2, sel(b.x2, e), sel(b.d2, e), x_up)
                              : (evtime)t;
        }
#endif
        return up;
    }
    __device__ __forceinline__ bool on_event(CLODE_HOOK_ARGS)
    {
#if CLODE_PRECISE
        const evtime te = t_ev;
#else
        const evtime te = t;
#endif
        ++events;
        is_up = 1;
        if (events > 1) {
            unsigned int n = events - 1;
            npk.push((realtype)peaks_now, n);
            realtype per = (realtype)(te - t_last_event);
            period.push(per, n);
            realtype up = (realtype)(t_down - t_last_event);
            updur.push(up, n);
            downdur.push((realtype)(te - t_down), n);
            duty.push(up / per, n);
            dip.push(down_mean - x_last_min, n);
        }
        if (events <= N_STORE_EVENTS)
            put(tup_list, events - 1, (realtype)te);
        t_last_event = te;
        peaks_now = 0;
        return events == op.maxEventCount;
    }
    __device__ __forceinline__ void write(FOut &o) const
    {
        bool two = events > 1;
        o(two ? period.hi : ZERO); o(two ? period.lo : ZERO); o(two ? period.mean : ZERO);
        o(two ? npk.hi : ZERO); o(two ? npk.lo : ZERO); o(two ? npk.mean : ZERO);
        o(two ? updur.hi : ZERO); o(two ? updur.lo : ZERO); o(two ? updur.mean : ZERO);
        o(two ? downdur.hi : ZERO); o(two ? downdur.lo : ZERO); o(two ? downdur.mean : ZERO);
        o(two ? duty.hi : ZERO); o(two ? duty.lo : ZERO); o(two ? duty.mean : ZERO);
        o(two ? dip.hi : ZERO); o(two ? dip.lo : ZERO); o(two ? dip.mean : ZERO);
#pragma unroll
        for (int j = 0; j < N_VAR; ++j) {
            o(ext.xmax[j]); o(ext.xmin[j]); o(ext.xm(j)); o(ext.dxmax[j]); o(ext.dxmin[j]);
        }
#pragma unroll
        for (int j = 0; j < N_AUX; ++j) {
            o(ext.amax[j]); o(ext.amin[j]); o(ext.am(j));
        }
#pragma unroll
        for (int j = 0; j < N_STORE_EVENTS; ++j) {
            o(tup_list[j]); o(tdown_list[j]);
        }
        o((realtype)events);
        o((realtype)steps);
        o(hstat.hi); o(hstat.lo); o(hstat.mean);
    }
    __device__ __forceinline__ void rebase(realtype T)
    {
        t_start -= T;
        t_last_event -= T;
        t_down -= T;
        t_last_max -= T;
        t_last_min -= T;
        b.rebase(T);
    }
};
#else
#define CLODE_HAVE_OBSERVER 0
#endif

}  // namespace clode
