/* Test infrastructure (the oracle), not product code.
 *
 * CPU restatement of clODE's ensemble integration path: the transient,
 * initializeObserver, features and trajectory kernels, their steppers,
 * observers and RNG stream.  One ensemble member is integrated per loop
 * iteration with the reference's exact sequence of floating-point operations
 * (compile with -ffp-contract=off), so that on the same inputs it reproduces
 * the reference's arithmetic.  Each function names the reference file:line it
 * restates (paths inside the clODE project).
 *
 * Compile-time configuration uses the reference's define set
 * (clode/cpp/CLODE.cpp:118-138, clode/cpp/CLODEfeatures.cpp:37-38):
 *   CLODE_SINGLE_PRECISION | CLODE_DOUBLE_PRECISION
 *   EXPLICIT_EULER | EXPLICIT_HEUN | EXPLICIT_RK4 | EXPLICIT_BS23 |
 *   EXPLICIT_DOPRI5 | STOCHASTIC_EULER
 *   N_VAR, N_PAR, N_AUX, N_WIENER
 *   USE_OBSERVER_{BASIC,BASIC_ALLVAR,LOCAL_MAX,NEIGHBORHOOD_1,NEIGHBORHOOD_2,THRESHOLD_2}
 *   N_STORE_EVENTS
 * and CLODE_RHS_FILE naming the model source that defines getRHS.
 *
 * Exported entry points (same ABI as the reference-kernel driver
 * ref_driver.c, so one runner drives both): o_transient, o_trajectory,
 * o_init_observer, o_features, o_real_size, o_odata_size, o_is_reference. */
#include "port_shim.h"

#ifdef _OPENMP
#include <omp.h>
#define OMP_MEMBERS _Pragma("omp parallel for schedule(dynamic, 8) num_threads(nthreads)")
#else
#define OMP_MEMBERS
#endif

#define NA1 (N_AUX > 0 ? N_AUX : 1)
#define NW1 (N_WIENER > 0 ? N_WIENER : 1)
#define NSE1 (N_STORE_EVENTS > 0 ? N_STORE_EVENTS : 1)

void getRHS(const realtype t, const realtype x_[], const realtype p_[], realtype dx_[],
            realtype aux_[], const realtype w_[]);

/* Solver and observer parameter blocks: field order and types of
 * clode/cpp/clODE_struct_defs.cl:11-20 and clode/cpp/observers.cl:25-46. */
typedef struct {
    realtype dt, dtmax, abstol, reltol;
    unsigned int max_steps, max_store, nout;
} o_solver_params;

typedef struct {
    unsigned int eVarIx, fVarIx, maxEventCount, maxEventTimestamps;
    realtype minXamp, minIMI, nHoodRadius, xUpThresh, xDownThresh, dxUpThresh, dxDownThresh, eps_dx;
} o_observer_params;

/* ------------------------------------------------------------------ RNG -- */
/* xoroshiro128+ with rotations 55/14/36: clode/cpp/clODE_random.cl:28-44 */
static inline uint64_t o_rotl(uint64_t v, int k) { return (v << k) | (v >> (64 - k)); }

static inline uint64_t o_next(uint64_t s[2])
{
    uint64_t a = s[0], b = s[1];
    uint64_t out = a + b;
    b ^= a;
    s[0] = o_rotl(a, 55) ^ b ^ (b << 14);
    s[1] = o_rotl(b, 36);
    return out;
}

typedef struct {
    uint64_t s[2];
    int spare_ready;
    realtype spare;
} o_rng;

/* uniform in [0,1): u64 * 2^-64 in working precision, clODE_random.cl:26,81-85 */
static inline realtype o_uniform(uint64_t s[2])
{
    return (realtype)o_next(s) * RCONST(5.421010862427522e-20);
}

/* polar Box-Muller with a cached second deviate, clODE_random.cl:88-114 */
static inline realtype o_randn(o_rng *r)
{
    if (r->spare_ready) {
        r->spare_ready = 0;
        return r->spare;
    }
    realtype u, v, s;
    do {
        u = RCONST(2.0) * o_uniform(r->s) - ONE;
        v = RCONST(2.0) * o_uniform(r->s) - ONE;
        s = u * u + v * v;
    } while (s >= ONE);
    realtype m = sqrt((-RCONST(2.0) * log(s)) / s);
    r->spare = v * m;
    r->spare_ready = 1;
    return u * m;
}

/* ------------------------------------------------------------- steppers -- */
#if defined(STOCHASTIC_EULER)
#define O_STOCHASTIC 1
#else
#define O_STOCHASTIC 0
#endif

#if defined(EXPLICIT_EULER) || defined(STOCHASTIC_EULER) || defined(EXPLICIT_HEUN) || defined(EXPLICIT_RK4)
#define O_FIXED_STEP 1

/* one fixed step, updates t and x in place given k1 = f(t, x) */
static inline void o_do_step(realtype *t, realtype x[], const realtype k1[], const realtype p[],
                             const realtype dt, realtype aux[], const realtype w[])
{
#if defined(EXPLICIT_EULER) || defined(STOCHASTIC_EULER)
    /* clode/cpp/steppers/fixed_explicit_Euler.clh:5-18 */
    for (int k = 0; k < N_VAR; ++k)
        x[k] += dt * k1[k];
    *t += dt;
#elif defined(EXPLICIT_HEUN)
    /* clode/cpp/steppers/fixed_explicit_Trapezoidal.clh:5-23 */
    realtype tnew = *t + dt;
    realtype xp[N_VAR], k2[N_VAR];
    for (int k = 0; k < N_VAR; ++k)
        xp[k] = fma(dt, k1[k], x[k]);
    getRHS(tnew, xp, p, k2, aux, w);
    for (int k = 0; k < N_VAR; ++k)
        x[k] += dt * RCONST(0.5) * (k1[k] + k2[k]);
    *t = tnew;
#else
    /* clode/cpp/steppers/fixed_explicit_RK4.clh:5-40 */
    realtype xs[N_VAR], k2[N_VAR], k3[N_VAR], k4[N_VAR];
    realtype half = dt * RCONST(0.5);
    realtype tmid = *t + half;
    realtype tend = *t + dt;
    for (int k = 0; k < N_VAR; ++k)
        xs[k] = x[k] + half * k1[k];
    getRHS(tmid, xs, p, k2, aux, w);
    for (int k = 0; k < N_VAR; ++k)
        xs[k] = x[k] + half * k2[k];
    getRHS(tmid, xs, p, k3, aux, w);
    for (int k = 0; k < N_VAR; ++k)
        xs[k] = x[k] + dt * k3[k];
    getRHS(tend, xs, p, k4, aux, w);
    for (int k = 0; k < N_VAR; ++k)
        x[k] += dt * (k1[k] + RCONST(2.0) * k2[k] + RCONST(2.0) * k3[k] + k4[k]) / RCONST(6.0);
    *t = tend;
#endif
}

/* fixed-step wrapper: clode/cpp/steppers/fixed_explicit_step.clh:9-37 */
static inline int o_stepper(realtype *t, realtype x[], realtype k1[], const realtype p[],
                            const o_solver_params *sp, realtype *dt, const realtype *tspan,
                            realtype aux[], realtype w[], o_rng *r)
{
    (void)sp; (void)tspan; (void)r;
    o_do_step(t, x, k1, p, *dt, aux, w);
#if O_STOCHASTIC
    for (int j = 0; j < N_WIENER; ++j)
        w[j] = o_randn(r) / sqrt(*dt);
#endif
    getRHS(*t, x, p, k1, aux, w);
    return 0;
}

#elif defined(EXPLICIT_BS23) || defined(EXPLICIT_DOPRI5)
#define O_FIXED_STEP 0

#if defined(EXPLICIT_BS23)
/* clode/cpp/steppers/adaptive_bs23.clh:1-20 */
#define O_ERR_ORDER RCONST(2.0)
#define O_MAX_SHRINK RCONST(0.5)
#define O_MAX_GROW RCONST(5.0)

/* Bogacki-Shampine 3(2) attempt, FSAL: clode/cpp/steppers/adaptive_bs23.clh:27-63 */
static inline realtype o_attempt(realtype *t, realtype x[], realtype k1[], const realtype p[],
                                 const realtype dt, realtype aux[], realtype err[], const realtype w[])
{
    const realtype b1 = RCONST(2.0) / RCONST(9.0), b2 = RCONST(1.0) / RCONST(3.0), b3 = RCONST(4.0) / RCONST(9.0);
    const realtype e1 = RCONST(-5.0) / RCONST(72.0), e2 = RCONST(1.0) / RCONST(12.0);
    const realtype e3 = RCONST(1.0) / RCONST(9.0), e4 = RCONST(-1.0) / RCONST(8.0);
    realtype tnew = *t + dt;
    realtype h = tnew - *t;
    realtype xs[N_VAR], k2[N_VAR], k3[N_VAR], k4[N_VAR];
    for (int k = 0; k < N_VAR; ++k)
        xs[k] = x[k] + h * RCONST(0.5) * k1[k];
    getRHS(*t + h * RCONST(0.5), xs, p, k2, aux, w);
    for (int k = 0; k < N_VAR; ++k)
        xs[k] = x[k] + h * RCONST(0.75) * k2[k];
    getRHS(*t + h * RCONST(0.75), xs, p, k3, aux, w);
    for (int k = 0; k < N_VAR; ++k)
        x[k] = x[k] + h * (b1 * k1[k] + b2 * k2[k] + b3 * k3[k]);
    getRHS(tnew, x, p, k4, aux, w);
    for (int k = 0; k < N_VAR; ++k) {
        err[k] = h * (e1 * k1[k] + e2 * k2[k] + e3 * k3[k] + e4 * k4[k]);
        k1[k] = k4[k];
    }
    *t = tnew;
    return h;
}
#else
/* clode/cpp/steppers/adaptive_dp45.clh:1-9 */
#define O_ERR_ORDER RCONST(4.0)
#define O_MAX_SHRINK RCONST(0.1)
#define O_MAX_GROW RCONST(5.0)

/* Dormand-Prince 5(4) attempt, FSAL: clode/cpp/steppers/adaptive_dp45.clh:58-111,
 * tableau :10-56 (each coefficient is the quotient rounded to working precision). */
static inline realtype o_attempt(realtype *t, realtype x[], realtype k1[], const realtype p[],
                                 const realtype dt, realtype aux[], realtype err[], const realtype w[])
{
    const realtype a2 = RCONST(1.0) / RCONST(5.0), a3 = RCONST(3.0) / RCONST(10.0);
    const realtype a4 = RCONST(4.0) / RCONST(5.0), a5 = RCONST(8.0) / RCONST(9.0);
    const realtype b21 = RCONST(1.0) / RCONST(5.0);
    const realtype b31 = RCONST(3.0) / RCONST(40.0), b32 = RCONST(9.0) / RCONST(40.0);
    const realtype b41 = RCONST(44.0) / RCONST(45.0), b42 = RCONST(-56.0) / RCONST(15.0), b43 = RCONST(32.0) / RCONST(9.0);
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

    realtype tnew = *t + dt;
    realtype h = tnew - *t;
    realtype xs[N_VAR], k2[N_VAR], k3[N_VAR], k4[N_VAR], k5[N_VAR], k6[N_VAR], k7[N_VAR];
    for (int k = 0; k < N_VAR; ++k)
        xs[k] = x[k] + h * (b21 * k1[k]);
    getRHS(*t + a2 * h, xs, p, k2, aux, w);
    for (int k = 0; k < N_VAR; ++k)
        xs[k] = x[k] + h * (b31 * k1[k] + b32 * k2[k]);
    getRHS(*t + a3 * h, xs, p, k3, aux, w);
    for (int k = 0; k < N_VAR; ++k)
        xs[k] = x[k] + h * (b41 * k1[k] + b42 * k2[k] + b43 * k3[k]);
    getRHS(*t + a4 * h, xs, p, k4, aux, w);
    for (int k = 0; k < N_VAR; ++k)
        xs[k] = x[k] + h * (b51 * k1[k] + b52 * k2[k] + b53 * k3[k] + b54 * k4[k]);
    getRHS(*t + a5 * h, xs, p, k5, aux, w);
    for (int k = 0; k < N_VAR; ++k)
        xs[k] = x[k] + h * (b61 * k1[k] + b62 * k2[k] + b63 * k3[k] + b64 * k4[k] + b65 * k5[k]);
    getRHS(*t + h, xs, p, k6, aux, w);
    for (int k = 0; k < N_VAR; ++k)
        x[k] = x[k] + h * (c1 * k1[k] + c3 * k3[k] + c4 * k4[k] + c5 * k5[k] + c6 * k6[k]);
    getRHS(tnew, x, p, k7, aux, w);
    for (int k = 0; k < N_VAR; ++k) {
        err[k] = h * (e1 * k1[k] + e3 * k3[k] + e4 * k4[k] + e5 * k5[k] + e6 * k6[k] + e7 * k7[k]);
        k1[k] = k7[k];
    }
    *t = tnew;
    return h;
}
#endif

/* adaptive step-size controller: clode/cpp/steppers/adaptive_explicit_step.clh:4-81 */
static inline int o_stepper(realtype *t, realtype x[], realtype k1[], const realtype p[],
                            const o_solver_params *sp, realtype *dt, const realtype *tspan,
                            realtype aux[], realtype w[], o_rng *r)
{
    (void)r;
    const realtype safety = RCONST(0.8);
    const realtype expon = RCONST(1.0) / (O_ERR_ORDER + RCONST(1.0));
    realtype tnew, nerr = ZERO, err[N_VAR], xnew[N_VAR], k1new[N_VAR];
    realtype h = *dt;
    realtype threshold = sp->abstol / sp->reltol;
    realtype hmin = RCONST(16.0) * fabs(fabs(nextafter(*t, RCONST(1.1) * tspan[1])) - *t);
    int first_try = 1;
    for (;;) {
        tnew = *t;
        for (int j = 0; j < N_VAR; ++j) {
            xnew[j] = x[j];
            k1new[j] = k1[j];
        }
        h = clamp(h, hmin, sp->dtmax);
        h = o_attempt(&tnew, xnew, k1new, p, h, aux, err, w);
        for (int j = 0; j < N_VAR; ++j)
            err[j] /= fmax(fmax(fabs(x[j]), fabs(xnew[j])), threshold);
        /* inf-norm, clode/cpp/clODE_utilities.cl:40-46 */
        nerr = ZERO;
        for (int j = 0; j < N_VAR; ++j)
            nerr = fmax(fabs(err[j]), nerr);
        if (!(nerr > sp->reltol))
            break;
        if (h <= hmin) {
            *dt = hmin;
            return -1;
        }
        if (first_try) {
            first_try = 0;
            h *= fmax(O_MAX_SHRINK, safety * pow(sp->reltol / nerr, expon));
        } else {
            h *= RCONST(0.5);
        }
    }
    if (first_try)
        h *= fmin(O_MAX_GROW, safety * pow(sp->reltol / nerr, expon));
    h = fmin(h, tspan[1] - tnew);
    h = clamp(h, hmin, sp->dtmax);
    *dt = h;
    *t = tnew;
    for (int j = 0; j < N_VAR; ++j) {
        x[j] = xnew[j];
        k1[j] = k1new[j];
    }
    return 0;
}
#else
#error "no stepper selected"
#endif

/* ------------------------------------------------------------ observers -- */
#if defined(USE_OBSERVER_BASIC) || defined(USE_OBSERVER_BASIC_ALLVAR) || defined(USE_OBSERVER_LOCAL_MAX) || \
    defined(USE_OBSERVER_NEIGHBORHOOD_1) || defined(USE_OBSERVER_NEIGHBORHOOD_2) || defined(USE_OBSERVER_THRESHOLD_2)
#define O_HAVE_OBSERVER 1
#else
#define O_HAVE_OBSERVER 0
#endif

/* running means: clode/cpp/clODE_utilities.cl:167-177 */
static inline realtype o_mean_time(realtype mean, realtype v, realtype dt, realtype elapsed)
{
    return mean + (v - mean) * dt / elapsed;
}

static inline void o_mean_count(realtype *mean, realtype v, unsigned int n)
{
    if (n == 1)
        *mean = v;
    else if (n > 1)
        *mean += (v - *mean) / (realtype)n;
}

/* argmax / argmin returning the first occurrence: clODE_utilities.cl:49-127 */
static inline int o_argmax3(const realtype v[3])
{
    realtype best = -BIG_REAL;
    int ix = 0;
    for (int k = 0; k < 3; ++k)
        if (v[k] > best) { best = v[k]; ix = k; }
    return ix;
}

static inline int o_argmin3(const realtype v[3])
{
    realtype best = BIG_REAL;
    int ix = 0;
    for (int k = 0; k < 3; ++k)
        if (v[k] < best) { best = v[k]; ix = k; }
    return ix;
}

/* the 3-point solution buffer and whole-trajectory extrema shared by the
 * event observers (localmax, nhood1, nhood2, thresh2) */
#define O_BUFFERS realtype tb[3]; realtype xb[3 * N_VAR]; realtype db[3 * N_VAR];
#define O_EXTENT realtype xmax[N_VAR], xmin[N_VAR], xmean[N_VAR], dxmax[N_VAR], dxmin[N_VAR]; \
                 realtype amax[NA1], amin[NA1], amean[NA1];

static inline void o_extent_init(realtype xmax[], realtype xmin[], realtype xmean[], realtype dxmax[],
                                 realtype dxmin[], realtype amax[], realtype amin[], realtype amean[])
{
    for (int j = 0; j < N_VAR; ++j) {
        xmax[j] = -BIG_REAL; xmin[j] = BIG_REAL; xmean[j] = ZERO;
        dxmax[j] = -BIG_REAL; dxmin[j] = BIG_REAL;
    }
    for (int j = 0; j < N_AUX; ++j) {
        amax[j] = -BIG_REAL; amin[j] = BIG_REAL; amean[j] = ZERO;
    }
}

static inline void o_extent_update(realtype xmax[], realtype xmin[], realtype xmean[], realtype dxmax[],
                                   realtype dxmin[], realtype amax[], realtype amin[], realtype amean[],
                                   const realtype x[], const realtype dx[], const realtype aux[],
                                   realtype dt, realtype elapsed)
{
    for (int j = 0; j < N_VAR; ++j) {
        xmax[j] = fmax(x[j], xmax[j]);
        xmin[j] = fmin(x[j], xmin[j]);
        xmean[j] = o_mean_time(xmean[j], x[j], dt, elapsed);
        dxmax[j] = fmax(dx[j], dxmax[j]);
        dxmin[j] = fmin(dx[j], dxmin[j]);
    }
    for (int j = 0; j < N_AUX; ++j) {
        amax[j] = fmax(aux[j], amax[j]);
        amin[j] = fmin(aux[j], amin[j]);
        amean[j] = o_mean_time(amean[j], aux[j], dt, elapsed);
    }
}

static inline void o_buffers_seed(realtype tb[], realtype xb[], realtype db[], realtype t,
                                  const realtype x[], const realtype dx[])
{
    tb[2] = t;
    for (int j = 0; j < N_VAR; ++j) {
        xb[j * 3 + 2] = x[j];
        db[j * 3 + 2] = dx[j];
    }
}

static inline void o_buffers_shift(realtype tb[], realtype xb[], realtype db[], realtype t,
                                   const realtype x[], const realtype dx[])
{
    tb[0] = tb[1]; tb[1] = tb[2]; tb[2] = t;
    for (int j = 0; j < N_VAR; ++j) {
        xb[j * 3 + 0] = xb[j * 3 + 1]; xb[j * 3 + 1] = xb[j * 3 + 2]; xb[j * 3 + 2] = x[j];
        db[j * 3 + 0] = db[j * 3 + 1]; db[j * 3 + 1] = db[j * 3 + 2]; db[j * 3 + 2] = dx[j];
    }
}

#define O_F(k, v) F[(long)(k) * nPts + i] = (v)

#if defined(USE_OBSERVER_BASIC)
/* clode/cpp/observers/observer_basic.clh:21-90 */
#define O_TWO_PASS 0
typedef struct {
    realtype xmax, xmin, xmean, dxmax, dxmin, t_last, t_start;
    unsigned int steps;
} o_obs;

static void ob_init(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                    const o_observer_params *op)
{
    o->xmax = -BIG_REAL; o->xmin = BIG_REAL; o->xmean = ZERO;
    o->dxmax = -BIG_REAL; o->dxmin = BIG_REAL;
    o->t_last = t; o->t_start = t; o->steps = 0;
}
static void ob_warmup(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                      const o_observer_params *op) {}
static void ob_arm(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                   const o_observer_params *op) {}
static void ob_update(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                      const o_observer_params *op)
{
    ++o->steps;
    realtype dt = t - o->t_last;
    o->t_last = t;
    realtype elapsed = t - o->t_start;
    unsigned int f = op->fVarIx;
    o->xmax = fmax(x[f], o->xmax);
    o->xmin = fmin(x[f], o->xmin);
    o->xmean = o_mean_time(o->xmean, x[f], dt, elapsed);
    o->dxmax = fmax(dx[f], o->dxmax);
    o->dxmin = fmin(dx[f], o->dxmin);
}
static bool ob_event(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                     const o_observer_params *op) { return false; }
static bool ob_on_event(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                        const o_observer_params *op) { return false; }
static void ob_write(o_obs *o, realtype *F, int i, int nPts)
{
    O_F(0, o->xmax); O_F(1, o->xmin); O_F(2, o->xmean); O_F(3, o->dxmax); O_F(4, o->dxmin);
    O_F(5, (realtype)o->steps);
}
static void ob_rebase(realtype T, o_obs *o) { o->t_start -= T; }

#elif defined(USE_OBSERVER_BASIC_ALLVAR)
/* clode/cpp/observers/observer_basic_allVar.clh:35-130 */
#define O_TWO_PASS 0
typedef struct {
    O_EXTENT
    realtype t_last, t_start;
    unsigned int steps;
} o_obs;

static void ob_init(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                    const o_observer_params *op)
{
    o_extent_init(o->xmax, o->xmin, o->xmean, o->dxmax, o->dxmin, o->amax, o->amin, o->amean);
    o->t_last = t; o->t_start = t; o->steps = 0;
}
static void ob_warmup(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                      const o_observer_params *op) {}
static void ob_arm(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                   const o_observer_params *op) {}
static void ob_update(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                      const o_observer_params *op)
{
    ++o->steps;
    realtype dt = t - o->t_last;
    o->t_last = t;
    realtype elapsed = t - o->t_start;
    o_extent_update(o->xmax, o->xmin, o->xmean, o->dxmax, o->dxmin, o->amax, o->amin, o->amean, x, dx, aux,
                    dt, elapsed);
}
static bool ob_event(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                     const o_observer_params *op) { return false; }
static bool ob_on_event(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                        const o_observer_params *op) { return false; }
static void ob_write(o_obs *o, realtype *F, int i, int nPts)
{
    int k = 0;
    for (int j = 0; j < N_VAR; ++j) {
        O_F(k++, o->xmax[j]); O_F(k++, o->xmin[j]); O_F(k++, o->xmean[j]);
        O_F(k++, o->dxmax[j]); O_F(k++, o->dxmin[j]);
    }
    for (int j = 0; j < N_AUX; ++j) {
        O_F(k++, o->amax[j]); O_F(k++, o->amin[j]); O_F(k++, o->amean[j]);
    }
    O_F(k++, (realtype)o->steps);
}
static void ob_rebase(realtype T, o_obs *o) { o->t_start -= T; }

#elif defined(USE_OBSERVER_LOCAL_MAX)
/* clode/cpp/observers/observer_local_maximum.clh:54-328 */
#define O_TWO_PASS 0
typedef struct {
    O_BUFFERS
    O_EXTENT
    realtype tmax_list[NSE1], xmax_list[NSE1], tmin_list[NSE1], xmin_list[NSE1];
    realtype imi[3], amp[3];
    realtype t_start, t_last_max, t_last_min, x_last_min;
    unsigned int events, steps;
} o_obs;

static void ob_init(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                    const o_observer_params *op)
{
    o_buffers_seed(o->tb, o->xb, o->db, t, x, dx);
    o_extent_init(o->xmax, o->xmin, o->xmean, o->dxmax, o->dxmin, o->amax, o->amin, o->amean);
    for (int j = 0; j < N_STORE_EVENTS; ++j)
        o->tmax_list[j] = o->xmax_list[j] = o->tmin_list[j] = o->xmin_list[j] = ZERO;
    o->imi[0] = -BIG_REAL; o->imi[1] = BIG_REAL; o->imi[2] = ZERO;
    o->amp[0] = -BIG_REAL; o->amp[1] = BIG_REAL; o->amp[2] = ZERO;
    o->t_start = t; o->t_last_max = ZERO; o->t_last_min = ZERO; o->x_last_min = BIG_REAL;
    o->events = 0; o->steps = 0;
}
static void ob_warmup(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                      const o_observer_params *op) {}
static void ob_arm(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                   const o_observer_params *op) {}

/* A local minimum found before the first maximum (eventcount == 0) is not
 * stored.  The reference indexes tMinList/xMinList with the unsigned
 * eventcount-1 (observer_local_maximum.clh:278-281), i.e. element 2^32-1, an
 * out-of-bounds write: compiled for the host it crashes when N_STORE_EVENTS > 0
 * and the compiler drops the store when N_STORE_EVENTS == 0.  Skipping the
 * write is the only defined behaviour and matches the latter. */
static void ob_update(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                      const o_observer_params *op)
{
    ++o->steps;
    o_buffers_shift(o->tb, o->xb, o->db, t, x, dx);
    realtype dt = o->tb[2] - o->tb[1];
    realtype elapsed = t - o->t_start;
    o_extent_update(o->xmax, o->xmin, o->xmean, o->dxmax, o->dxmin, o->amax, o->amin, o->amean, x, dx, aux,
                    dt, elapsed);
    if (o->steps < 2)
        return;
    unsigned int f = op->fVarIx;
    if (o->db[f * 3 + 1] < 0.0 && o->db[f * 3 + 2] > 0.0) {
        realtype xs[3] = {o->xb[f * 3 + 0], o->xb[f * 3 + 1], o->xb[f * 3 + 2]};
        int ix = o_argmin3(xs);
        o->t_last_min = o->tb[ix];
        o->x_last_min = xs[ix];
        if (o->events > 0 && o->events <= N_STORE_EVENTS) {
            o->tmin_list[o->events - 1] = o->t_last_min;
            o->xmin_list[o->events - 1] = o->x_last_min;
        }
    }
}
static bool ob_event(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                     const o_observer_params *op)
{
    if (o->steps < 2)
        return false;
    unsigned int f = op->fVarIx;
    return o->db[f * 3 + 1] > 0.0 && o->db[f * 3 + 2] < 0.0;
}
static bool ob_on_event(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                        const o_observer_params *op)
{
    unsigned int f = op->fVarIx;
    realtype xs[3] = {o->xb[f * 3 + 0], o->xb[f * 3 + 1], o->xb[f * 3 + 2]};
    int ix = o_argmax3(xs);
    realtype tpk = o->tb[ix], xpk = xs[ix];
    ++o->events;
    if (o->events > 1) {
        realtype imi = tpk - o->t_last_max;
        o->imi[0] = fmax(imi, o->imi[0]);
        o->imi[1] = fmin(imi, o->imi[1]);
        o_mean_count(&o->imi[2], imi, o->events - 1);
        realtype amp = xpk - o->x_last_min;
        o->amp[0] = fmax(amp, o->amp[0]);
        o->amp[1] = fmin(amp, o->amp[1]);
        o_mean_count(&o->amp[2], amp, o->events - 1);
    }
    o->t_last_max = tpk;
    if (o->events <= N_STORE_EVENTS) {
        o->tmax_list[o->events - 1] = tpk;
        o->xmax_list[o->events - 1] = xpk;
    }
    return o->events == op->maxEventCount;
}
static void ob_write(o_obs *o, realtype *F, int i, int nPts)
{
    int k = 0;
    int two = o->events > 1;
    O_F(k++, two ? o->imi[0] : ZERO); O_F(k++, two ? o->imi[1] : ZERO); O_F(k++, two ? o->imi[2] : ZERO);
    O_F(k++, two ? o->amp[0] : ZERO); O_F(k++, two ? o->amp[1] : ZERO); O_F(k++, two ? o->amp[2] : ZERO);
    for (int j = 0; j < N_VAR; ++j) {
        O_F(k++, o->xmax[j]); O_F(k++, o->xmin[j]); O_F(k++, o->xmean[j]);
        O_F(k++, o->dxmax[j]); O_F(k++, o->dxmin[j]);
    }
    for (int j = 0; j < N_AUX; ++j) {
        O_F(k++, o->amax[j]); O_F(k++, o->amin[j]); O_F(k++, o->amean[j]);
    }
    for (int j = 0; j < N_STORE_EVENTS; ++j) {
        O_F(k++, o->tmax_list[j]); O_F(k++, o->xmax_list[j]);
        O_F(k++, o->tmin_list[j]); O_F(k++, o->xmin_list[j]);
    }
    O_F(k++, (realtype)o->events);
    O_F(k++, (realtype)o->steps);
}
static void ob_rebase(realtype T, o_obs *o)
{
    o->t_start -= T;
    o->t_last_max = o->t_last_max - T;
    o->t_last_min = o->t_last_min - T;
    for (int k = 0; k < 3; ++k)
        o->tb[k] = o->tb[k] - T;
}

#elif defined(USE_OBSERVER_NEIGHBORHOOD_1)
/* clode/cpp/observers/observer_neighborhood_1.clh:44-364 */
#define O_TWO_PASS 0
typedef struct {
    O_BUFFERS
    realtype x0[N_VAR];
    O_EXTENT
    realtype npk[3], period[3], hstat[3];
    realtype t_start, t_last_event, norm_now, norm_prev;
    unsigned int peaks_now, events, steps, have_x0, inside;
} o_obs;

static void ob_init(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                    const o_observer_params *op)
{
    o_buffers_seed(o->tb, o->xb, o->db, t, x, dx);
    o_extent_init(o->xmax, o->xmin, o->xmean, o->dxmax, o->dxmin, o->amax, o->amin, o->amean);
    o->npk[0] = -BIG_REAL; o->npk[1] = BIG_REAL; o->npk[2] = ZERO;
    o->period[0] = -BIG_REAL; o->period[1] = BIG_REAL; o->period[2] = ZERO;
    o->hstat[0] = -BIG_REAL; o->hstat[1] = BIG_REAL; o->hstat[2] = ZERO;
    o->peaks_now = 0; o->events = 0; o->steps = 0; o->have_x0 = 0; o->inside = 0;
}
static void ob_warmup(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                      const o_observer_params *op) {}
static void ob_arm(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                   const o_observer_params *op) {}
static void ob_update(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                      const o_observer_params *op)
{
    ++o->steps;
    o_buffers_shift(o->tb, o->xb, o->db, t, x, dx);
    realtype h = o->tb[2] - o->tb[1];
    o->hstat[0] = fmax(h, o->hstat[0]);
    o->hstat[1] = fmin(h, o->hstat[1]);
    o_mean_count(&o->hstat[2], h, o->steps);
    /* this observer's means are per-step (not time-weighted), nhood_1.clh:249-260 */
    for (int j = 0; j < N_VAR; ++j) {
        o->xmax[j] = fmax(x[j], o->xmax[j]);
        o->xmin[j] = fmin(x[j], o->xmin[j]);
        o_mean_count(&o->xmean[j], x[j], o->steps);
        o->dxmax[j] = fmax(dx[j], o->dxmax[j]);
        o->dxmin[j] = fmin(dx[j], o->dxmin[j]);
    }
    for (int j = 0; j < N_AUX; ++j) {
        o->amax[j] = fmax(aux[j], o->amax[j]);
        o->amin[j] = fmin(aux[j], o->amin[j]);
        o_mean_count(&o->amean[j], aux[j], o->steps);
    }
    if (o->steps > 1) {
        unsigned int e = op->eVarIx, f = op->fVarIx;
        if (!o->have_x0) {
            if (o->db[e * 3 + 1] <= 0.0 && o->db[e * 3 + 2] > 0.0) {
                realtype xs[3] = {o->xb[e * 3 + 0], o->xb[e * 3 + 1], o->xb[e * 3 + 2]};
                int ix = o_argmin3(xs);
                o->t_last_event = o->tb[ix];
                o->have_x0 = 1;
                for (int j = 0; j < N_VAR; ++j)
                    o->x0[j] = o->xb[j * 3 + ix];
            }
        } else if (o->db[f * 3 + 1] >= 0.0 && o->db[f * 3 + 2] < 0.0) {
            o->peaks_now++;
        }
    }
}
static bool ob_event(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                     const o_observer_params *op)
{
    if (o->steps < 2 || !o->have_x0)
        return false;
    unsigned int f = op->fVarIx;
    if (o->xmax[f] - o->xmin[f] < op->minXamp)
        return false;
    unsigned int was_inside = o->inside;
    o->norm_prev = o->norm_now;
    /* 2-norm of the range-normalised distance, clODE_utilities.cl:31-37 */
    realtype acc = ZERO;
    for (int j = 0; j < N_VAR; ++j) {
        realtype d = fabs(x[j] - o->x0[j]) / (o->xmax[j] - o->xmin[j]);
        acc += d * d;
    }
    o->norm_now = sqrt(acc);
    o->inside = o->norm_now <= op->nHoodRadius;
    return o->inside && !was_inside;
}
static bool ob_on_event(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                        const o_observer_params *op)
{
    ++o->events;
    if (o->events > 1) {
        o->npk[0] = fmax((realtype)o->peaks_now, o->npk[0]);
        o->npk[1] = fmin((realtype)o->peaks_now, o->npk[1]);
        o_mean_count(&o->npk[2], (realtype)o->peaks_now, o->events - 1);
        realtype per = t - o->t_last_event;
        o->period[0] = fmax(per, o->period[0]);
        o->period[1] = fmin(per, o->period[1]);
        o_mean_count(&o->period[2], per, o->events - 1);
    }
    o->t_last_event = t;
    o->peaks_now = 0;
    return o->events >= op->maxEventCount;
}
static void ob_write(o_obs *o, realtype *F, int i, int nPts)
{
    int k = 0;
    int two = o->events > 1;
    O_F(k++, two ? o->period[0] : ZERO); O_F(k++, two ? o->period[1] : ZERO); O_F(k++, two ? o->period[2] : ZERO);
    O_F(k++, two ? o->npk[0] : ZERO); O_F(k++, two ? o->npk[1] : ZERO); O_F(k++, two ? o->npk[2] : ZERO);
    for (int j = 0; j < N_VAR; ++j) {
        O_F(k++, o->xmax[j]); O_F(k++, o->xmin[j]); O_F(k++, o->xmean[j]);
        O_F(k++, o->dxmax[j]); O_F(k++, o->dxmin[j]);
    }
    for (int j = 0; j < N_AUX; ++j) {
        O_F(k++, o->amax[j]); O_F(k++, o->amin[j]); O_F(k++, o->amean[j]);
    }
    /* "period count" is eventcount - 1 in unsigned arithmetic (nhood_1.clh:343) */
    O_F(k++, (realtype)(o->events - 1u));
    O_F(k++, (realtype)o->steps);
    O_F(k++, o->hstat[0]); O_F(k++, o->hstat[1]); O_F(k++, o->hstat[2]);
}
static void ob_rebase(realtype T, o_obs *o)
{
    o->t_start -= T;
    o->t_last_event -= T;
    for (int k = 0; k < 3; ++k)
        o->tb[k] -= T;
}

#elif defined(USE_OBSERVER_NEIGHBORHOOD_2)
/* clode/cpp/observers/observer_neighborhood_2.clh:50-313 */
#define O_TWO_PASS 1
typedef struct {
    O_BUFFERS
    realtype x0[N_VAR];
    O_EXTENT
    realtype xrange[N_VAR];
    realtype tex_list[NSE1];
    realtype npk[3], period[3], hstat[3];
    realtype t_start, t_last_event, x_thresh;
    unsigned int peaks_now, have_x0, inside, events, steps;
} o_obs;

static void ob_init(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                    const o_observer_params *op)
{
    o_buffers_seed(o->tb, o->xb, o->db, t, x, dx);
    o_extent_init(o->xmax, o->xmin, o->xmean, o->dxmax, o->dxmin, o->amax, o->amin, o->amean);
    for (int j = 0; j < N_VAR; ++j) {
        o->x0[j] = x[j];
        o->xrange[j] = ZERO;
    }
    for (int j = 0; j < N_STORE_EVENTS; ++j)
        o->tex_list[j] = ZERO;
    o->npk[0] = -BIG_REAL; o->npk[1] = BIG_REAL; o->npk[2] = ZERO;
    o->period[0] = -BIG_REAL; o->period[1] = BIG_REAL; o->period[2] = ZERO;
    o->hstat[0] = -BIG_REAL; o->hstat[1] = BIG_REAL; o->hstat[2] = ZERO;
    o->t_start = t; o->t_last_event = ZERO; o->x_thresh = ZERO;
    o->peaks_now = 0; o->have_x0 = 0; o->inside = 0; o->events = 0; o->steps = 0;
}
/* first pass: whole-trajectory extent, nhood_2.clh:142-147 */
static void ob_warmup(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                      const o_observer_params *op)
{
    for (int j = 0; j < N_VAR; ++j) {
        o->xmax[j] = fmax(x[j], o->xmax[j]);
        o->xmin[j] = fmin(x[j], o->xmin[j]);
    }
}
static void ob_arm(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                   const o_observer_params *op)
{
    for (int j = 0; j < N_VAR; ++j)
        o->xrange[j] = o->xmax[j] - o->xmin[j];
    unsigned int e = op->eVarIx;
    o->x_thresh = o->xmin[e] + op->xDownThresh * o->xrange[e];
}
static void ob_update(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                      const o_observer_params *op)
{
    ++o->steps;
    o_buffers_shift(o->tb, o->xb, o->db, t, x, dx);
    realtype h = o->tb[2] - o->tb[1];
    realtype elapsed = t - o->t_start;
    o->hstat[0] = fmax(h, o->hstat[0]);
    o->hstat[1] = fmin(h, o->hstat[1]);
    o_mean_count(&o->hstat[2], h, o->steps);
    o_extent_update(o->xmax, o->xmin, o->xmean, o->dxmax, o->dxmin, o->amax, o->amin, o->amean, x, dx, aux,
                    h, elapsed);
    if (o->steps < 2)
        return;
    if (o->have_x0) {
        unsigned int f = op->fVarIx;
        if (o->db[f * 3 + 1] >= 0.0 && o->db[f * 3 + 2] < 0.0)
            o->peaks_now++;
        return;
    }
    unsigned int e = op->eVarIx;
    if (o->xb[e * 3 + 1] > o->x_thresh && o->xb[e * 3 + 2] < o->x_thresh) {
        o->have_x0 = 1;
        o->inside = 1;
        for (int j = 0; j < N_VAR; ++j)
            o->x0[j] = x[j];
    }
}
/* exit from the L2 ball around x0 in range-normalised coordinates, nhood_2.clh:157-175 */
static bool ob_event(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                     const o_observer_params *op)
{
    if (o->steps < 2 || !o->have_x0)
        return false;
    realtype acc = ZERO;
    for (int j = 0; j < N_VAR; ++j) {
        realtype d = (x[j] - o->x0[j]) / o->xrange[j];
        acc += d * d;
    }
    unsigned int was_inside = o->inside;
    o->inside = sqrt(acc) < op->nHoodRadius;
    return was_inside && !o->inside;
}
static bool ob_on_event(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                        const o_observer_params *op)
{
    ++o->events;
    if (o->events > 1) {
        o->npk[0] = fmax((realtype)o->peaks_now, o->npk[0]);
        o->npk[1] = fmin((realtype)o->peaks_now, o->npk[1]);
        o_mean_count(&o->npk[2], (realtype)o->peaks_now, o->events - 1);
        realtype per = t - o->t_last_event;
        o->period[0] = fmax(per, o->period[0]);
        o->period[1] = fmin(per, o->period[1]);
        o_mean_count(&o->period[2], per, o->events - 1);
    }
    o->t_last_event = t;
    o->peaks_now = 0;
    if (o->events <= N_STORE_EVENTS)
        o->tex_list[o->events - 1] = t;
    return o->events == op->maxEventCount;
}
static void ob_write(o_obs *o, realtype *F, int i, int nPts)
{
    int k = 0;
    int two = o->events > 1;
    O_F(k++, two ? o->period[0] : ZERO); O_F(k++, two ? o->period[1] : ZERO); O_F(k++, two ? o->period[2] : ZERO);
    O_F(k++, two ? o->npk[0] : ZERO); O_F(k++, two ? o->npk[1] : ZERO); O_F(k++, two ? o->npk[2] : ZERO);
    for (int j = 0; j < N_VAR; ++j) {
        O_F(k++, o->xmax[j]); O_F(k++, o->xmin[j]); O_F(k++, o->xmean[j]); O_F(k++, o->xrange[j]);
        O_F(k++, o->x0[j]); O_F(k++, o->dxmax[j]); O_F(k++, o->dxmin[j]);
    }
    for (int j = 0; j < N_AUX; ++j) {
        O_F(k++, o->amax[j]); O_F(k++, o->amin[j]); O_F(k++, o->amean[j]);
    }
    for (int j = 0; j < N_STORE_EVENTS; ++j)
        O_F(k++, o->tex_list[j]);
    O_F(k++, (realtype)o->events);
    O_F(k++, (realtype)o->steps);
    O_F(k++, o->hstat[0]); O_F(k++, o->hstat[1]); O_F(k++, o->hstat[2]);
}
static void ob_rebase(realtype T, o_obs *o)
{
    o->t_start -= T;
    o->t_last_event -= T;
    for (int k = 0; k < 3; ++k)
        o->tb[k] -= T;
}

#elif defined(USE_OBSERVER_THRESHOLD_2)
/* clode/cpp/observers/observer_threshold_2.clh:63-470 */
#define O_TWO_PASS 1
typedef struct {
    O_BUFFERS
    O_EXTENT
    realtype tup_list[NSE1], tdown_list[NSE1];
    realtype npk[3], period[3], updur[3], downdur[3], duty[3], dip[3], hstat[3];
    realtype up_mean, down_mean;
    realtype gxmax, gxmin, gdxmax, gdxmin, x_up, x_down, dx_up, dx_down;
    realtype t_start, t_last_event, t_down, t_last_max, t_last_min, x_last_min;
    unsigned int peaks_now, steps, events, is_up;
} o_obs;

static void o_stat_reset(realtype s[3]) { s[0] = -BIG_REAL; s[1] = BIG_REAL; s[2] = ZERO; }
static void o_stat_push(realtype s[3], realtype v, unsigned int n)
{
    s[0] = fmax(v, s[0]);
    s[1] = fmin(v, s[1]);
    o_mean_count(&s[2], v, n);
}

static void ob_init(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                    const o_observer_params *op)
{
    o_buffers_seed(o->tb, o->xb, o->db, t, x, dx);
    o_extent_init(o->xmax, o->xmin, o->xmean, o->dxmax, o->dxmin, o->amax, o->amin, o->amean);
    for (int j = 0; j < N_STORE_EVENTS; ++j)
        o->tup_list[j] = o->tdown_list[j] = ZERO;
    o_stat_reset(o->npk); o_stat_reset(o->period); o_stat_reset(o->updur); o_stat_reset(o->downdur);
    o_stat_reset(o->duty); o_stat_reset(o->dip); o_stat_reset(o->hstat);
    o->down_mean = ZERO;
    o->gxmax = -BIG_REAL; o->gxmin = BIG_REAL; o->gdxmax = -BIG_REAL; o->gdxmin = BIG_REAL;
    o->x_up = ZERO; o->x_down = ZERO; o->dx_up = ZERO; o->dx_down = ZERO;
    o->t_start = t; o->t_last_event = ZERO; o->t_down = ZERO; o->t_last_max = ZERO; o->t_last_min = ZERO;
    o->x_last_min = BIG_REAL;
    o->is_up = 0; o->peaks_now = 0; o->steps = 0; o->events = 0;
}
/* first pass: extent of the event variable and its slope, thresh_2.clh:197-203 */
static void ob_warmup(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                      const o_observer_params *op)
{
    unsigned int e = op->eVarIx;
    o->gxmax = fmax(o->gxmax, x[e]);
    o->gxmin = fmin(o->gxmin, x[e]);
    o->gdxmax = fmax(o->gdxmax, dx[e]);
    o->gdxmin = fmin(o->gdxmin, dx[e]);
}
/* thresholds from the first pass, thresh_2.clh:206-224 */
static void ob_arm(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                   const o_observer_params *op)
{
    realtype amp = o->gxmax - o->gxmin;
    o->x_up = o->gxmin + op->xUpThresh * amp;
    o->x_down = op->xDownThresh > ZERO ? o->gxmin + op->xDownThresh * amp : o->x_up;
    o->dx_up = op->dxUpThresh * o->gdxmax;
    o->dx_down = op->dxDownThresh > ZERO ? op->dxDownThresh * o->gdxmin : o->gdxmin;
    o->is_up = x[op->eVarIx] > o->x_up ? 1 : 0;
}
static void ob_update(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                      const o_observer_params *op)
{
    ++o->steps;
    o_buffers_shift(o->tb, o->xb, o->db, t, x, dx);
    realtype h = o->tb[2] - o->tb[1];
    realtype elapsed = t - o->t_start;
    o_stat_push(o->hstat, h, o->steps);
    o_extent_update(o->xmax, o->xmin, o->xmean, o->dxmax, o->dxmin, o->amax, o->amin, o->amean, x, dx, aux,
                    h, elapsed);
    if (o->steps > 1) {
        unsigned int f = op->fVarIx, e = op->eVarIx;
        realtype xs[3] = {o->xb[f * 3 + 0], o->xb[f * 3 + 1], o->xb[f * 3 + 2]};
        if (o->db[f * 3 + 1] > 0.0 && o->db[f * 3 + 2] < 0.0) {
            int ix = o_argmax3(xs);
            o->peaks_now++;
            o->t_last_max = o->tb[ix];
        }
        if (o->db[f * 3 + 1] < 0.0 && o->db[f * 3 + 2] > 0.0) {
            int ix = o_argmin3(xs);
            o->x_last_min = xs[ix];
            o->t_last_min = o->tb[ix];
        }
        if (o->is_up) {
            if (x[e] <= o->x_down && dx[e] >= o->dx_down) {
                o->t_down = t;
                o->is_up = 0;
                if (o->events > 0 && o->events <= N_STORE_EVENTS)
                    o->tdown_list[o->events - 1] = o->t_down;
                o->down_mean = x[f];
            }
        } else {
            realtype since_down = t - o->t_down;
            if (since_down > 0.0)
                o->down_mean = o_mean_time(o->down_mean, x[f], h, since_down);
        }
    }
}
static bool ob_event(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                     const o_observer_params *op)
{
    if (o->steps < 2)
        return false;
    if (o->gxmax - o->gxmin < op->minXamp)
        return false;
    if (o->is_up)
        return false;
    unsigned int e = op->eVarIx;
    return x[e] > o->x_up && dx[e] > o->dx_up;
}
static bool ob_on_event(realtype t, const realtype x[], const realtype dx[], const realtype aux[], o_obs *o,
                        const o_observer_params *op)
{
    ++o->events;
    o->is_up = 1;
    if (o->events > 1) {
        unsigned int n = o->events - 1;
        o_stat_push(o->npk, (realtype)o->peaks_now, n);
        realtype per = t - o->t_last_event;
        o_stat_push(o->period, per, n);
        realtype up = o->t_down - o->t_last_event;
        o_stat_push(o->updur, up, n);
        realtype down = t - o->t_down;
        o_stat_push(o->downdur, down, n);
        realtype duty = up / per;
        o_stat_push(o->duty, duty, n);
        realtype dip = o->down_mean - o->x_last_min;
        o_stat_push(o->dip, dip, n);
    }
    if (o->events <= N_STORE_EVENTS)
        o->tup_list[o->events - 1] = t;
    o->t_last_event = t;
    o->peaks_now = 0;
    return o->events == op->maxEventCount;
}
static void ob_write(o_obs *o, realtype *F, int i, int nPts)
{
    int k = 0;
    int two = o->events > 1;
    const realtype *groups[6] = {o->period, o->npk, o->updur, o->downdur, o->duty, o->dip};
    for (int g = 0; g < 6; ++g)
        for (int s = 0; s < 3; ++s)
            O_F(k++, two ? groups[g][s] : ZERO);
    for (int j = 0; j < N_VAR; ++j) {
        O_F(k++, o->xmax[j]); O_F(k++, o->xmin[j]); O_F(k++, o->xmean[j]);
        O_F(k++, o->dxmax[j]); O_F(k++, o->dxmin[j]);
    }
    for (int j = 0; j < N_AUX; ++j) {
        O_F(k++, o->amax[j]); O_F(k++, o->amin[j]); O_F(k++, o->amean[j]);
    }
    for (int j = 0; j < N_STORE_EVENTS; ++j) {
        O_F(k++, o->tup_list[j]);
        O_F(k++, o->tdown_list[j]);
    }
    O_F(k++, (realtype)o->events);
    O_F(k++, (realtype)o->steps);
    O_F(k++, o->hstat[0]); O_F(k++, o->hstat[1]); O_F(k++, o->hstat[2]);
}
static void ob_rebase(realtype T, o_obs *o)
{
    o->t_start -= T;
    o->t_last_event -= T;
    o->t_down -= T;
    o->t_last_max -= T;
    o->t_last_min -= T;
    for (int k = 0; k < 3; ++k)
        o->tb[k] -= T;
}
#endif

/* -------------------------------------------------------- member loops -- */
/* SoA member access: element j of member i at j*nPts + i (clode/cpp/transient.cl:32-39) */
#define SOA(arr, j) (arr)[(long)(j) * nPts + i]

typedef struct {
    realtype t, dt;
    realtype p[N_PAR > 0 ? N_PAR : 1], x[N_VAR], dx[N_VAR], aux[NA1], w[NW1];
    o_rng r;
} o_member;

/* private copies and the initial slope, clode/cpp/transient.cl:20-51 */
static inline void o_member_load(o_member *m, int i, int nPts, const realtype *tspan, const realtype *x0,
                                 const realtype *pars, const uint64_t *rng, const realtype *dtv)
{
    m->t = tspan[0];
    m->dt = dtv[i];
    for (int j = 0; j < N_PAR; ++j)
        m->p[j] = SOA(pars, j);
    for (int j = 0; j < N_VAR; ++j)
        m->x[j] = SOA(x0, j);
    m->r.s[0] = SOA(rng, 0);
    m->r.s[1] = SOA(rng, 1);
    m->r.spare_ready = 0;
    m->r.spare = ZERO;
    for (int j = 0; j < NW1; ++j)
        m->w[j] = ZERO;
    for (int j = 0; j < NA1; ++j)
        m->aux[j] = ZERO;
#if O_STOCHASTIC
    for (int j = 0; j < N_WIENER; ++j)
        m->w[j] = o_randn(&m->r) / sqrt(m->dt);
#endif
    getRHS(m->t, m->x, m->p, m->dx, m->aux, m->w);
}

/* final state, RNG state, step size and time, clode/cpp/transient.cl:64-76 */
static inline void o_member_store(const o_member *m, int i, int nPts, realtype *xf, uint64_t *rng, realtype *dtv,
                                  realtype *tf)
{
    for (int j = 0; j < N_VAR; ++j)
        SOA(xf, j) = m->x[j];
    SOA(rng, 0) = m->r.s[0];
    SOA(rng, 1) = m->r.s[1];
    dtv[i] = m->dt;
    tf[i] = m->t;
}

int o_real_size(void) { return (int)sizeof(realtype); }
int o_is_reference(void) { return 0; }

/* clode/cpp/transient.cl:9-77 */
void o_transient(int nPts, int i0, int i1, int nthreads, const realtype *tspan, int tspan_stride, realtype *x0,
                 const realtype *pars, const void *spv, realtype *xf, uint64_t *rng, realtype *dtv, realtype *tf)
{
    const o_solver_params *sp = (const o_solver_params *)spv;
    if (nthreads < 1) nthreads = 1;
    OMP_MEMBERS
    for (int i = i0; i < i1; ++i) {
        const realtype *ts = tspan + (long)tspan_stride * i;
        o_member m;
        o_member_load(&m, i, nPts, ts, x0, pars, rng, dtv);
        unsigned int step = 0;
        while (m.t <= ts[1] && step < sp->max_steps) {
            ++step;
            o_stepper(&m.t, m.x, m.dx, m.p, sp, &m.dt, ts, m.aux, m.w, &m.r);
        }
        o_member_store(&m, i, nPts, xf, rng, dtv, tf);
    }
}

/* clode/cpp/trajectory.cl:14-112; rows are [store][var][member] */
void o_trajectory(int nPts, int i0, int i1, int nthreads, const realtype *tspan, int tspan_stride, realtype *x0,
                  const realtype *pars, const void *spv, realtype *xf, uint64_t *rng, realtype *dtv, realtype *tf,
                  realtype *tout, realtype *xout, realtype *dxout, realtype *auxout, int *nStored)
{
    const o_solver_params *sp = (const o_solver_params *)spv;
    if (nthreads < 1) nthreads = 1;
    OMP_MEMBERS
    for (int i = i0; i < i1; ++i) {
        const realtype *ts = tspan + (long)tspan_stride * i;
        o_member m;
        o_member_load(&m, i, nPts, ts, x0, pars, rng, dtv);
        long row = 0;
#define O_STORE_ROW()                                                                 \
        do {                                                                          \
            tout[row * nPts + i] = m.t;                                               \
            for (int j = 0; j < N_VAR; ++j)                                           \
                xout[row * nPts * N_VAR + (long)j * nPts + i] = m.x[j];               \
            for (int j = 0; j < N_VAR; ++j)                                           \
                dxout[row * nPts * N_VAR + (long)j * nPts + i] = m.dx[j];             \
            for (int j = 0; j < N_AUX; ++j)                                           \
                auxout[row * nPts * N_AUX + (long)j * nPts + i] = m.aux[j];           \
        } while (0)
        O_STORE_ROW();
        unsigned int step = 0;
        while (m.t <= ts[1] && step < sp->max_steps && row < (long)sp->max_store) {
            ++step;
            o_stepper(&m.t, m.x, m.dx, m.p, sp, &m.dt, ts, m.aux, m.w, &m.r);
            if (step % sp->nout == 0) {
                ++row;
                O_STORE_ROW();
            }
        }
#undef O_STORE_ROW
        nStored[i] = (int)row;
        o_member_store(&m, i, nPts, xf, rng, dtv, tf);
    }
}

#if O_HAVE_OBSERVER
int o_odata_size(void) { return (int)sizeof(o_obs); }

/* clode/cpp/initializeObserver.cl:9-84 */
void o_init_observer(int nPts, int i0, int i1, int nthreads, const realtype *tspan, int tspan_stride,
                     realtype *x0, const realtype *pars, const void *spv, uint64_t *rng, realtype *dtv,
                     void *odata, const void *opv)
{
    const o_solver_params *sp = (const o_solver_params *)spv;
    const o_observer_params *op = (const o_observer_params *)opv;
    o_obs *obs = (o_obs *)odata;
    if (nthreads < 1) nthreads = 1;
    OMP_MEMBERS
    for (int i = i0; i < i1; ++i) {
        const realtype *ts = tspan + (long)tspan_stride * i;
        o_member m;
        o_member_load(&m, i, nPts, ts, x0, pars, rng, dtv);
        o_obs o = obs[i];
        ob_init(m.t, m.x, m.dx, m.aux, &o, op);
#if O_TWO_PASS
        unsigned int step = 0;
        while (m.t < ts[1] && step < sp->max_steps) {
            ++step;
            o_stepper(&m.t, m.x, m.dx, m.p, sp, &m.dt, ts, m.aux, m.w, &m.r);
            ob_warmup(m.t, m.x, m.dx, m.aux, &o, op);
        }
        /* rewind to the initial state; the noise sample in w is kept as is */
        m.t = ts[0];
        for (int j = 0; j < N_VAR; ++j)
            m.x[j] = SOA(x0, j);
        getRHS(m.t, m.x, m.p, m.dx, m.aux, m.w);
#endif
        ob_arm(m.t, m.x, m.dx, m.aux, &o, op);
        obs[i] = o; /* RNG state and dt are not written back */
    }
}

/* clode/cpp/features.cl:10-106 */
void o_features(int nPts, int i0, int i1, int nthreads, const realtype *tspan, int tspan_stride, realtype *x0,
                const realtype *pars, const void *spv, realtype *xf, uint64_t *rng, realtype *dtv, realtype *tf,
                void *odata, const void *opv, realtype *F)
{
    const o_solver_params *sp = (const o_solver_params *)spv;
    const o_observer_params *op = (const o_observer_params *)opv;
    o_obs *obs = (o_obs *)odata;
    if (nthreads < 1) nthreads = 1;
    OMP_MEMBERS
    for (int i = i0; i < i1; ++i) {
        const realtype *ts = tspan + (long)tspan_stride * i;
        o_member m;
        o_member_load(&m, i, nPts, ts, x0, pars, rng, dtv);
        o_obs o = obs[i];
        unsigned int step = 0;
        while (m.t <= ts[1] && step < sp->max_steps) {
            ++step;
            o_stepper(&m.t, m.x, m.dx, m.p, sp, &m.dt, ts, m.aux, m.w, &m.r);
            ob_update(m.t, m.x, m.dx, m.aux, &o, op);
            if (ob_event(m.t, m.x, m.dx, m.aux, &o, op) && ob_on_event(m.t, m.x, m.dx, m.aux, &o, op))
                break;
        }
        ob_write(&o, F, i, nPts);
        /* time-shift for continuation, e.g. observer_threshold_2.clh:459-470 */
        ob_rebase(m.t - ts[0], &o);
        obs[i] = o;
        o_member_store(&m, i, nPts, xf, rng, dtv, tf);
    }
}

/* Features with storage (no reference counterpart: the reference's unified
 * driver clode/cpp/odedriver.cl:10-162 does not compile): o_features, plus
 * the trajectory rows of that pass stored as o_trajectory stores them
 * (trajectory.cl:63-95: row 0, then every nout-th step while row < max_store,
 * without ending the loop) and the state at each of the first ev_rows
 * observer events, rows [k][var][member]; n_stored and n_events per member. */
void o_features_store(int nPts, int i0, int i1, int nthreads, const realtype *tspan, int tspan_stride,
                      realtype *x0, const realtype *pars, const void *spv, realtype *xf, uint64_t *rng, realtype *dtv,
                      realtype *tf, void *odata, const void *opv, realtype *F, realtype *tout, realtype *xout,
                      realtype *dxout, realtype *auxout, int *nStored, int ev_rows, realtype *evt, realtype *evx,
                      realtype *evdx, realtype *evaux, int *nEvents)
{
    const o_solver_params *sp = (const o_solver_params *)spv;
    const o_observer_params *op = (const o_observer_params *)opv;
    o_obs *obs = (o_obs *)odata;
    if (nthreads < 1) nthreads = 1;
    OMP_MEMBERS
    for (int i = i0; i < i1; ++i) {
        const realtype *ts = tspan + (long)tspan_stride * i;
        o_member m;
        o_member_load(&m, i, nPts, ts, x0, pars, rng, dtv);
        o_obs o = obs[i];
        long row = 0, ev = 0;
#define O_STORE_STATE(T, X, DX, AUX, R)                                               \
        do {                                                                          \
            T[(R) * nPts + i] = m.t;                                                  \
            for (int j = 0; j < N_VAR; ++j)                                           \
                X[(R) * nPts * N_VAR + (long)j * nPts + i] = m.x[j];                  \
            for (int j = 0; j < N_VAR; ++j)                                           \
                DX[(R) * nPts * N_VAR + (long)j * nPts + i] = m.dx[j];                \
            for (int j = 0; j < N_AUX; ++j)                                           \
                AUX[(R) * nPts * N_AUX + (long)j * nPts + i] = m.aux[j];              \
        } while (0)
        O_STORE_STATE(tout, xout, dxout, auxout, row);
        unsigned int step = 0;
        while (m.t <= ts[1] && step < sp->max_steps) {
            ++step;
            o_stepper(&m.t, m.x, m.dx, m.p, sp, &m.dt, ts, m.aux, m.w, &m.r);
            if (step % sp->nout == 0 && row < (long)sp->max_store) {
                ++row;
                O_STORE_STATE(tout, xout, dxout, auxout, row);
            }
            ob_update(m.t, m.x, m.dx, m.aux, &o, op);
            if (ob_event(m.t, m.x, m.dx, m.aux, &o, op)) {
                if (ev < ev_rows)
                    O_STORE_STATE(evt, evx, evdx, evaux, ev);
                ++ev;
                if (ob_on_event(m.t, m.x, m.dx, m.aux, &o, op))
                    break;
            }
        }
#undef O_STORE_STATE
        nStored[i] = (int)row;
        nEvents[i] = (int)ev;
        ob_write(&o, F, i, nPts);
        ob_rebase(m.t - ts[0], &o);
        obs[i] = o;
        o_member_store(&m, i, nPts, xf, rng, dtv, tf);
    }
}
#else
int o_odata_size(void) { return 0; }
#endif

#include CLODE_RHS_FILE
