/* Test infrastructure (the checker), not product code.
 *
 * Host loop over ensemble members for the reference's own kernels, compiled
 * from clode/cpp/{transient,initializeObserver,features,trajectory}.cl in
 * place.  Each exported function runs members [i0, i1) of an nPts-member
 * ensemble (SoA stride nPts), one member per loop iteration, exactly as one
 * OpenCL work-item would (clode/cpp/CLODE.cpp:484).  tspan_stride is 0 for
 * the reference's single global tspan, or 2 to hand each member its own
 * [t0, t1] pair (the kernels only read tspan[0] and tspan[1]).
 *
 * Built by oracle/build.py with the -D set of clode/cpp/CLODE.cpp:118-138 and
 * clode/cpp/CLODEfeatures.cpp:37-38, the model's getRHS file given by
 * -DCLODE_RHS_FILE. */
#include "ref_shim.h"

__thread int clode_ref_gid;
__thread int clode_ref_gsize;

#include "transient.cl"
#include "trajectory.cl"
#ifdef CLODE_WITH_OBSERVER
#include "initializeObserver.cl"
#include "features.cl"
#endif

#include CLODE_RHS_FILE

#ifdef _OPENMP
#include <omp.h>
#define CLODE_OMP_FOR _Pragma("omp parallel for schedule(dynamic, 8) num_threads(nthreads)")
#else
#define CLODE_OMP_FOR
#endif

int o_real_size(void) { return (int)sizeof(realtype); }

int o_odata_size(void)
{
#ifdef CLODE_WITH_OBSERVER
    return (int)sizeof(ObserverData);
#else
    return 0;
#endif
}

int o_is_reference(void) { return 1; }

void o_transient(int nPts, int i0, int i1, int nthreads, const realtype *tspan, int tspan_stride,
                 realtype *x0, const realtype *pars, const void *sp, realtype *xf,
                 ulong *rng, realtype *dt, realtype *tf)
{
    if (nthreads < 1) nthreads = 1;
    CLODE_OMP_FOR
    for (int i = i0; i < i1; ++i) {
        clode_ref_gid = i;
        clode_ref_gsize = nPts;
        transient(tspan + (long)tspan_stride * i, x0, pars, (const struct SolverParams *)sp, xf, rng, dt, tf);
    }
}

void o_trajectory(int nPts, int i0, int i1, int nthreads, const realtype *tspan, int tspan_stride,
                  realtype *x0, const realtype *pars, const void *sp, realtype *xf,
                  ulong *rng, realtype *dt, realtype *tf, realtype *t, realtype *x,
                  realtype *dx, realtype *aux, int *nStored)
{
    if (nthreads < 1) nthreads = 1;
    CLODE_OMP_FOR
    for (int i = i0; i < i1; ++i) {
        clode_ref_gid = i;
        clode_ref_gsize = nPts;
        trajectory(tspan + (long)tspan_stride * i, x0, pars, (const struct SolverParams *)sp, xf, rng, dt, tf,
                   t, x, dx, aux, nStored);
    }
}

#ifdef CLODE_WITH_OBSERVER
void o_init_observer(int nPts, int i0, int i1, int nthreads, const realtype *tspan, int tspan_stride,
                     realtype *x0, const realtype *pars, const void *sp, ulong *rng,
                     realtype *dt, void *odata, const void *op)
{
    if (nthreads < 1) nthreads = 1;
    CLODE_OMP_FOR
    for (int i = i0; i < i1; ++i) {
        clode_ref_gid = i;
        clode_ref_gsize = nPts;
        initializeObserver(tspan + (long)tspan_stride * i, x0, pars, (const struct SolverParams *)sp, rng, dt,
                           (ObserverData *)odata, (const struct ObserverParams *)op);
    }
}

void o_features(int nPts, int i0, int i1, int nthreads, const realtype *tspan, int tspan_stride,
                realtype *x0, const realtype *pars, const void *sp, realtype *xf,
                ulong *rng, realtype *dt, realtype *tf, void *odata, const void *op, realtype *F)
{
    if (nthreads < 1) nthreads = 1;
    CLODE_OMP_FOR
    for (int i = i0; i < i1; ++i) {
        clode_ref_gid = i;
        clode_ref_gsize = nPts;
        features(tspan + (long)tspan_stride * i, x0, pars, (const struct SolverParams *)sp, xf, rng, dt, tf,
                 (ObserverData *)odata, (const struct ObserverParams *)op, F);
    }
}
#endif
