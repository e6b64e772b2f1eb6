/* Test infrastructure (the checker), not product code.
 *
 * Lets the reference's OpenCL-C kernel sources compile unchanged as plain C11
 * on the host, so the reference's own arithmetic can pin the oracle and the
 * CUDA engine.  Included ahead of the reference sources by ref_driver.c.
 * Compile as C (not C++): the reference headers switch to their host-side
 * halves under __cplusplus (clode/cpp/steppers.cl:19, clode/cpp/observers.cl:22).
 * <stdlib.h> must stay out: clode/cpp/clODE_random.cl:81 defines rand(). */
#ifndef CLODE_REF_SHIM_H
#define CLODE_REF_SHIM_H

#include <stdbool.h>
#include <float.h>
#include <stdint.h>
#include <tgmath.h>

typedef uint64_t ulong;

/* vector types are only typedef'd by clode/cpp/realtype.cl:12-15,34-37 */
typedef struct { float v[2]; } float2;
typedef struct { float v[4]; } float4;
typedef struct { float v[8]; } float8;
typedef struct { float v[16]; } float16;
typedef struct { double v[2]; } double2;
typedef struct { double v[4]; } double4;
typedef struct { double v[8]; } double8;
typedef struct { double v[16]; } double16;

#define cl_khr_fp64 1
#define __kernel
#define __global
#define __private
#define __local
#define __constant const

/* work-item identity, set per member by the host loop */
extern __thread int clode_ref_gid;
extern __thread int clode_ref_gsize;
#define get_global_id(d) (clode_ref_gid)
#define get_global_size(d) (clode_ref_gsize)

/* OpenCL clamp = fmin(fmax(x, lo), hi) */
#define clamp(x, lo, hi) fmin(fmax((x), (lo)), (hi))

#endif
