/* Test infrastructure (the oracle), not product code.
 *
 * Precision typedefs and the OpenCL-C builtins a model's getRHS source may
 * use, so that the same model file the engine compiles for the GPU also
 * compiles as C11 for the CPU restatement in clode_oracle.c.
 * Precision selection follows clode/cpp/realtype.cl:9-45 (CLODE_SINGLE_PRECISION
 * / CLODE_DOUBLE_PRECISION, RCONST, BIG_REAL). */
#ifndef CLODE_PORT_SHIM_H
#define CLODE_PORT_SHIM_H

#include <stdbool.h>
#include <stdint.h>
#include <float.h>
#include <tgmath.h>

#if defined(CLODE_SINGLE_PRECISION)
typedef float realtype;
#define RCONST(x) (x##f)
#define BIG_REAL FLT_MAX
#elif defined(CLODE_DOUBLE_PRECISION)
typedef double realtype;
#define RCONST(x) (x)
#define BIG_REAL DBL_MAX
#else
#error "define CLODE_SINGLE_PRECISION or CLODE_DOUBLE_PRECISION"
#endif

#define ZERO RCONST(0.0)
#define ONE RCONST(1.0)

/* OpenCL address-space qualifiers are no-ops on the host */
#define __kernel
#define __global
#define __private
#define __local
#define __constant const

/* clode/cpp/clODE_utilities.cl:19 */
#define heaviside(x) ((x) >= ZERO ? ONE : ZERO)

/* OpenCL builtins that C lacks (OpenCL C 1.2 spec, section 6.12.2) */
static inline realtype acospi(realtype x) { return acos(x) / RCONST(3.14159265358979323846); }
static inline realtype asinpi(realtype x) { return asin(x) / RCONST(3.14159265358979323846); }
static inline realtype atanpi(realtype x) { return atan(x) / RCONST(3.14159265358979323846); }
static inline realtype atan2pi(realtype y, realtype x) { return atan2(y, x) / RCONST(3.14159265358979323846); }
static inline realtype cospi(realtype x) { return cos(x * RCONST(3.14159265358979323846)); }
static inline realtype sinpi(realtype x) { return sin(x * RCONST(3.14159265358979323846)); }
static inline realtype tanpi(realtype x) { return tan(x * RCONST(3.14159265358979323846)); }
static inline realtype exp10_(realtype x) { return pow(RCONST(10.0), x); }
#define exp10(x) exp10_(x)
static inline realtype pown(realtype x, int n) { return pow(x, (realtype)n); }
static inline realtype powr(realtype x, realtype y) { return pow(x, y); }
static inline realtype rootn(realtype x, int n) { return pow(x, ONE / (realtype)n); }
static inline realtype rsqrt(realtype x) { return ONE / sqrt(x); }
static inline realtype mad(realtype a, realtype b, realtype c) { return a * b + c; }
#define clamp(x, lo, hi) fmin(fmax((x), (lo)), (hi))

#endif
