// OpenCL-C compatibility for user model sources compiled by NVRTC.
//
// A clODE model is an OpenCL-C function
//   void getRHS(const realtype t, const realtype x_[], const realtype p_[],
//               realtype dx_[], realtype aux_[], const realtype w_[]);
// (forward declaration: clode/cpp/steppers.cl:50).  It is compiled unchanged
// as CUDA C++ with NVRTC's -default-device, so everything it may name from
// the OpenCL side is defined here: the precision typedefs and constants of
// clode/cpp/realtype.cl:9-45, the heaviside macro of
// clode/cpp/clODE_utilities.cl:19, address-space qualifiers, OpenCL scalar
// type names, and the OpenCL math builtins that CUDA lacks (the set the
// reference's Python converter may emit, clode/function_converter.py:54-124).
// This header is self-contained: NVRTC compiles it without system headers.
#pragma once

#if defined(CLODE_SINGLE_PRECISION)
typedef float realtype;
#define RCONST(x) (x##f)
#define BIG_REAL 3.402823466e+38f
#define SMALL_REAL 1.175494351e-38f
#define UNIT_ROUNDOFF 1.192092896e-07f
#elif defined(CLODE_DOUBLE_PRECISION)
typedef double realtype;
#define RCONST(x) (x)
#define BIG_REAL 1.7976931348623157e+308
#define SMALL_REAL 2.2250738585072014e-308
#define UNIT_ROUNDOFF 2.2204460492503131e-16
#else
#error "CLODE_SINGLE_PRECISION or CLODE_DOUBLE_PRECISION must be defined"
#endif

#ifndef ZERO
#define ZERO RCONST(0.0)
#endif
#ifndef ONE
#define ONE RCONST(1.0)
#endif

#define __kernel
#define __global
#define __private
#define __local
#define __constant const

typedef unsigned char uchar;
typedef unsigned short ushort;
typedef unsigned int uint;
typedef unsigned long long ulong;

#define heaviside(x) ((x) >= ZERO ? ONE : ZERO)
#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
#ifndef M_PI_F
#define M_PI_F 3.14159265358979323846f
#endif

// OpenCL builtins without a CUDA counterpart of the same name (OpenCL C 1.2, 6.12.2)
__device__ __forceinline__ float acospi(float x) { return acosf(x) / M_PI_F; }
__device__ __forceinline__ double acospi(double x) { return acos(x) / M_PI; }
__device__ __forceinline__ float asinpi(float x) { return asinf(x) / M_PI_F; }
__device__ __forceinline__ double asinpi(double x) { return asin(x) / M_PI; }
__device__ __forceinline__ float atanpi(float x) { return atanf(x) / M_PI_F; }
__device__ __forceinline__ double atanpi(double x) { return atan(x) / M_PI; }
__device__ __forceinline__ float atan2pi(float y, float x) { return atan2f(y, x) / M_PI_F; }
__device__ __forceinline__ double atan2pi(double y, double x) { return atan2(y, x) / M_PI; }
__device__ __forceinline__ float tanpi(float x) { return tanf(x * M_PI_F); }
__device__ __forceinline__ double tanpi(double x) { return tan(x * M_PI); }
__device__ __forceinline__ float pown(float x, int n) { return powf(x, (float)n); }
__device__ __forceinline__ double pown(double x, int n) { return pow(x, (double)n); }
__device__ __forceinline__ float powr(float x, float y) { return powf(x, y); }
__device__ __forceinline__ double powr(double x, double y) { return pow(x, y); }
__device__ __forceinline__ float rootn(float x, int n) { return powf(x, 1.0f / (float)n); }
__device__ __forceinline__ double rootn(double x, int n) { return pow(x, 1.0 / (double)n); }
__device__ __forceinline__ float mad(float a, float b, float c) { return a * b + c; }
__device__ __forceinline__ double mad(double a, double b, double c) { return a * b + c; }
__device__ __forceinline__ float fract(float x, float *ip) { float f = floorf(x); *ip = f; return fminf(x - f, 0x1.fffffep-1f); }
__device__ __forceinline__ double fract(double x, double *ip) { double f = floor(x); *ip = f; return fmin(x - f, 0x1.fffffffffffffp-1); }
__device__ __forceinline__ float clamp(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
__device__ __forceinline__ double clamp(double x, double lo, double hi) { return fmin(fmax(x, lo), hi); }
__device__ __forceinline__ float sign(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : (x == x ? 0.0f * x : 0.0f)); }
__device__ __forceinline__ double sign(double x) { return x > 0.0 ? 1.0 : (x < 0.0 ? -1.0 : (x == x ? 0.0 * x : 0.0)); }
__device__ __forceinline__ float step(float edge, float x) { return x < edge ? 0.0f : 1.0f; }
__device__ __forceinline__ double step(double edge, double x) { return x < edge ? 0.0 : 1.0; }
__device__ __forceinline__ float mix(float a, float b, float t) { return a + (b - a) * t; }
__device__ __forceinline__ double mix(double a, double b, double t) { return a + (b - a) * t; }
__device__ __forceinline__ float degrees(float r) { return r * (180.0f / M_PI_F); }
__device__ __forceinline__ double degrees(double r) { return r * (180.0 / M_PI); }
__device__ __forceinline__ float radians(float d) { return d * (M_PI_F / 180.0f); }
__device__ __forceinline__ double radians(double d) { return d * (M_PI / 180.0); }
__device__ __forceinline__ float maxmag(float x, float y) { float ax = fabsf(x), ay = fabsf(y); return ax > ay ? x : (ay > ax ? y : fmaxf(x, y)); }
__device__ __forceinline__ double maxmag(double x, double y) { double ax = fabs(x), ay = fabs(y); return ax > ay ? x : (ay > ax ? y : fmax(x, y)); }
__device__ __forceinline__ float minmag(float x, float y) { float ax = fabsf(x), ay = fabsf(y); return ax < ay ? x : (ay < ax ? y : fminf(x, y)); }
__device__ __forceinline__ double minmag(double x, double y) { double ax = fabs(x), ay = fabs(y); return ax < ay ? x : (ay < ax ? y : fmin(x, y)); }
__device__ __forceinline__ float smoothstep(float e0, float e1, float x) { float t = clamp((x - e0) / (e1 - e0), 0.0f, 1.0f); return t * t * (3.0f - 2.0f * t); }
__device__ __forceinline__ double smoothstep(double e0, double e1, double x) { double t = clamp((x - e0) / (e1 - e0), 0.0, 1.0); return t * t * (3.0 - 2.0 * t); }
// OpenCL sincos(x, *cosval) returns the sine and stores the cosine
__device__ __forceinline__ float sincos(float x, float *c) { float s; sincosf(x, &s, c); return s; }
__device__ __forceinline__ double sincos(double x, double *c) { double s; ::sincos(x, &s, c); return s; }
// gamma is what the reference converter emits for Python's math.gamma
__device__ __forceinline__ float gamma(float x) { return tgammaf(x); }
__device__ __forceinline__ double gamma(double x) { return tgamma(x); }

// Optional faster FP32 exp (build define CLODE_FAST_EXP=1, simulator option
// "fast_exp"): Cody-Waite splitting of x * log2(e) into the rounded product
// y and its exact remainder r (two fma), 2^y from the hardware base-2
// exponential, times (1 + r ln 2).  Within a few ulp of the correctly rounded
// result over the normal range (tested against CUDA's expf); where 2^y
// overflows or underflows the hardware result (inf, 0) is returned as is.
// FP64 keeps exp().
#if defined(CLODE_FAST_EXP) && CLODE_FAST_EXP
__device__ __forceinline__ float clode_exp_f32(float x)
{
    const float l2e_hi = 1.44269502162933349609375f;  // log2(e) rounded to FP32
    const float l2e_lo = 1.925963033500011e-08f;       // log2(e) - l2e_hi
    const float y = x * l2e_hi;
    float r = fmaf(x, l2e_hi, -y);
    r = fmaf(x, l2e_lo, r);
    float e;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(e) : "f"(y));
    const float corr = fmaf(e, r * 0.693147182464599609375f, e);
    return fabsf(y) < 128.0f ? corr : e;  // beyond: inf or 0, where the correction would give NaN
}
__device__ __forceinline__ float clode_exp(float x) { return clode_exp_f32(x); }
__device__ __forceinline__ double clode_exp(double x) { return ::exp(x); }
#define exp(x) clode_exp(x)
#endif

// native_* and half_* variants map to the accurate functions
#define native_exp exp
#define native_exp2 exp2
#define native_exp10 exp10
#define native_log log
#define native_log2 log2
#define native_log10 log10
#define native_sqrt sqrt
#define native_rsqrt rsqrt
#define native_sin sin
#define native_cos cos
#define native_tan tan
#define native_powr powr
#define native_recip(x) (ONE / (x))
#define native_divide(a, b) ((a) / (b))
#define half_exp exp
#define half_log log
#define half_sqrt sqrt
#define half_rsqrt rsqrt
#define half_sin sin
#define half_cos cos
#define half_powr powr
#define half_recip(x) (ONE / (x))
#define half_divide(a, b) ((a) / (b))
