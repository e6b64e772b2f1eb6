// Per-member random stream, bit-compatible with clODE's: xoroshiro128+
// (rotations 55/14/36, clode/cpp/clODE_random.cl:28-44), uniforms as
// u64 * 2^-64 rounded to working precision (:26, :81-85), and polar
// Box-Muller normals with the second deviate cached (:88-114).  The state is
// two u64 words per member, SoA [j * nPts + i] in global memory; the cache
// flag is reset at every launch as in clode/cpp/transient.cl:42.
#pragma once

namespace clode {

struct Rng {
    unsigned long long s0, s1;
    realtype spare;
    bool have_spare;
};

__device__ __forceinline__ unsigned long long rotl64(unsigned long long v, int k)
{
    return (v << k) | (v >> (64 - k));
}

__device__ __forceinline__ unsigned long long rng_next(Rng &r)
{
    unsigned long long a = r.s0, b = r.s1;
    unsigned long long out = a + b;
    b ^= a;
    r.s0 = rotl64(a, 55) ^ b ^ (b << 14);
    r.s1 = rotl64(b, 36);
    return out;
}

// products and sums that must never be contracted into an FMA: the rejection
// test below decides how many draws a normal costs, so it has to round
// exactly like the reference whatever --fmad the rest of the program uses
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }

__device__ __forceinline__ realtype rng_uniform(Rng &r)
{
    // u64 -> working precision with round-to-nearest, then scale by 2^-64
    return mul_rn((realtype)rng_next(r), RCONST(5.421010862427522e-20));
}

// one candidate of the polar method: (u, v) from two uniforms, and s =
// u^2 + v^2; the candidate is accepted when s < 1
__device__ __forceinline__ realtype polar_candidate(Rng &r, realtype &u, realtype &v)
{
    u = add_rn(mul_rn(RCONST(2.0), rng_uniform(r)), -ONE);
    v = add_rn(mul_rn(RCONST(2.0), rng_uniform(r)), -ONE);
    return add_rn(mul_rn(u, u), mul_rn(v, v));
}

// the two deviates of an accepted candidate, in the order they are used
__device__ __forceinline__ void polar_pair(realtype u, realtype v, realtype s, realtype &y1, realtype &y2)
{
    const realtype m = sqrt((-RCONST(2.0) * log(s)) / s);
    y1 = u * m;
    y2 = v * m;
}

__device__ __forceinline__ realtype rng_normal(Rng &r)
{
    if (r.have_spare) {
        r.have_spare = false;
        return r.spare;
    }
    realtype u, v, s;
    do {
        s = polar_candidate(r, u, v);
    } while (s >= ONE);
    realtype y1;
    polar_pair(u, v, s, y1, r.spare);
    r.have_spare = true;
    return y1;
}

}  // namespace clode
