// Jump-ahead of the per-member random stream (xoroshiro128+, the generator
// of clode/cpp/clODE_random.cl:28-44).  Its state transition is linear over
// GF(2) on the 128 state bits (rotations, shifts and xors only; the output
// s0 + s1 is not part of the state), so k steps are one 128 x 128 bit
// matrix, M^k, computed here by repeated squaring.  A matrix is stored as
// its 128 columns, column c = the image of the state with only bit c set
// (bits 0-63: s0, 64-127: s1), two 64-bit words each; applying it to a
// state xors the columns of the state's set bits.
#pragma once

#include <cstdint>
#include <vector>

namespace clode {

struct Gf2Mat {
    uint64_t col[128][2];
};

inline void xoroshiro_step(uint64_t &s0, uint64_t &s1)
{
    const uint64_t b = s1 ^ s0;
    s0 = ((s0 << 55) | (s0 >> 9)) ^ b ^ (b << 14);
    s1 = (b << 36) | (b >> 28);
}

inline void gf2_apply(const Gf2Mat &m, uint64_t &s0, uint64_t &s1)
{
    uint64_t r0 = 0, r1 = 0;
    for (int c = 0; c < 128; ++c) {
        const uint64_t bit = c < 64 ? (s0 >> c) & 1u : (s1 >> (c - 64)) & 1u;
        const uint64_t mask = 0 - bit;
        r0 ^= m.col[c][0] & mask;
        r1 ^= m.col[c][1] & mask;
    }
    s0 = r0;
    s1 = r1;
}

// a after b (the product a * b)
inline Gf2Mat gf2_mul(const Gf2Mat &a, const Gf2Mat &b)
{
    Gf2Mat r;
    for (int c = 0; c < 128; ++c) {
        uint64_t s0 = b.col[c][0], s1 = b.col[c][1];
        gf2_apply(a, s0, s1);
        r.col[c][0] = s0;
        r.col[c][1] = s1;
    }
    return r;
}

inline Gf2Mat gf2_step()
{
    Gf2Mat m;
    for (int c = 0; c < 128; ++c) {
        uint64_t s0 = c < 64 ? (uint64_t)1 << c : 0, s1 = c < 64 ? 0 : (uint64_t)1 << (c - 64);
        xoroshiro_step(s0, s1);
        m.col[c][0] = s0;
        m.col[c][1] = s1;
    }
    return m;
}

inline Gf2Mat gf2_identity()
{
    Gf2Mat m;
    for (int c = 0; c < 128; ++c) {
        m.col[c][0] = c < 64 ? (uint64_t)1 << c : 0;
        m.col[c][1] = c < 64 ? 0 : (uint64_t)1 << (c - 64);
    }
    return m;
}

// M^k: k steps of the generator
inline Gf2Mat gf2_jump(uint64_t k)
{
    Gf2Mat r = gf2_identity(), p = gf2_step();
    while (k) {
        if (k & 1u)
            r = gf2_mul(p, r);
        k >>= 1;
        if (k)
            p = gf2_mul(p, p);
    }
    return r;
}

}  // namespace clode
