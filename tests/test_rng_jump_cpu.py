"""The random stream's jump matrices (host code, no GPU): the stream of
clode/cpp/clODE_random.cl:28-44 (xoroshiro128+, rotations 55/14/36) advanced
by k draws with one GF(2) matrix equals k sequential draws.  The pre-drawn
deviates of stochastic trajectory runs start each lane's block with these
matrices."""
import ctypes as C

import pytest

from clode_gb300 import _native as N

M64 = (1 << 64) - 1


def _step(s0, s1):
    b = s1 ^ s0
    s0 = (((s0 << 55) | (s0 >> 9)) & M64) ^ b ^ ((b << 14) & M64)
    s1 = ((b << 36) | (b >> 28)) & M64
    return s0, s1


@pytest.mark.parametrize("k", [0, 1, 2, 3, 63, 64, 1000, 2048, 4097])
def test_jump_equals_sequential_draws(k):
    s0, s1 = 0x9E3779B97F4A7C15, 0xD1B54A32D192ED03
    o0, o1 = C.c_ulonglong(), C.c_ulonglong()
    N.check(N.lib.clode_rng_jump(s0, s1, k, C.byref(o0), C.byref(o1)))
    a, b = s0, s1
    for _ in range(k):
        a, b = _step(a, b)
    assert (o0.value, o1.value) == (a, b)


def test_jumps_compose():
    s0, s1 = 12345, 67890
    o = [C.c_ulonglong() for _ in range(4)]
    N.check(N.lib.clode_rng_jump(s0, s1, 700, C.byref(o[0]), C.byref(o[1])))
    N.check(N.lib.clode_rng_jump(o[0].value, o[1].value, 324, C.byref(o[2]), C.byref(o[3])))
    d0, d1 = C.c_ulonglong(), C.c_ulonglong()
    N.check(N.lib.clode_rng_jump(s0, s1, 1024, C.byref(d0), C.byref(d1)))
    assert (o[2].value, o[3].value) == (d0.value, d1.value)
