"""The mixed stage's join of a float pair into one FP64 value by integer
operations (pair_to_double, nekgpu_pair.cuh), through its test hook
nekgpu_selftest_pair_join, against exact rational sums.

The pairs are two-sum outputs (s = fl(p + e), t = p + e - s exactly, so
|t| <= ulp(s)/2), as the finish forms them: random magnitudes and signs,
s a power of two with t of either sign (the borrow across a binade), t zero,
t far below s (bits beyond 53 truncated), and s near the float range ends.
The result must equal the exact sum whenever that is an FP64 value, and lie
within one FP64 ulp of it otherwise.
"""
from __future__ import annotations

import math
from fractions import Fraction

import numpy as np
import pytest

from nekcem_gb300 import _lib as L

pytestmark = pytest.mark.gpu


def two_sum32(p: np.ndarray, e: np.ndarray):
    p = p.astype(np.float32)
    e = e.astype(np.float32)
    s = (p + e).astype(np.float32)
    bb = (s - p).astype(np.float32)
    t = ((p - (s - bb)) + (e - bb)).astype(np.float32)
    return s, t


def pairs(n: int, seed: int):
    rng = np.random.default_rng(seed)
    mag = np.ldexp(rng.random(n) + 0.5, rng.integers(-60, 60, n))
    p = (mag * rng.choice([-1.0, 1.0], n)).astype(np.float32)
    rel = np.ldexp(rng.random(n), -rng.integers(0, 60, n)) * rng.choice([-1.0, 1.0], n)
    e = (p.astype(np.float64) * rel).astype(np.float32)
    k = n // 8
    # powers of two with t of either sign
    p[:k] = np.ldexp(rng.choice([-1.0, 1.0], k), rng.integers(-40, 40, k)).astype(np.float32)
    e[:k] = (p[:k].astype(np.float64) * np.ldexp(rng.random(k), -rng.integers(1, 40, k))
             * rng.choice([-1.0, 1.0], k)).astype(np.float32)
    e[k:2 * k] = 0.0                                   # t = 0
    p[2 * k:2 * k + 4] = [1e38, -1e38, 3e-37, -3e-37]  # near the float range ends
    return two_sum32(p, e)


def test_pair_join_matches_exact_sums():
    s, t = pairs(20000, 11)
    out = np.empty(s.size)
    L.check(L.load().nekgpu_selftest_pair_join(s.ctypes.data, t.ctypes.data,
                                               out.ctypes.data_as(L.dp), s.size),
            "nekgpu_selftest_pair_join")
    exact_hits = 0
    tiny = Fraction(2) ** -126  # subnormal t is dropped (documented bound)
    for si, ti, oi in zip(s.tolist(), t.tolist(), out.tolist()):
        assert abs(ti) <= float(np.spacing(np.float32(abs(si)))) / 2 or si == 0.0
        exact = Fraction(si) + Fraction(ti)
        if abs(ti) < 2.0 ** -126:
            assert abs(Fraction(oi) - exact) < tiny, (si, ti, oi)
        elif Fraction(float(exact)) == exact:  # the sum is an FP64 value
            assert oi == float(exact), (si, ti, oi)
            exact_hits += 1
        else:
            assert abs(Fraction(oi) - exact) < Fraction(math.ulp(oi)), (si, ti, oi)
    assert exact_hits > s.size // 4  # the pairs whose sum fits in 53 bits (~40 % here)


def test_pair_join_rejects_bad_arguments():
    s = np.zeros(4, np.float32)
    out = np.empty(4)
    lib = L.load()
    assert lib.nekgpu_selftest_pair_join(s.ctypes.data, s.ctypes.data, out.ctypes.data_as(L.dp), 0) == -1
    assert lib.nekgpu_selftest_pair_join(None, s.ctypes.data, out.ctypes.data_as(L.dp), 4) == -1
