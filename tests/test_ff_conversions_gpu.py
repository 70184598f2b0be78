"""The FP64 <-> float-float conversions of the float-float attempt, which the
device does with integer bit operations (no FP64-pipe conversions), against
NumPy's own conversions on the values the steppers reach only in rare states:
FP32 subnormals, zeros, infinities and NaN widened to FP64; FP64 values in and
outside the split's fast range [2^-60, 2^127); and the float-float norm of the
update kernel |(x, y)| against numpy.hypot."""
import ctypes

import numpy as np
import pytest

from pyquake3d_gb300 import _lib

pytestmark = pytest.mark.gpu


def _run(x, f, y):
    L = _lib.load()
    n = len(x)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    f = np.ascontiguousarray(f, dtype=np.float32)
    ff = np.empty(2 * n, dtype=np.float32)
    d = np.empty(n)
    h = np.empty(n)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    _lib.check(L.pq3d_selftest_ff_conversions(p(x), p(f), p(y), n, p(ff), p(d), p(h)))
    return ff.reshape(n, 2), d, h


def test_float_to_fp64_by_bits_matches_conversion(cuda):
    rng = np.random.default_rng(0)
    sub = np.array([1, 2, 3, 0x400000, 0x7fffff, 0x123456] + list(rng.integers(1, 1 << 23, size=200)), dtype=np.uint32)
    bits = np.concatenate([sub, sub | 0x80000000,
                           np.array([0, 0x80000000, 0x7f800000, 0xff800000, 0x7fc00000, 0x7f7fffff, 0x00800000,
                                     0x3f800000], dtype=np.uint32),
                           rng.integers(0, 1 << 32, size=2000, dtype=np.uint64).astype(np.uint32)])
    f = bits.view(np.float32)
    n = len(f)
    _, d, _ = _run(np.ones(n), f, np.ones(n))
    with np.errstate(invalid="ignore"):   # signalling NaN inputs
        ref = f.astype(np.float64)
    nan = np.isnan(ref)
    assert np.array_equal(np.isnan(d), nan)
    assert np.array_equal(d[~nan].view(np.uint64), ref[~nan].view(np.uint64))   # bit for bit, signed zeros included


def test_fp64_split_and_norm(cuda):
    rng = np.random.default_rng(1)
    fast = rng.uniform(-1, 1, 3000) * 2.0 ** rng.uniform(-59, 126, 3000)
    rare = np.array([1e-30, -3e-25, 2.0 ** -61, 1e40, -1e300, 5e-324, 0.0, -0.0, np.inf, -np.inf, 2.0 ** 127,
                     2.0 ** -60])
    x = np.concatenate([fast, rare])
    y = np.concatenate([rng.uniform(-1, 1, len(fast)) * 10 ** rng.uniform(-20, 2, len(fast)),
                        np.array([1e-30, 0.0, 1.0, 1e-20, 2.0, 0.0, 0.0, 0.0, 1.0, 1.0, 1.0, 1.0])])
    ff, _, h = _run(x, np.ones(len(x), dtype=np.float32), y)
    hi, lo = ff[:, 0].astype(np.float64), ff[:, 1].astype(np.float64)
    # fast range: hi + lo within 2^-47 |x|, normalised (hi = hi + lo rounded)
    k = len(fast)
    assert np.all(np.abs(x[:k] - (hi[:k] + lo[:k])) <= 2.0 ** -47 * np.abs(x[:k]))
    assert np.all((ff[:k, 0] + ff[:k, 1]) == ff[:k, 0])
    # outside it: the plain conversions, hi = float(x), lo = float(x - hi)
    r = slice(k, None)
    with np.errstate(over="ignore", invalid="ignore"):
        h_ref = x[r].astype(np.float32)
        l_ref = np.where(np.isfinite(h_ref), (x[r] - h_ref.astype(np.float64)), 0.0).astype(np.float32)
    ok = np.isfinite(h_ref)
    assert np.array_equal(ff[r, 0][ok], h_ref[ok]) and np.array_equal(ff[r, 1][ok], l_ref[ok])
    assert np.array_equal(np.isinf(ff[r, 0]), np.isinf(h_ref))
    # the norm: float-float accuracy wherever both components and |(x, y)| are FP32 numbers
    m = (np.abs(x) < 1e30) & (np.abs(x) > 1e-30) | (x == 0)
    m &= (np.abs(y) < 1e30) & ((np.abs(y) > 1e-30) | (y == 0))
    with np.errstate(invalid="ignore"):   # the infinite inputs, masked out below
        ref = np.hypot(hi + lo, y)
    rel = np.abs(h[m] - ref[m]) / np.where(ref[m] > 0, ref[m], 1.0)
    assert rel.max() < 1e-13, rel.max()
