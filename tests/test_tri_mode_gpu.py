"""The dense assembly's configuration test (pq3d_selftest_tri_mode): the
barycentric coordinates from the reciprocal of the denominator, decisions in
FP32 where the coordinates are well separated, the division-based test of
the reference (src/TDstressFS_C.cpp:125-166) elsewhere.  Its result must be
the division-based test's on every point, above all on the points where the
two could part: on the side lines and their extensions, on the lines where
two barycentric coordinates are equal (the boundaries of the -1 wedges), and
at every distance from them down to rounding."""
import numpy as np
import pytest

from pyquake3d_gb300 import _lib

pytestmark = pytest.mark.gpu


def _points(rng, n_tri=2000):
    rows = []
    for _ in range(n_tri):
        P1 = rng.normal(size=2) * rng.choice([1.0, 1e3, 1e5])
        P3 = rng.normal(size=2) * abs(P1).max() * rng.uniform(0.2, 2.0)
        den = -P3[1] * (P1[0] - P3[0]) + P3[0] * (P1[1] - P3[1])
        V = np.stack([P1, np.zeros(2), P3])
        lam = []
        lam.append(rng.uniform(-3, 4, size=(40, 3)))                 # anywhere
        t = rng.uniform(-3, 4, size=(30, 1))                          # side lines and extensions
        for k in range(3):
            l = np.concatenate([t, 1 - t, np.zeros_like(t)], axis=1)
            lam.append(np.roll(l, k, axis=1))
        t = rng.uniform(-3, 4, size=(30, 1))                          # two coordinates equal
        for k in range(3):
            l = np.concatenate([t, t, 1 - 2 * t], axis=1)
            lam.append(np.roll(l, k, axis=1))
        lam = np.concatenate(lam)
        yz = lam @ V
        # at every distance from those lines, down to rounding
        scale = abs(yz).max(axis=1, keepdims=True) + abs(V).max()
        eps = rng.choice([0.0, 1e-16, 1e-14, 1e-11, 1e-8, 1e-6, 1e-5, 1e-4], size=(len(yz), 1))
        yz = yz + eps * scale * rng.normal(size=yz.shape)
        x = np.where(rng.uniform(size=len(yz)) < 0.5, 0.0, rng.normal(size=len(yz)) * abs(V).max())
        for (y, z), xx in zip(yz, x):
            rows.append((xx, y, z, P1[0], P1[1], P3[0], P3[1], den))
    return np.ascontiguousarray(np.array(rows, dtype=np.float64))


def test_fast_configuration_test_equals_division_based(cuda):
    L = _lib.load()
    pts = _points(np.random.default_rng(3))
    n = pts.shape[0]
    fast = np.zeros(n, dtype=np.int32)
    exact = np.zeros(n, dtype=np.int32)
    _lib.check(L.pq3d_selftest_tri_mode(pts.ctypes.data, n, fast.ctypes.data, exact.ctypes.data))
    assert set(np.unique(exact)) == {-1, 0, 1}          # every outcome is exercised
    bad = np.nonzero(fast != exact)[0]
    assert len(bad) == 0, pts[bad[:5]]
