"""Edge cases of the reference C ABI (TDstressFS_C, TDstressEachSourceAtReceiver_C)
on the GPU: empty inputs, degenerate sources (the reference returns NaN for a
triangle of zero area), and a point set of 2^21 receivers in one call against
the CPU oracle on a seeded sample."""
import ctypes

import numpy as np
import pytest

import oracle
from pyquake3d_gb300 import _lib
from tests.util import normwise_rel

pytestmark = pytest.mark.gpu
MU = 32038120320.0
D = ctypes.POINTER(ctypes.c_double)


def _p(a):
    return a.ctypes.data_as(D)


def _call(L, R, P, b=(1.0, 0.0, 0.0), half=False):
    x, y, z = (np.ascontiguousarray(R[:, k]) for k in range(3))
    n = R.shape[0]
    s = np.full((max(n, 1), 6), 7.0)
    e = np.full((max(n, 1), 6), 7.0)
    P1, P2, P3 = (np.ascontiguousarray(p, dtype=np.float64) for p in P)
    L.TDstressFS_C(_p(x), _p(y), _p(z), n, _p(P1), _p(P2), _p(P3), b[0], b[1], b[2], MU, MU, half, _p(s), _p(e))
    return s, e


TRI = (np.array([-1000.0, 0.0, -3000.0]), np.array([1000.0, 0.0, -3000.0]), np.array([0.0, 0.0, -1500.0]))


@pytest.mark.parametrize("half", [False, True])
def test_empty_point_set_writes_nothing(cuda, half):
    L = _lib.load()
    s, e = _call(L, np.zeros((0, 3)), TRI, half=half)
    assert np.all(s == 7.0) and np.all(e == 7.0)
    so, eo = np.full((1, 6), 7.0), np.full((1, 6), 7.0)
    P = np.zeros((1, 3))
    L.TDstressEachSourceAtReceiver_C(0.0, 0.0, -100.0, _p(P), _p(P), _p(P), 0, 1.0, 0.0, 0.0, MU, MU, half,
                                     _p(so), _p(eo))
    assert np.all(so == 7.0) and np.all(eo == 7.0)
    assert _lib.load().pq3d_last_error().decode() == ""


@pytest.mark.parametrize("P", [
    (np.array([0.0, 0.0, -1000.0]), np.array([1000.0, 0.0, -1000.0]), np.array([2000.0, 0.0, -1000.0])),
    (np.array([0.0, 0.0, -1000.0]),) * 3])
def test_degenerate_source_gives_nan_like_the_reference(cuda, P):
    """Collinear vertices and a point triangle: the reference C++ returns NaN
    for every receiver (its normal is 0/0); so does this library."""
    L = _lib.load()
    R = np.array([[100.0, 200.0, -500.0], [0.0, 0.0, -1000.0], [50.0, -30.0, -2000.0]])
    s, e = _call(L, R, P)
    assert np.all(np.isnan(s)) and np.all(np.isnan(e))


def test_two_million_receivers_in_one_call(cuda):
    """2^21 receivers of one source (one launch of 16,384 blocks) against the
    C oracle on 2,000 seeded receivers, normwise 1e-10."""
    L = _lib.load()
    rng = np.random.default_rng(21)
    n = 1 << 21
    R = np.empty((n, 3))
    R[:, 0] = rng.uniform(-20e3, 20e3, n)
    R[:, 1] = rng.uniform(-20e3, 20e3, n)
    R[:, 2] = rng.uniform(-20e3, -10.0, n)
    s, e = _call(L, R, TRI, b=(0.3, 1.0, -0.2))
    pick = np.sort(rng.choice(n, 2000, replace=False))
    Rp = R[pick]
    so, eo = oracle.tdstress(Rp[:, 0].copy(), Rp[:, 1].copy(), Rp[:, 2].copy(), *TRI, 0.3, 1.0, -0.2, MU, MU)
    assert normwise_rel(so, s[pick]) < 1e-10
    assert normwise_rel(eo, e[pick]) < 1e-10
    assert np.all(np.isfinite(s))
