"""CPU oracle (test infrastructure only).

Loaded by tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline
leg -- never by the product package.  ``gf`` wraps the C restatement in
tdstress_oracle.c (built by ``make -C oracle``); ``stepping`` and ``hmatrix``
are NumPy restatements.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_D = ctypes.POINTER(ctypes.c_double)
_L = ctypes.POINTER(ctypes.c_longlong)
_lib = None


def build() -> str:
    subprocess.check_call(["make", "-s", "-C", HERE])
    return os.path.join(HERE, "liboracle_gf.so")


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "liboracle_gf.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        L.oracle_TDstressFS_C.argtypes = [_D, _D, _D, ctypes.c_size_t, _D, _D, _D] + [ctypes.c_double] * 5 + [ctypes.c_bool, _D, _D]
        L.oracle_TDstressFS_C.restype = None
        L.oracle_TDstressEachSourceAtReceiver_C.argtypes = [ctypes.c_double] * 3 + [_D, _D, _D, ctypes.c_size_t] + [ctypes.c_double] * 5 + [ctypes.c_bool, _D, _D]
        L.oracle_TDstressEachSourceAtReceiver_C.restype = None
        L.oracle_element_frames.argtypes = [_D, _L, ctypes.c_size_t, _D, _D]
        L.oracle_element_frames.restype = None
        L.oracle_assemble_dense.argtypes = [_D, _L, ctypes.c_size_t, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                            ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int, _D]
        L.oracle_assemble_dense.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(_D)


def tdstress(X, Y, Z, P1, P2, P3, Ss, Ds, Ts, mu, lam, halfspace=False):
    """Stress, strain (n, 6) at receivers from one triangle (reference TDstressFS_C)."""
    X, Y, Z = (np.ascontiguousarray(v, dtype=np.float64) for v in (X, Y, Z))
    P1, P2, P3 = (np.ascontiguousarray(v, dtype=np.float64) for v in (P1, P2, P3))
    n = X.size
    s = np.zeros((n, 6))
    e = np.zeros((n, 6))
    lib().oracle_TDstressFS_C(_p(X), _p(Y), _p(Z), n, _p(P1), _p(P2), _p(P3), Ss, Ds, Ts, mu, lam,
                              bool(halfspace), _p(s), _p(e))
    return s, e


def tdstress_each_source(x, y, z, P1, P2, P3, Ss, Ds, Ts, mu, lam, halfspace=False):
    """Stress, strain (ns, 6) at one receiver from many triangles."""
    P1, P2, P3 = (np.ascontiguousarray(v, dtype=np.float64) for v in (P1, P2, P3))
    ns = P1.shape[0]
    s = np.zeros((ns, 6))
    e = np.zeros((ns, 6))
    lib().oracle_TDstressEachSourceAtReceiver_C(x, y, z, _p(P1), _p(P2), _p(P3), ns, Ss, Ds, Ts, mu, lam,
                                                bool(halfspace), _p(s), _p(e))
    return s, e


def assemble_dense(nodes, tris, mu, lam, halfspace=False, cols=None, nthreads=1):
    """Six N x N traction operators (A1s, A2s, Bs, A1d, A2d, Bd) -> array (6, N, N).

    ``cols=(c0, c1)`` restricts the work to source columns [c0, c1)."""
    nodes = np.ascontiguousarray(nodes, dtype=np.float64)
    tris = np.ascontiguousarray(tris, dtype=np.int64)
    N = tris.shape[0]
    c0, c1 = (0, N) if cols is None else cols
    out = np.zeros((6, N, N))
    rc = lib().oracle_assemble_dense(_p(nodes), tris.ctypes.data_as(_L), N, mu, lam, int(bool(halfspace)),
                                     c0, c1, int(nthreads), _p(out))
    if rc != 0:
        raise MemoryError("oracle_assemble_dense failed")
    return out


OPS = ("A1s", "A2s", "Bs", "A1d", "A2d", "Bd")
