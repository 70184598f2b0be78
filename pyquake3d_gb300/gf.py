"""Green's-function assembly on the GPU (torch tensors as device containers).

``assemble_dense`` builds the dense traction operator of a triangulated fault
as one (3N) x (2N) row-major FP64 matrix (and optionally its FP32 copy):
row 3i+c = traction component c (e1, e2, normal) at the centroid of element i,
column 2j+s = unit slip s (strike, dip) on element j.  ``split_ops`` returns
the reference's six N x N matrices A1s, A2s, Bs, A1d, A2d, Bd as strided views
(src/QDsim_gpu.py:1787-1878 builds them one source column at a time).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib

OPS = ("A1s", "A2s", "Bs", "A1d", "A2d", "Bd")
# (component c, slip s) of each reference matrix
OP_INDEX = {"A1s": (0, 0), "A2s": (1, 0), "Bs": (2, 0), "A1d": (0, 1), "A2d": (1, 1), "Bd": (2, 1)}


def _stream(device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def mesh_to_device(nodes, tris, device="cuda"):
    nodes_t = torch.as_tensor(np.ascontiguousarray(nodes, dtype=np.float64), device=device)
    tris_t = torch.as_tensor(np.ascontiguousarray(tris, dtype=np.int64), device=device)
    return nodes_t, tris_t


def assemble_dense(nodes, tris, mu, lam, *, halfspace=False, fp32_copy=True, device="cuda",
                   rows=None, out64=None, out32=None, workspace=None):
    """Assemble K (FP64) and its FP32 copy on ``device``.

    nodes: (Nn, 3) metres; tris: (N, 3) 1-based.  ``rows=(r0, r1)`` assembles
    receivers [r0, r1) only (the returned tensors then have 3*(r1-r0) rows).
    Returns (K64, K32 or None).
    """
    L = _lib.load()
    if not torch.cuda.is_available():
        raise RuntimeError("assemble_dense needs a CUDA device")
    if isinstance(nodes, torch.Tensor) and nodes.is_cuda:
        nodes_t, tris_t = nodes.contiguous(), tris.contiguous()
    else:
        nodes_t, tris_t = mesh_to_device(nodes, tris, device)
    N = int(tris_t.shape[0])
    r0, r1 = (0, N) if rows is None else rows
    dev = nodes_t.device
    K64 = out64 if out64 is not None else torch.empty((3 * (r1 - r0), 2 * N), dtype=torch.float64, device=dev)
    K32 = None
    if fp32_copy:
        K32 = out32 if out32 is not None else torch.empty((3 * (r1 - r0), 2 * N), dtype=torch.float32, device=dev)
    wsb = L.pq3d_gf_workspace_bytes(N)
    ws = workspace if workspace is not None else torch.empty(wsb, dtype=torch.uint8, device=dev)
    rc = L.pq3d_assemble_dense(nodes_t.data_ptr(), tris_t.data_ptr(), N, r0, r1, float(mu), float(lam),
                               int(bool(halfspace)), K64.data_ptr(), K32.data_ptr() if K32 is not None else None,
                               ws.data_ptr(), ws.numel(), _stream(dev))
    _lib.check(rc)
    return K64, K32


def assemble_dense_host(nodes, tris, mu, lam, *, halfspace=False, fp32_copy=False, out64=None, out32=None):
    """Host-buffer assembly: mesh and operator live in host memory (pinned
    torch tensors are used when no output is given).  Returns (K64, K32)."""
    L = _lib.load()
    nodes = np.ascontiguousarray(nodes, dtype=np.float64)
    tris = np.ascontiguousarray(tris, dtype=np.int64)
    N = tris.shape[0]
    K64 = out64 if out64 is not None else torch.empty((3 * N, 2 * N), dtype=torch.float64).pin_memory()
    K32 = None
    if fp32_copy:
        K32 = out32 if out32 is not None else torch.empty((3 * N, 2 * N), dtype=torch.float32).pin_memory()
    rc = L.pq3d_assemble_dense_host(nodes.ctypes.data, nodes.shape[0], tris.ctypes.data, N, float(mu), float(lam),
                                    int(bool(halfspace)), K64.data_ptr(), K32.data_ptr() if K32 is not None else None)
    _lib.check(rc)
    return K64, K32


def split_ops(K):
    """The six reference matrices as strided views of K ((3N) x (2N))."""
    N = K.shape[1] // 2
    V = K.view(K.shape[0] // 3, 3, N, 2)
    return {name: V[:, c, :, s] for name, (c, s) in OP_INDEX.items()}


def join_ops(ops):
    """Inverse of split_ops for host arrays: dict of six N x N -> (3N, 2N)."""
    A = ops["A1s"]
    N = A.shape[0]
    K = np.empty((N, 3, N, 2), dtype=np.asarray(A).dtype)
    for name, (c, s) in OP_INDEX.items():
        K[:, c, :, s] = ops[name]
    return K.reshape(3 * N, 2 * N)


def _dp(a):
    return a.ctypes.data_as(_lib.c_double_p)


def TDstressFS(X, Y, Z, P1, P2, P3, Ss, Ds, Ts, mu, lambda_, halfspace=False):
    """Reference-shaped call (src/SH_greenfunction.py:200, src/TDstressFS_C.cpp:2095)
    on the GPU: returns (Stress (6, n), Strain (6, n)) like the NumPy twin."""
    L = _lib.load()
    X, Y, Z = (np.ascontiguousarray(np.atleast_1d(v), dtype=np.float64) for v in (X, Y, Z))
    P1, P2, P3 = (np.ascontiguousarray(v, dtype=np.float64) for v in (P1, P2, P3))
    n = X.size
    s = np.empty((n, 6))
    e = np.empty((n, 6))
    L.TDstressFS_C(_dp(X), _dp(Y), _dp(Z), n, _dp(P1), _dp(P2), _dp(P3), float(Ss), float(Ds), float(Ts),
                   float(mu), float(lambda_), bool(halfspace), _dp(s), _dp(e))
    err = L.pq3d_last_error().decode()
    if err:
        raise _lib.PQ3DError(_lib.PQ3D_ERR_UNSUPPORTED, err)
    return s.T.copy(), e.T.copy()


def TDstressHS(X, Y, Z, P1, P2, P3, Ss, Ds, Ts, mu, lambda_):
    return TDstressFS(X, Y, Z, P1, P2, P3, Ss, Ds, Ts, mu, lambda_, halfspace=True)
