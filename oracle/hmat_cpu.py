"""CPU restatement of the reference's H-matrix build and product, for the CPU
baseline of bench.py -- test infrastructure, never the product path.

* Row and column generators as the reference calls them
  (src/Hmatrix.py:329-658): one receiver x many sources through
  TDstressEachSourceAtReceiver_C, one source x many receivers through
  TDstressFS_C (here the oracle's C restatement of src/TDstressFS_C.cpp),
  then the traction projection of src/Hmatrix.py:306-324 on the receiver
  frames of src/readmsh.py:75-134.
* ACA with partial pivoting on one combined block (3m traction rows x 2n
  slip columns; the same iteration and stopping rule as the GPU build, so the
  work per block is comparable; the reference runs ACA_plus_full_traceS/D,
  src/Hmatrix.py:661-1289, per slip direction with shared pivots).
* The product as the reference's blocks_process_MVM (src/Hmatrix.py:1773-1866):
  a Python loop over the blocks, per block a gather of x, U (V x) or D x, and a
  scatter-add into y.
"""
from __future__ import annotations

import numpy as np

from . import lib, tdstress, tdstress_each_source, _p, _L


def element_frames(nodes, tris):
    """(frames [N][9] = e1, e2, n; centroids [N][3]) by the oracle's C code."""
    nodes = np.ascontiguousarray(nodes, dtype=np.float64)
    tris = np.ascontiguousarray(tris, dtype=np.int64)
    N = tris.shape[0]
    frames = np.zeros((N, 9))
    xg = np.zeros((N, 3))
    lib().oracle_element_frames(_p(nodes), tris.ctypes.data_as(_L), N, _p(frames), _p(xg))
    return frames, xg


def _tractions(stress, frames):
    """(k, 6) stress (xx yy zz xy xz yz) on (k, 9) frames -> (k, 3) tractions (e1, e2, n)."""
    n = frames[:, 6:9]
    t0 = stress[:, 0] * n[:, 0] + stress[:, 3] * n[:, 1] + stress[:, 4] * n[:, 2]
    t1 = stress[:, 3] * n[:, 0] + stress[:, 1] * n[:, 1] + stress[:, 5] * n[:, 2]
    t2 = stress[:, 4] * n[:, 0] + stress[:, 5] * n[:, 1] + stress[:, 2] * n[:, 2]
    out = np.empty((stress.shape[0], 3))
    for c in range(3):
        e = frames[:, 3 * c:3 * c + 3]
        out[:, c] = e[:, 0] * t0 + e[:, 1] * t1 + e[:, 2] * t2
    return out


class BlockGen:
    """Rows and columns of one block (receivers ri, sources sj: element
    indices) through the reference's two generator calls."""

    def __init__(self, nodes, tris, frames, xg, ri, sj, mu, lam):
        self.mu, self.lam = mu, lam
        v = nodes[tris - 1]                      # (N, 3 vertices, 3)
        self.P1, self.P2, self.P3 = (np.ascontiguousarray(v[sj, k]) for k in range(3))
        self.frames_r = frames[ri]
        self.xr = xg[ri]
        self.ri, self.sj = ri, sj
        self.evals = 0

    def row(self, i):
        """Traction row 3p + c over the 2n slip columns (2q + s)."""
        p, c = divmod(i, 3)
        x, y, z = self.xr[p]
        out = np.empty(2 * len(self.sj))
        for s, (Ss, Ds) in enumerate(((1.0, 0.0), (0.0, 1.0))):
            st, _ = tdstress_each_source(x, y, z, self.P1, self.P2, self.P3, Ss, Ds, 0.0, self.mu, self.lam)
            out[s::2] = _tractions(st, np.broadcast_to(self.frames_r[p], (len(self.sj), 9)))[:, c]
        self.evals += 2 * len(self.sj)
        return out

    def col(self, j):
        """Slip column 2q + s over the 3m traction rows (3p + c)."""
        q, s = divmod(j, 2)
        Ss, Ds = (1.0, 0.0) if s == 0 else (0.0, 1.0)
        st, _ = tdstress(self.xr[:, 0], self.xr[:, 1], self.xr[:, 2], self.P1[q], self.P2[q], self.P3[q], Ss, Ds,
                         0.0, self.mu, self.lam)
        self.evals += len(self.ri)
        return _tractions(st, self.frames_r).reshape(-1)


def aca_block(gen: BlockGen, kmax: int, tol: float):
    """Partial-pivot ACA of the combined block: (rank, U [k][3m], V [k][2n])."""
    M, Nc = 3 * len(gen.ri), 2 * len(gen.sj)
    U, V = [], []
    used = np.zeros(M, dtype=bool)
    frob2, istar, k, guard = 0.0, 0, 0, 0
    while k < kmax and guard < M + kmax:
        guard += 1
        v = gen.row(istar)
        for l in range(k):
            v -= U[l][istar] * V[l]
        used[istar] = True
        jstar = int(np.argmax(np.abs(v)))
        if not np.abs(v[jstar]) > 0.0:
            nxt = np.nonzero(~used)[0]
            if len(nxt) == 0:
                break
            istar = int(nxt[0])
            continue
        u = gen.col(jstar)
        for l in range(k):
            u -= V[l][jstar] * U[l]
        u /= v[jstar]
        nu2, nv2 = float(u @ u), float(v @ v)
        cross = sum(float(u @ U[l]) * float(v @ V[l]) for l in range(k))
        frob2 += 2.0 * cross + nu2 * nv2
        U.append(u)
        V.append(v)
        k += 1
        if np.sqrt(nu2 * nv2) <= tol * np.sqrt(max(frob2, 0.0)):
            break
        au = np.abs(u)
        au[used] = -1.0
        if au.max() < 0.0:
            break
        istar = int(np.argmax(au))
    return k, U, V


def dense_block(gen: BlockGen):
    """(3m, 2n) block by the column generator."""
    return np.stack([gen.col(j) for j in range(2 * len(gen.sj))], axis=1)


def matvec(blocks, data, off, rank, x):
    """y = H x in the permuted (position) order: the reference's per-block
    loop.  blocks [nb][4] (r0, r1, c0, c1), data the block storage (dense
    3m x 2n column-major, or U 3m x k column-major then V k x 2n row-major),
    off / rank per block, x of length 2N (positions)."""
    y = np.zeros(3 * (len(x) // 2), dtype=data.dtype)
    for b in range(len(blocks)):
        r0, r1, c0, c1 = (int(v) for v in blocks[b])
        M, Nc = 3 * (r1 - r0), 2 * (c1 - c0)
        o, k = int(off[b]), int(rank[b])
        x_ = x[2 * c0:2 * c1]
        if k >= 0:
            U = data[o:o + M * k].reshape(k, M)
            Vt = data[o + M * k:o + M * k + k * Nc].reshape(k, Nc)
            y[3 * r0:3 * r1] += U.T @ (Vt @ x_)
        else:
            D = data[o:o + M * Nc].reshape(Nc, M)
            y[3 * r0:3 * r1] += D.T @ x_
    return y


__all__ = ["element_frames", "BlockGen", "aca_block", "dense_block", "matvec"]
