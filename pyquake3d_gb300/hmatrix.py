"""H-matrix of the traction operator on the GPU.

Partition (device, set-up; csrc/htree.cu): the reference's geometric rules
(src/Hmatrix.py:68-192, 2077-2142): binary cluster tree over the element
centroids by bisecting the longest bounding-box axis at its midpoint (points
<= midpoint go left, order kept, a leaf at <= min_size points or when a side
would be empty), built level by level; block tree by quad-splitting of (row,
column) cluster pairs, level by level, a leaf block when admissible
(min(diam) <= eta * dist, eta = 2) or when either side has <= mini_leaf points
or no children.  Low-rank blocks:
both sides > mini_leaf (src/Hmatrix.py:1292-1344); the rest are dense.
Elements are renumbered in depth-first leaf order, so every cluster is a
contiguous range and a block is a pair of ranges.

Compression and product (device, csrc/hmat.cu): ACA with partial pivoting on
the combined (3m x 2n) block (all six operators at once) with a relative
tolerance, FP32 factors, dense near field in FP32, and a deterministic product
for B right-hand sides.

Reference-shaped API: ``createHmatrix(xg, nodelst, elelst, eleVec, Para0,
mini_leaf)`` -> :class:`BlockTree` with ``calc_Hmatrix_ACA(dir,
save_corefunc)`` and ``blocks_process_MVM(x, blocks, type)``.
"""
from __future__ import annotations

import ctypes
import json
import os

import numpy as np
import torch

from . import _lib
from .mesh import element_frames



def build_partition(xg, min_size=16, mini_leaf=32, eta=2.0, device="cuda"):
    """The partition on the device (pq3d_hmat_partition, csrc/htree.cu):
    returns (perm, blocks, leaves) as host arrays -- perm[p] = element at
    position p; blocks = int64 (nb, 5): r0, r1, c0, c1, lowrank (0/1) in
    depth-first order; leaves = int64 (nl, 2) leaf cluster ranges -- and
    records the device time and tree depth in ``build_partition.last``."""
    import time
    L = _lib.load()
    dev = torch.device(device)
    xg_t = torch.as_tensor(np.ascontiguousarray(xg, dtype=np.float64), device=dev).contiguous()
    N = xg_t.shape[0]
    perm = torch.empty(N, dtype=torch.int64, device=dev)
    leaves = torch.empty((N, 2), dtype=torch.int64, device=dev)
    nl, nb, depth = ctypes.c_int64(0), ctypes.c_int64(0), ctypes.c_int32(0)
    cap = max(1024, 4 * N)
    st = torch.cuda.current_stream(dev)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    while True:
        blocks = torch.empty((cap, 5), dtype=torch.int64, device=dev)
        rc = L.pq3d_hmat_partition(xg_t.data_ptr(), N, int(min_size), int(mini_leaf), float(eta), perm.data_ptr(),
                                   leaves.data_ptr(), ctypes.byref(nl), blocks.data_ptr(), cap, ctypes.byref(nb),
                                   ctypes.byref(depth), st.cuda_stream)
        if rc == _lib.PQ3D_ERR_ARG and nb.value > cap:
            cap = int(nb.value)
            continue
        _lib.check(rc)
        break
    build_partition.last = {"seconds": time.perf_counter() - t0, "depth": int(depth.value),
                            "blocks": int(nb.value), "leaves": int(nl.value)}
    return (perm.cpu().numpy(), blocks[:nb.value].cpu().numpy(), leaves[:nl.value].cpu().numpy())


build_partition.last = {}


def cluster_order(xg, min_size=1, device="cuda") -> torch.Tensor:
    """Depth-first leaf order of the bisection cluster tree on the device
    (pq3d_hmat_cluster_order): order[p] = element at position p, a spatially
    compact order (every run of consecutive positions lies in a small region
    of the fault).  Device int64 tensor."""
    L = _lib.load()
    dev = torch.device(device)
    xg_t = torch.as_tensor(np.ascontiguousarray(xg, dtype=np.float64), device=dev).contiguous()
    order = torch.empty(xg_t.shape[0], dtype=torch.int64, device=dev)
    _lib.check(L.pq3d_hmat_cluster_order(xg_t.data_ptr(), xg_t.shape[0], int(min_size), order.data_ptr(), None,
                                         torch.cuda.current_stream(dev).cuda_stream))
    return order


class HMatrix:
    """Device H-matrix of the (3N)x(2N) traction operator of a mesh."""

    def __init__(self, nodes, tris, mu, lam, *, min_size=16, mini_leaf=32, eta=2.0, tol=1e-4, kmax=128,
                 device="cuda", chunk_bytes=8 << 30, halfspace=False):
        L = _lib.load()
        self.device = torch.device(device)
        dev = self.device
        nodes = np.ascontiguousarray(nodes, dtype=np.float64)
        tris = np.ascontiguousarray(tris, dtype=np.int64)
        N = tris.shape[0]
        self.N = N
        import time as _time
        phases = {}
        tp = [_time.perf_counter()]

        def phase(name):   # wall time of the phase just finished (device synchronised)
            torch.cuda.synchronize(dev)
            t = _time.perf_counter()
            phases[name] = t - tp[0]
            tp[0] = t

        _, xg = element_frames(nodes, tris)
        phase("frames_host")
        perm, blocks, leaves = build_partition(xg, min_size, mini_leaf, eta, device=dev)
        self.partition_info = dict(build_partition.last)
        phase("partition_device")
        self.perm_host, self.blocks_host, self.leaves_host = perm, blocks, leaves
        st = torch.cuda.current_stream(dev).cuda_stream
        self.nodes_t = torch.as_tensor(nodes, device=dev)
        self.tris_t = torch.as_tensor(tris, device=dev)
        self.tables = torch.empty(L.pq3d_gf_workspace_bytes(N), dtype=torch.uint8, device=dev)
        hs = int(bool(halfspace))
        self.halfspace = bool(halfspace)
        _lib.check(L.pq3d_gf_setup(self.nodes_t.data_ptr(), self.tris_t.data_ptr(), N, hs, self.tables.data_ptr(),
                                   self.tables.numel(), st))
        phase("gf_tables")
        self.perm = torch.as_tensor(perm, device=dev)
        nb = blocks.shape[0]
        blk = np.ascontiguousarray(blocks[:, :4])
        self.blk = torch.as_tensor(blk, device=dev)
        m = blocks[:, 1] - blocks[:, 0]
        n = blocks[:, 3] - blocks[:, 2]
        lowrank = blocks[:, 4].astype(bool)
        kcap = np.minimum(kmax, np.minimum(3 * m, 2 * n)).astype(np.int32)
        kcap[~lowrank] = 0
        self.kcap = torch.as_tensor(kcap, device=dev)
        rank = np.full(nb, -1, dtype=np.int32)
        status = np.zeros(nb, dtype=np.int32)
        lr = np.nonzero(lowrank)[0]
        # ACA in chunks of blocks (at most chunk_bytes of FP64 factors each).
        # One FP64 scratch, sized for the largest chunk, serves every chunk:
        # each chunk's converged factors are packed to FP32 right after its
        # ACA, so the FP64 factors of all blocks never coexist (N = 100,000:
        # 22 GB of FP64 factors, 3 GB packed).
        uv_need = kcap.astype(np.int64) * (3 * m + 2 * n)
        bounds = []
        i = 0
        while i < len(lr):
            j = i
            tot = 0
            while j < len(lr) and (j == i or tot + uv_need[lr[j]] * 8 <= chunk_bytes):
                tot += uv_need[lr[j]] * 8
                j += 1
            bounds.append((i, j))
            i = j
        self.aca_chunks = len(bounds)
        # wall-clock split of the ACA phase (each part device-synchronised):
        # scratch allocation, per-chunk set-up (allocations, uploads), the
        # launch up to its results on the host, the FP32 packing
        aca_split = {"scratch_alloc": 0.0, "chunk_setup": 0.0, "launch_to_host": 0.0, "pack": 0.0}

        def lap(key, t0):
            torch.cuda.synchronize(dev)
            t = _time.perf_counter()
            aca_split[key] += t - t0
            return t

        t_l = _time.perf_counter()
        UV = torch.empty(max([int(uv_need[lr[i:j]].sum()) for i, j in bounds] + [1]), dtype=torch.float64,
                         device=dev)
        t_l = lap("scratch_alloc", t_l)
        lr_parts = []     # per chunk: block ids, FP32 offsets inside the chunk, packed factors
        aca_events = []   # (start, end) CUDA events around each ACA launch
        for (i, j) in bounds:
            ids = lr[i:j]
            uv_off = np.concatenate([[0], np.cumsum(uv_need[ids])[:-1]]).astype(np.int64)
            used_off = np.concatenate([[0], np.cumsum(3 * m[ids])[:-1]]).astype(np.int64)
            used = torch.zeros(int((3 * m[ids]).sum()), dtype=torch.uint8, device=dev)
            # the kernel indexes blocks by grid position: pass the chunk's
            # sub-arrays, gathered on the host (no device indexing kernel)
            blk_c = torch.as_tensor(np.ascontiguousarray(blk[ids]), device=dev)
            kcap_c = torch.as_tensor(np.ascontiguousarray(kcap[ids]), device=dev)
            uvo_c = torch.as_tensor(uv_off, device=dev)
            uso_c = torch.as_tensor(used_off, device=dev)
            rk_c = torch.empty(len(ids), dtype=torch.int32, device=dev)
            stt_c = torch.empty(len(ids), dtype=torch.int32, device=dev)
            t_l = lap("chunk_setup", t_l)
            ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            ev[0].record()
            _lib.check(L.pq3d_hmat_aca(self.tables.data_ptr(), N, self.perm.data_ptr(), len(ids), blk_c.data_ptr(),
                                       kcap_c.data_ptr(), float(tol), float(mu), float(lam), hs, UV.data_ptr(),
                                       uvo_c.data_ptr(), used.data_ptr(), uso_c.data_ptr(), rk_c.data_ptr(),
                                       stt_c.data_ptr(), st))
            ev[1].record()
            aca_events.append(ev)
            st_h = stt_c.cpu().numpy()
            rk_h = np.where(st_h == 0, rk_c.cpu().numpy(), -1).astype(np.int32)   # not converged: dense
            t_l = lap("launch_to_host", t_l)
            rank[ids] = rk_h
            status[ids] = st_h
            # packed FP32 factors k (3m + 2n), each block padded to a multiple
            # of 4 floats (16-byte aligned starts), zero padding
            sz = np.maximum(rk_h, 0).astype(np.int64) * (3 * m[ids] + 2 * n[ids])
            sz = (sz + 3) // 4 * 4
            loc = np.concatenate([[0], np.cumsum(sz)[:-1]]).astype(np.int64)
            buf = torch.zeros(max(int(sz.sum()), 4), dtype=torch.float32, device=dev)
            good = np.nonzero(rk_h >= 0)[0].astype(np.int32)   # positions inside the chunk
            if len(good):
                pos = torch.as_tensor(good, device=dev)
                loc_t = torch.as_tensor(loc, device=dev)
                _lib.check(L.pq3d_hmat_pack_factors(UV.data_ptr(), uvo_c.data_ptr(), blk_c.data_ptr(),
                                                    kcap_c.data_ptr(), rk_c.data_ptr(), pos.data_ptr(), len(good),
                                                    buf.data_ptr(), loc_t.data_ptr(), st))
            lr_parts.append((ids, rk_h, loc, int(sz.sum()), buf))
            t_l = lap("pack", t_l)
        del UV
        phase("aca")
        phases["aca_split"] = aca_split
        # device time of the ACA launches alone (the rest of the phase is the
        # FP32 packing of each chunk, the small allocations and the rank and
        # status copies back)
        phases["aca_kernels"] = sum(a.elapsed_time(b) for a, b in aca_events) / 1e3
        self.aca_status = status
        # storage: the converged low-rank blocks first, in block order (U
        # column-major 3m x k, then V k x 2n), then the dense blocks in block
        # order (3m x 2n column-major); every block padded to a multiple of 4
        # floats so that each starts 16-byte aligned
        off = np.zeros(nb, dtype=np.int64)
        base = 0
        for (ids, rk_h, loc, used_f, _) in lr_parts:
            ok = rk_h >= 0
            off[ids[ok]] = base + loc[ok]
            base += used_f
        dense_ids = np.nonzero(rank < 0)[0].astype(np.int32)
        dsz = (6 * m[dense_ids].astype(np.int64) * n[dense_ids] + 3) // 4 * 4
        off[dense_ids] = base + np.concatenate([[0], np.cumsum(dsz)[:-1]]).astype(np.int64)
        total = base + int(dsz.sum())
        assert np.all(off % 4 == 0)
        self.data = torch.zeros(max(total, 4), dtype=torch.float32, device=dev)   # padding defined
        self.off = torch.as_tensor(off, device=dev)
        self.rank = torch.as_tensor(rank, device=dev)
        phase("storage_alloc")
        if len(dense_ids):
            ids_t = torch.as_tensor(dense_ids, device=dev)
            _lib.check(L.pq3d_hmat_dense_blocks(self.tables.data_ptr(), N, self.perm.data_ptr(), self.blk.data_ptr(),
                                                ids_t.data_ptr(), len(dense_ids), float(mu), float(lam), hs,
                                                self.data.data_ptr(), self.off.data_ptr(), st))
        phase("dense_blocks")
        base = 0
        for (_, _, _, used_f, buf) in lr_parts:
            if used_f:
                self.data[base:base + used_f].copy_(buf[:used_f])
            base += used_f
        del lr_parts
        phase("place_factors")
        # low-rank bookkeeping and leaf lists
        lr_ids = np.nonzero(rank >= 0)[0].astype(np.int32)
        ranks = rank[lr_ids].astype(np.int64)
        prefix = np.concatenate([[0], np.cumsum(ranks)]).astype(np.int64)
        t_off = np.zeros(nb, dtype=np.int64)
        t_off[lr_ids] = prefix[:-1]
        self.t_rows = int(prefix[-1])
        self.lr_ids = torch.as_tensor(lr_ids if len(lr_ids) else np.zeros(1, np.int32), device=dev)
        self.t_off = torch.as_tensor(t_off, device=dev)
        # per rank row: offset of its V row, and (2 c0) | (2n) << 32
        if len(lr_ids):
            bl = np.repeat(lr_ids, ranks)
            l = np.arange(self.t_rows, dtype=np.int64) - np.repeat(prefix[:-1], ranks)
            Mb, Nb = 3 * m[bl].astype(np.int64), 2 * n[bl].astype(np.int64)
            info = np.empty((self.t_rows, 2), dtype=np.int64)
            info[:, 0] = off[bl] + Mb * rank[bl].astype(np.int64) + l * Nb
            info[:, 1] = 2 * blocks[bl, 2].astype(np.int64) | (Nb << 32)
        else:
            info = np.zeros((1, 2), dtype=np.int64)
        self.t_info = torch.as_tensor(info, device=dev)
        self._make_sched(info)
        # per leaf row cluster, the blocks whose row range covers it, in block order
        nl = leaves.shape[0]
        leaf_start = leaves[:, 0]
        a = np.searchsorted(leaf_start, blocks[:, 0], side="left")
        z = np.searchsorted(leaf_start, blocks[:, 1], side="left")
        cnt = z - a
        bl = np.repeat(np.arange(nb, dtype=np.int64), cnt)
        q = np.repeat(a, cnt) + (np.arange(int(cnt.sum()), dtype=np.int64) - np.repeat(np.cumsum(cnt) - cnt, cnt))
        srt = np.argsort(q, kind="stable")
        leaf_ptr = np.concatenate([[0], np.cumsum(np.bincount(q, minlength=nl))]).astype(np.int64)
        self.leaf = torch.as_tensor(np.ascontiguousarray(leaves), device=dev)
        self.leaf_ptr = torch.as_tensor(leaf_ptr, device=dev)
        self.leaf_blocks = torch.as_tensor(bl[srt].astype(np.int32), device=dev)
        phase("host_lists")
        self._make_struct()
        self.stats = {"N": N, "blocks": int(nb), "lowrank_blocks": int(len(lr_ids)),
                      "dense_blocks": int(len(dense_ids)), "aca_not_converged": int(np.sum(lowrank & (status != 0))),
                      "max_rank": int(ranks.max()) if len(ranks) else 0,
                      "mean_rank": float(ranks.mean()) if len(ranks) else 0.0,
                      "bytes": int(self.data.numel() * 4), "dense_fp32_bytes": int(6 * N * N * 4),
                      "leaves": int(nl)}
        self.build_phases = phases

    _ARRAYS = ("perm", "blk", "rank", "off", "data", "lr_ids", "t_info", "t_off", "leaf", "leaf_ptr", "leaf_blocks")

    LONG_ROW = 8192   # columns above which a rank row gets a whole CTA in the product

    T_GROUP = 4       # short rank rows of one block handled together (they share the x values)

    def _make_sched(self, info):
        info = np.asarray(info, dtype=np.int64).reshape(-1, 2)
        Nc = (info[:, 1] >> 32) if self.t_rows else np.zeros(0, np.int64)
        rows = np.arange(len(Nc), dtype=np.int32)
        longm = Nc > self.LONG_ROW
        sched = np.concatenate([rows[~longm], rows[longm]]) if len(Nc) else np.zeros(1, np.int32)
        self.t_sched = torch.as_tensor(np.ascontiguousarray(sched, dtype=np.int32), device=self.device)
        self.t_nlong = int(longm.sum())
        # groups of up to T_GROUP consecutive short rows of one low-rank block
        # (all rows of a block have the same length), in block order; one
        # 16-byte record each: V offset of the first row | row length << 40 |
        # size << 56, then first column | first row << 32
        rec = np.zeros((0, 2), dtype=np.int64)
        if self.t_rows:
            ranks = self.rank.cpu().numpy()[self.lr_ids.cpu().numpy()].astype(np.int64)
            first = np.concatenate([[0], np.cumsum(ranks)[:-1]]).astype(np.int64)
            keep = ranks > 0
            keep[keep] = ~longm[first[keep]]
            k, f = ranks[keep], first[keep]
            ng = (k + self.T_GROUP - 1) // self.T_GROUP
            j = np.arange(int(ng.sum()), dtype=np.int64) - np.repeat(np.cumsum(ng) - ng, ng)
            w0 = np.repeat(f, ng) + self.T_GROUP * j
            size = np.minimum(self.T_GROUP, np.repeat(k, ng) - self.T_GROUP * j)
            off, col, nc = info[w0, 0], info[w0, 1] & 0xffffffff, info[w0, 1] >> 32
            assert np.all(off < 2 ** 40) and np.all(nc <= self.LONG_ROW) and self.t_rows < 2 ** 31
            rec = np.stack([off | (nc << 40) | (size << 56), col | (w0 << 32)], axis=1)
        self.t_grp = torch.as_tensor(rec if len(rec) else np.zeros((1, 2), np.int64), device=self.device)
        self.t_ngrp = len(rec)

    def _make_struct(self):
        H = _lib.HMat()
        H.N, H.nblocks, H.nleaves, H.t_rows = self.N, int(self.blk.shape[0]), int(self.leaf.shape[0]), self.t_rows
        for k in self._ARRAYS:
            setattr(H, k, getattr(self, k).data_ptr())
        H.t_sched, H.t_nlong = self.t_sched.data_ptr(), self.t_nlong
        H.t_grp, H.t_ngrp = self.t_grp.data_ptr(), self.t_ngrp
        self.H = H

    def save(self, path):
        """Write the compressed operator (the device arrays, one .npz): the
        warm-start cache of a mesh, in place of the reference's pickled block
        list (src/Hmatrix.py:1552-1555)."""
        arrs = {k: getattr(self, k).cpu().numpy() for k in self._ARRAYS}
        np.savez(path, N=self.N, t_rows=self.t_rows, stats=json.dumps(self.stats), halfspace=self.halfspace, **arrs)

    @classmethod
    def load(cls, path, device="cuda"):
        """An H-matrix written by :meth:`save` (no ACA, no GF evaluation)."""
        g = np.load(path)
        self = cls.__new__(cls)
        self.device = torch.device(device)
        self.N = int(g["N"])
        self.t_rows = int(g["t_rows"])
        self.stats = json.loads(str(g["stats"]))
        self.halfspace = bool(g["halfspace"]) if "halfspace" in g else False
        for k in cls._ARRAYS:
            setattr(self, k, torch.as_tensor(g[k], device=self.device))
        self._make_sched(g["t_info"])
        self._make_struct()
        return self

    def workspace_bytes(self, B):
        return _lib.load().pq3d_hmat_workspace_bytes(ctypes.byref(self.H), int(B))

    def apply(self, X, out=None, workspace=None, active=None):
        """Y = H X for X of shape (B, 2N) (FP64, element order, interleaved
        strike/dip); returns Y (B, 3N).  ``active``: optional int32 device
        tensor of B flags; runs with flag 0 are skipped (their rows of ``out``
        are left as they are)."""
        L = _lib.load()
        X = X.contiguous()
        B = X.shape[0]
        Y = out if out is not None else torch.empty((B, 3 * self.N), dtype=torch.float64, device=self.device)
        ws = workspace if workspace is not None else torch.empty(self.workspace_bytes(B), dtype=torch.uint8,
                                                                 device=self.device)
        st = torch.cuda.current_stream(self.device).cuda_stream
        if active is None:
            _lib.check(L.pq3d_hmat_apply(ctypes.byref(self.H), X.data_ptr(), B, Y.data_ptr(), ws.data_ptr(),
                                         ws.numel(), st))
        else:
            assert active.dtype == torch.int32 and active.numel() == B
            _lib.check(L.pq3d_hmat_apply_masked(ctypes.byref(self.H), X.data_ptr(), B, Y.data_ptr(),
                                                active.data_ptr(), 1, ws.data_ptr(), ws.numel(), st))
        return Y

    def matvec(self, v):
        return self.apply(v.reshape(1, -1))[0]


OP_INDEX = {"A1s": (0, 0), "A2s": (1, 0), "Bs": (2, 0), "A1d": (0, 1), "A2d": (1, 1), "Bd": (2, 1)}


class BlockTree:
    """Reference-shaped wrapper (src/Hmatrix.py:277): the partition is built
    by createHmatrix, calc_Hmatrix_ACA compresses on the GPU,
    blocks_process_MVM applies one of the six operators."""

    def __init__(self, nodelst, elelst, mu, lam, halfspace, mini_leaf, eta=2.0, tol=1e-4, device="cuda"):
        self.halfspace = bool(halfspace)
        self.nodelst, self.elelst = nodelst, elelst
        self.mu_, self.lambda_, self.mini_leaf, self.eta, self.tol, self.device = mu, lam, mini_leaf, eta, tol, device
        _, xg = element_frames(np.asarray(nodelst, dtype=np.float64), np.asarray(elelst, dtype=np.int64))
        self.perm, self.blocks, self.leaves = build_partition(xg, 16, mini_leaf, eta, device=device)
        self.H = None
        self.blocks_to_process = [tuple(b) for b in self.blocks]

    def calc_Hmatrix_ACA(self, dir=None, save_corefunc=False):
        """Compress on the GPU; with ``dir``, reuse ``dir/hmatrix.npz`` when it
        exists and write it when ``save_corefunc`` (the reference's cache
        switch, src/Hmatrix.py:1552-1555)."""
        cache = os.path.join(dir, "hmatrix.npz") if dir else None
        if cache and os.path.exists(cache):
            self.H = HMatrix.load(cache, device=self.device)
        else:
            self.H = HMatrix(self.nodelst, self.elelst, self.mu_, self.lambda_, min_size=16,
                             mini_leaf=self.mini_leaf, eta=self.eta, tol=self.tol, device=self.device,
                             halfspace=self.halfspace)
            if cache and save_corefunc:
                os.makedirs(dir, exist_ok=True)
                self.H.save(cache)
        return self.blocks_to_process

    def blocks_process_MVM(self, xvector, blocks_to_process=None, type="A1s"):
        """y = op(type) x on all blocks (one GPU holds every block; the
        blocks argument is accepted for call compatibility)."""
        if self.H is None:
            self.calc_Hmatrix_ACA()
        c, s = OP_INDEX[type]
        N = self.H.N
        X = torch.zeros((1, 2 * N), dtype=torch.float64, device=self.H.device)
        X[0, s::2] = torch.as_tensor(np.asarray(xvector, dtype=np.float64), device=self.H.device)
        return self.H.apply(X)[0, c::3].cpu().numpy()


def createHmatrix(xg, nodelst, elelst, eleVec, Para0, mini_leaf=32):
    """src/Hmatrix.py:2147-2196: build the block tree (compression happens in
    calc_Hmatrix_ACA).  Para0 keys: 'Shear modulus', 'Lame constants',
    'Half space' (values or strings)."""
    mu = float(Para0["Shear modulus"])
    lam = float(Para0["Lame constants"])
    half = Para0.get("Half space", False)
    half = half if isinstance(half, bool) else str(half) == "True"
    return BlockTree(nodelst, elelst, mu, lam, half, mini_leaf)
