"""Receiver-row sharding of dense stepping across processes (one GPU each).

The reference steps one simulation on one device; its dense traction product
K.(V - Vpl) (src/QDsim_gpu.py:948-957) is the only term that couples cells.
Split the cells into contiguous ranges, one per rank: rank q holds rows
[3 c0, 3 c1) of the (3N) x (2N) operator (all source columns), the state of
its cells and v' of all cells.  One iteration is

  1. allgather of the v' slices        -> every rank has v' of all cells
  2. begin: product of the rank's rows, one Dormand-Prince attempt on its cells
  3. allreduce(MAX) of the runs' error norms (as FP64 bit patterns)
  4. end: accept/reject (the same on every rank: it reads only the reduced
     norms and the replicated control record) and the update of its cells

so the sharded run takes the steps of the unsharded one, and a cell's
arithmetic is that of the unsharded kernels (each operator row is reduced by
one warp in a fixed order): the results are bitwise those of one process.

Collectives go through an :class:`Exchange`: :class:`DistExchange` over
``torch.distributed`` (NCCL between GPUs, gloo on CPU), or
:class:`InProcessExchange` for several shards driven by one process (one GPU,
shards stepped in turn; no kernel waits on another).
"""
from __future__ import annotations

from typing import List, Sequence, Tuple

import torch


def receiver_partition(N: int, world: int) -> List[Tuple[int, int]]:
    """Contiguous cell ranges, one per rank; the first N % world ranks get one
    cell more."""
    if world < 1 or N < world:
        raise ValueError("need 1 <= world <= N (N=%d, world=%d)" % (N, world))
    base, extra = divmod(N, world)
    out, c = [], 0
    for q in range(world):
        n = base + (1 if q < extra else 0)
        out.append((c, c + n))
        c += n
    return out


class Exchange:
    """The two collectives of a sharded iteration over the shards this process
    drives.  A shard exposes ``cell0``, ``N`` (its cells), ``B``,
    ``vprime()`` (a writable (>= B, 2 N_total) view of v' of all cells),
    ``error_words()`` / ``set_error_words(w)`` ((B, 2) int64)."""

    def allgather_vprime(self, shards: Sequence) -> None:
        raise NotImplementedError

    def allreduce_max_errors(self, shards: Sequence) -> None:
        raise NotImplementedError


class InProcessExchange(Exchange):
    """All shards of the mesh live in this process."""

    def allgather_vprime(self, shards):
        for dst in shards:
            vd = dst.vprime()
            for src in shards:
                if src is dst:
                    continue
                a, b = 2 * src.cell0, 2 * (src.cell0 + src.N)
                vd[:src.B, a:b].copy_(src.vprime()[:src.B, a:b])

    def allreduce_max_errors(self, shards):
        w = shards[0].error_words()
        for s in shards[1:]:
            w = torch.maximum(w, s.error_words().to(w.device))
        for s in shards:
            s.set_error_words(w.to(s.error_words().device))


class DistExchange(Exchange):
    """One shard per process, collectives over ``torch.distributed`` (the
    process group must be initialised; NCCL needs device tensors, gloo CPU
    tensors -- the shard's own)."""

    def __init__(self, bounds: Sequence[Tuple[int, int]], group=None):
        import torch.distributed as dist
        self.dist = dist
        self.group = group
        self.bounds = list(bounds)
        self.nmax = max(b - a for a, b in self.bounds)

    def allgather_vprime(self, shards):
        (s,) = shards
        dist = self.dist
        v = s.vprime()
        B = s.B
        a, b = 2 * s.cell0, 2 * (s.cell0 + s.N)
        mine = torch.zeros((B, 2 * self.nmax), dtype=v.dtype, device=v.device)
        mine[:, :b - a] = v[:B, a:b]
        parts = [torch.empty_like(mine) for _ in self.bounds]
        dist.all_gather(parts, mine, group=self.group)
        for (c0, c1), p in zip(self.bounds, parts):
            if c0 == s.cell0:
                continue
            v[:B, 2 * c0:2 * c1] = p[:, :2 * (c1 - c0)]

    def allreduce_max_errors(self, shards):
        (s,) = shards
        w = s.error_words()
        self.dist.all_reduce(w, op=self.dist.ReduceOp.MAX, group=self.group)
        s.set_error_words(w)


def iterate_sharded(shards: Sequence, exchange: Exchange, n: int = 1) -> None:
    """n iterations of the sharded stepping (the call sites of the two
    collectives).  Every rank calls this with the same n."""
    for _ in range(n):
        exchange.allgather_vprime(shards)
        for s in shards:
            s.begin()
        exchange.allreduce_max_errors(shards)
        for s in shards:
            s.end()


def make_shards(K, tables, world, **ensemble_kw):
    """Row shards of one mesh for one process (the in-process group): K the
    full (3N, 2N) FP64 or FP32 operator, tables (B, N, 10).  Returns the
    :class:`~pyquake3d_gb300.ensemble.Ensemble` shards."""
    from .ensemble import Ensemble
    N = tables.shape[1]
    out = []
    for c0, c1 in receiver_partition(N, world):
        out.append(Ensemble(K[3 * c0:3 * c1].contiguous(), tables[:, c0:c1], shard=(c0, N), **ensemble_kw))
    return out
