"""Serving loop: earthquake-cycle simulation requests on pre-generated meshes,
continuously batched on one GPU.

* Requests arrive by a seeded Poisson process; each names a mesh, carries its
  own friction/stress draw (a per-cell table) and a simulated span.
* Every mesh keeps its traction operator resident (a dense packed operator
  for N <= dense_max_n -- the exact fixed-point BF16x18 product with the
  float-float Dormand-Prince attempt, or the faster BF16x6 product with the mixed
  attempt, ``dense_precision`` -- an H-matrix above) and an
  :class:`~pyquake3d_gb300.ensemble.Ensemble` with a fixed number of slots.
* Admission: a request enters a free slot of its mesh when the HBM budget
  (operators + the run state of occupied slots) allows; otherwise it waits
  (first come, first served per mesh).  Runs on the same mesh step together
  (one batched product per iteration), each with its own dt; a run retires
  when its simulated time reaches its span (or it fails), and its slot takes
  the next waiting request at the next round -- continuous batching.
* Each mesh replays a captured CUDA graph of a few iterations on its own
  stream, so the work of different meshes overlaps on the device.  The host
  reads only the small per-run control records between rounds.

A run's arithmetic does not depend on the other slots (the products keep a
fixed per-element order), so a request's result is the same alone and in the
mix (tests/test_serving_gpu.py).
"""
from __future__ import annotations

import dataclasses
import time
from typing import Dict, List, Optional

import numpy as np

YEAR = 365.0 * 24 * 3600


@dataclasses.dataclass
class Request:
    rid: int
    mesh: int
    arrival_s: float
    table: np.ndarray
    span_s: float
    slot: Optional[int] = None
    admitted_s: Optional[float] = None
    done_s: Optional[float] = None
    status: Optional[int] = None
    steps: int = 0
    attempts: int = 0
    sim_time: float = 0.0


def poisson_arrivals(n, rate_per_s, seed):
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate_per_s, size=n))


class Scheduler:
    """Slot and HBM-budget bookkeeping (host only).

    op_bytes[m]: resident operator bytes of mesh m; slot_bytes[m]: device bytes
    one occupied slot of mesh m adds; slots[m]: slots of mesh m."""

    def __init__(self, op_bytes: Dict[int, int], slot_bytes: Dict[int, int], slots: Dict[int, int], budget: float):
        self.op_bytes, self.slot_bytes, self.budget = dict(op_bytes), dict(slot_bytes), float(budget)
        self.free = {m: list(range(s)) for m, s in slots.items()}
        self.used = sum(op_bytes.values())
        if self.used > self.budget:
            raise MemoryError("operators alone exceed the HBM budget (%.1f GB > %.1f GB)" % (self.used / 1e9,
                                                                                          self.budget / 1e9))

    def try_admit(self, req: Request) -> Optional[int]:
        m = req.mesh
        if not self.free[m]:
            return None
        if self.used + self.slot_bytes[m] > self.budget:
            return None
        slot = self.free[m].pop(0)
        self.used += self.slot_bytes[m]
        return slot

    def release(self, mesh: int, slot: int):
        self.free[mesh].append(slot)
        self.free[mesh].sort()
        self.used -= self.slot_bytes[mesh]


def percentile(x, q):
    return float(np.percentile(np.asarray(x, dtype=np.float64), q)) if len(x) else float("nan")


class Server:
    """GPU runtime of the serving loop.

    meshes: list of dicts with keys nodes, tris, L (m), W (m); the operator
    kind follows N (dense for N <= dense_max_n, H-matrix above).
    dense_precision: "bf16x18" (fixed-point slices, float-float attempt: slip within
    1e-5 of the FP64 stepper for ~100 accepted steps at N = 10,000) or
    "bf16x6" (BF16 pieces, mixed attempt: ~25 steps, 4x the product rate)."""

    def __init__(self, meshes, *, mu, lam, cs, slots=16, budget_bytes=150e9, dense_max_n=20000, graph_iters=16,
                 max_steps=4000, device="cuda", hmat_kw=None, dense_precision="bf16x6"):
        import torch

        from . import gf
        from .ensemble import Ensemble, PackedFixOperator, PackedOperator
        from .hmatrix import HMatrix
        from .mesh import element_frames
        if dense_precision not in ("bf16x6", "bf16x18"):
            raise ValueError("dense_precision must be 'bf16x6' or 'bf16x18'")
        if dense_precision == "bf16x18" and slots > 64:
            raise ValueError("the bf16x18 product takes at most 64 slots")
        self.dense_precision = dense_precision
        self.torch = torch
        self.device = torch.device(device)
        self.meshes = meshes
        self.graph_iters = graph_iters
        self.max_steps = max_steps
        self.ens, self.streams, self.kind, self.build_s = {}, {}, {}, {}
        op_bytes, slot_bytes, nslots = {}, {}, {}
        hmat_kw = hmat_kw or dict(min_size=64, mini_leaf=64, eta=2.0, tol=1e-4)
        for m, spec in enumerate(meshes):
            nodes, tris = spec["nodes"], spec["tris"]
            N = tris.shape[0]
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            dummy = np.zeros((slots, N, 10))
            dummy[:, :, 1] = 0.01; dummy[:, :, 2] = 0.015; dummy[:, :, 3] = 0.1; dummy[:, :, 4] = 0.6
            dummy[:, :, 6] = 30.0; dummy[:, :, 7] = 1e-9
            if N <= dense_max_n:
                K64, _ = gf.assemble_dense(nodes, tris, mu, lam, fp32_copy=False, device=self.device)
                if dense_precision == "bf16x18":
                    op = PackedFixOperator(K64, element_frames(nodes, tris)[1])
                    del K64
                    torch.cuda.empty_cache()
                    ens = Ensemble(op, dummy, mu=mu, Cs=cs, precision="bf16x18", attempt="ff")
                else:
                    op = PackedOperator(K64)
                    del K64
                    torch.cuda.empty_cache()
                    ens = Ensemble(op, dummy, mu=mu, Cs=cs, precision="bf16x6")
                op_bytes[m] = op.data.numel() * op.data.element_size()
                self.kind[m] = "dense_" + dense_precision
            else:
                op = HMatrix(nodes, tris, mu, lam, device=self.device, **hmat_kw)
                ens = Ensemble(op, dummy, mu=mu, Cs=cs, precision="hmat")
                op_bytes[m] = op.stats["bytes"]
                self.kind[m] = "hmatrix"
            ens.set_ctrl(active=[0] * slots)
            ens.iterate(1)
            ens.capture(graph_iters)
            torch.cuda.synchronize()
            self.build_s[m] = time.perf_counter() - t0
            self.ens[m] = ens
            self.streams[m] = torch.cuda.Stream(self.device)
            slot_bytes[m] = ens.state_bytes() // slots
            nslots[m] = slots
        self.sched = Scheduler(op_bytes, slot_bytes, nslots, budget_bytes)
        self.op_bytes = op_bytes

    def run(self, requests: List[Request], time_limit_s=120.0):
        torch = self.torch
        pending = sorted(requests, key=lambda r: r.arrival_s)
        waiting: List[Request] = []
        running: Dict[int, Dict[int, Request]] = {m: {} for m in self.ens}
        done: List[Request] = []
        t0 = time.perf_counter()
        rounds = 0
        stages0 = {m: 0 for m in self.ens}
        while len(done) < len(requests):
            now = time.perf_counter() - t0
            if now > time_limit_s:
                break
            while pending and pending[0].arrival_s <= now:
                waiting.append(pending.pop(0))
            # admission (first come first served)
            still = []
            for req in waiting:
                slot = self.sched.try_admit(req)
                if slot is None:
                    still.append(req)
                    continue
                req.slot, req.admitted_s = slot, now
                ens = self.ens[req.mesh]
                with torch.cuda.stream(self.streams[req.mesh]):
                    ens.load_run(slot, req.table, t_end=req.span_s, max_steps=self.max_steps)
                running[req.mesh][slot] = req
            waiting = still
            busy = [m for m in self.ens if running[m]]
            if not busy:
                if pending:
                    time.sleep(max(0.0, min(0.05, pending[0].arrival_s - (time.perf_counter() - t0))))
                continue
            for m in busy:
                with torch.cuda.stream(self.streams[m]):
                    self.ens[m].replay(1)
            for m in busy:
                self.streams[m].synchronize()
            rounds += 1
            now = time.perf_counter() - t0
            for m in busy:
                ctrl = self.ens[m].read_ctrl()
                for slot, req in list(running[m].items()):
                    c = ctrl[slot]
                    if not c.active:
                        req.done_s, req.status = now, int(c.status)
                        req.steps, req.attempts, req.sim_time = int(c.steps), int(c.attempts), float(c.time)
                        self.sched.release(m, slot)
                        del running[m][slot]
                        done.append(req)
        wall = time.perf_counter() - t0
        ttr = [r.done_s - r.arrival_s for r in done]
        stages = 7 * sum(r.attempts for r in done)
        return {"requests": len(requests), "completed": len(done), "wall_s": wall, "rounds": rounds,
                "p50_time_to_result_s": percentile(ttr, 50), "p99_time_to_result_s": percentile(ttr, 99),
                "rk_stages": int(stages), "rk_stages_per_s": stages / wall if wall > 0 else float("nan"),
                "failed": int(sum(1 for r in done if r.status))}
