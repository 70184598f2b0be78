"""Autotuner of the launch shape of the tensor-core traction products.

``pq3d_batch_gemm_bf16x6`` streams the packed operator through one CTA per
(128-row tile, K slice).  Two launch parameters are free:

* ``nsplit``, the K slices: the grid is ceil(3N/128) x nsplit CTAs.  More
  slices fill more of the SMs' CTA slots and make the last wave finer, but
  write more FP32 partial sums, which the attempt kernel reads back.  nsplit
  fixes the order in which the slices' sums are added, so it is tuned per
  device and mesh size at one fixed width (``TUNE_RUNS`` runs) and cached:
  every ensemble of a mesh then uses the same value whatever its run count,
  and a run's bits do not depend on the batch it is in.
* ``ctas_per_sm``, the CTAs resident per SM (1-3; the library launches fewer
  where shared or tensor memory does not fit them, and each CTA's pipeline
  depth follows from the count).  It does not change the result, so it is
  tuned per mesh size and padded run count.

Every candidate is timed with CUDA events on the current stream (one warm-up
launch, then the best of ``REPEATS`` repeats of ``INNER`` back-to-back
launches) on the ensemble's own packed operator and a seeded right-hand side.
The fastest candidate wins; one within ``TIE`` of it that comes earlier in
candidate order (fewer slices; for the CTA count the order 2, 1, 3) is
preferred, so timing noise rarely flips the choice.  Results live in a
per-process cache; with ``PQ3D_TUNE_CACHE=<file.json>`` they are also read
from and written to that file, which makes the choice, and with it the bits
that depend on nsplit, the same across processes.
"""
from __future__ import annotations

import json
import os

import numpy as np
import torch

from . import _lib

TUNE_RUNS = 64        # width at which nsplit is tuned
MAX_NSPLIT = 16
MAX_NSPLIT_FIX = 24
CTAS_ORDER = (2, 1, 3)
TIE = 0.02
INNER = 2
REPEATS = 3
ENV_CACHE = "PQ3D_TUNE_CACHE"

_cache: dict = {}
_cache_file_loaded: str | None = None


def padded_runs(B: int) -> int:
    return (B + 15) // 16 * 16


def nsplit_candidates(N: int, max_nsplit: int = MAX_NSPLIT) -> list[int]:
    """1 .. min(max_nsplit, number of 32-column blocks of the 2N columns)."""
    return list(range(1, min(max_nsplit, (2 * N + 31) // 32) + 1))


def pick(times: dict, order: list, tie: float = TIE):
    """The candidate with the smallest time, or the first in ``order`` whose
    time is within ``tie`` (relative) of that smallest time."""
    best = min(times[c] for c in order)
    for c in order:
        if times[c] <= best * (1.0 + tie):
            return c
    raise ValueError("no candidate")


def tune(order: list, time_fn, tie: float = TIE):
    """Time every candidate with ``time_fn(candidate) -> seconds`` and pick
    one; returns (choice, {candidate: seconds})."""
    times = {c: float(time_fn(c)) for c in order}
    return pick(times, order, tie), times


def _key(device, *parts) -> str:
    name = torch.cuda.get_device_name(device).replace(" ", "_") if device is not None else "cpu"
    return "|".join([name] + [str(p) for p in parts])


def _cache_path():
    return os.environ.get(ENV_CACHE) or None


def _load_file():
    global _cache_file_loaded
    path = _cache_path()
    if path is None or path == _cache_file_loaded:
        return
    _cache_file_loaded = path
    try:
        with open(path) as f:
            data = json.load(f)
    except (OSError, ValueError):
        return
    for k, v in data.items():
        if isinstance(v, int):
            _cache.setdefault(k, v)


def _save_file():
    path = _cache_path()
    if path is None:
        return
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(_cache, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def lookup(key: str):
    _load_file()
    return _cache.get(key)


def store(key: str, value: int):
    _cache[key] = int(value)
    _save_file()


def clear():
    """Forget the per-process cache (the file, if any, is left as it is)."""
    global _cache_file_loaded
    _cache.clear()
    _cache_file_loaded = None


class _Bench:
    """Scratch buffers and the timed launch of one (operator, run count)."""

    def __init__(self, op, B: int, max_nsplit: int):
        L = _lib.load()
        self.L, self.op, self.B, self.N = L, op, B, op.N
        dev = op.device
        g = torch.Generator(device="cpu").manual_seed(1234)
        nb = L.pq3d_batch_rhs_bytes(self.N, B)
        v = torch.randn(nb // 2, generator=g).to(torch.bfloat16)
        self.vop = v.view(torch.uint8).to(dev)
        self.out = torch.empty(max_nsplit * padded_runs(B) * 3 * self.N, dtype=torch.float32, device=dev)
        self.ws = torch.zeros(256, dtype=torch.uint8, device=dev)
        self.stream = torch.cuda.current_stream(dev)
        self.err = 0

    def launch(self, nsplit: int, ctas: int):
        _lib.check(self.L.pq3d_batch_gemm_bf16x6(self.op.data.data_ptr(), self.vop.data_ptr(), self.N, self.B,
                                                 nsplit, ctas, self.out.data_ptr(), self.ws.data_ptr(),
                                                 self.ws.numel(), self.stream.cuda_stream))

    def time(self, nsplit: int, ctas: int) -> float:
        self.launch(nsplit, ctas)
        best = float("inf")
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for _ in range(REPEATS):
            s.record(self.stream)
            for _ in range(INNER):
                self.launch(nsplit, ctas)
            e.record(self.stream)
            e.synchronize()
            best = min(best, s.elapsed_time(e) / 1e3 / INNER)
        w = self.ws[:4].view(torch.int32).item()
        if w != 0:
            raise RuntimeError(f"tensor-core product reported error word {w} while tuning")
        return best


def ctas_candidates(B: int) -> list[int]:
    """Requested CTA counts in preference order, one per distinct launch
    (a request the library cannot fit launches like a smaller one)."""
    L = _lib.load()
    plan = np.zeros(2, dtype=np.int32)
    seen, out = set(), []
    for c in CTAS_ORDER:
        _lib.check(L.pq3d_batch_gemm_bf16x6_plan(B, c, plan.ctypes.data))
        p = (int(plan[0]), int(plan[1]))
        if p not in seen:
            seen.add(p)
            out.append(c)
    return out


def tune_bf16x6(op, B: int) -> dict:
    """Launch shape of the tensor-core product of B runs on the packed
    operator ``op``: {"nsplit", "ctas_per_sm", "tuned"} (tuned = False when
    both came from the cache)."""
    N, dev = op.N, op.device
    k_ns = _key(dev, f"N={N}", "nsplit")
    Bp = padded_runs(B)
    k_ct = _key(dev, f"N={N}", f"Bp={Bp}", "ctas")
    nsplit, ctas = lookup(k_ns), lookup(k_ct)
    tuned = False
    if nsplit is None:
        bench = _Bench(op, TUNE_RUNS, MAX_NSPLIT)
        order = [(ns, c) for ns in nsplit_candidates(N) for c in ctas_candidates(TUNE_RUNS)]
        (nsplit, c64), _ = tune(order, lambda nc: bench.time(*nc))
        store(k_ns, nsplit)
        store(_key(dev, f"N={N}", f"Bp={padded_runs(TUNE_RUNS)}", "ctas"), c64)
        ctas = lookup(k_ct)
        tuned = True
        del bench
    if ctas is None:
        cands = ctas_candidates(B)
        if len(cands) == 1:
            ctas = cands[0]
        else:
            bench = _Bench(op, B, nsplit)
            ctas, _ = tune(cands, lambda c: bench.time(nsplit, c))
            del bench
        store(k_ct, ctas)
        tuned = True
    return {"nsplit": int(nsplit), "ctas_per_sm": int(ctas), "tuned": tuned}


class _BenchFix:
    """Scratch buffers and the timed launch of the fixed-point product."""

    def __init__(self, op, B: int, max_nsplit: int):
        L = _lib.load()
        self.L, self.op, self.B, self.N = L, op, B, op.N
        dev = op.device
        g = torch.Generator(device="cpu").manual_seed(1234)
        v = torch.randn(B, 2 * self.N, generator=g, dtype=torch.float64).to(dev)
        self.vop = torch.zeros(L.pq3d_batch_rhs_fix_bytes(self.N, B), dtype=torch.uint8, device=dev)
        self.stream = torch.cuda.current_stream(dev)
        _lib.check(L.pq3d_batch_pack_rhs_fix(v.data_ptr(), self.N, B, None, self.vop.data_ptr(),
                                             self.stream.cuda_stream))
        self.out = torch.empty(max_nsplit * padded_runs(B) * 3 * self.N * 2, dtype=torch.float32, device=dev)
        self.ws = torch.zeros(256, dtype=torch.uint8, device=dev)

    def launch(self, nsplit: int):
        _lib.check(self.L.pq3d_batch_gemm_bf16x18(self.op.data.data_ptr(), self.vop.data_ptr(), self.N, self.B,
                                                  nsplit, self.out.data_ptr(), self.ws.data_ptr(), self.ws.numel(),
                                                  self.stream.cuda_stream))

    def time(self, nsplit: int) -> float:
        self.launch(nsplit)
        best = float("inf")
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for _ in range(REPEATS):
            s.record(self.stream)
            for _ in range(INNER):
                self.launch(nsplit)
            e.record(self.stream)
            e.synchronize()
            best = min(best, s.elapsed_time(e) / 1e3 / INNER)
        w = self.ws[:4].view(torch.int32).item()
        if w != 0:
            raise RuntimeError(f"fixed-point tensor-core product reported error word {w} while tuning")
        return best


def tune_bf16x18(op, B: int) -> dict:
    """K slices of the fixed-point product on the packed operator ``op``:
    {"nsplit", "tuned"}, tuned at TUNE_RUNS runs and cached per mesh size."""
    N, dev = op.N, op.device
    key = _key(dev, f"N={N}", "nsplit_fix")
    nsplit = lookup(key)
    if nsplit is not None:
        return {"nsplit": int(nsplit), "tuned": False}
    bench = _BenchFix(op, TUNE_RUNS, MAX_NSPLIT_FIX)
    nsplit, _ = tune(nsplit_candidates(N, MAX_NSPLIT_FIX), bench.time)
    del bench
    store(key, nsplit)
    return {"nsplit": int(nsplit), "tuned": True}
