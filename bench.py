#!/usr/bin/env python
"""Benchmark of the GB300 quasi-dynamic cycle hot path.

Workload (N=1 line): Green's-function assembly, mid size -- a rough
strike-slip fault 80 km x 30 km (self-affine height field, Hurst 0.8,
rms/length 1e-3, seed 0), 200 x 50 rectangles -> N = 20,000 triangles.  One
step = one full dense assembly of the (3N x 2N) FP64 traction operator (the
reference's six N x N matrices, 6 N^2 GF entries) plus its FP32 copy.
``value`` = GF entries/s with the mesh resident on the device; ``e2e`` = the
same through the host-buffer C-ABI call (mesh in, FP64 operator out to pinned
host memory).  The same run also measures plain FP64 and FP32-operator RK45
stepping on that operator (RK stages/s, 7 right-hand-side evaluations per
attempted step) and reports it under ``stepping``.

    python bench.py [--steps K] [--warmup W] [--gpus N] [--impl ours|reference]

--impl reference times the reference algorithm on the host cores (the C
restatement in oracle/, or the reference's own TDstressFS_C built from source
into oracle/_ref/ when present) on a bounded sample of the same workload.
Multi-GPU: replicas only (each rank assembles its own operator; no collective
on the data path).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "RK stages/s batched+mixed vs plain FP64, same GPU, ≤1e-5 slip err; GF entries/s"
MU = 32038120320.0
LAM = 32038120320.0
RHO = MU / 3464.0 ** 2


def workload(quick=False):
    from pyquake3d_gb300 import mesh
    if quick:
        L, W, nx, nz = 20.0, 10.0, 50, 20      # N = 2,000
    else:
        L, W, nx, nz = 80.0, 30.0, 200, 50     # N = 20,000
    nodes, tris = mesh.rough_fault(L, W, nx, nz, hurst=0.8, ratio=1e-3, seed=0)
    name = "gf_assembly_rough_%dx%dkm_N%d" % (L, W, tris.shape[0])
    return name, L, W, nodes, tris


class Clocks:
    """nvidia-smi samples every 200 ms while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.f = None

    def __enter__(self):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                p = [x.strip() for x in line.split(",")]
                if len(p) >= 9:
                    rows.append(p)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def fp64_peak_tflops(torch, dev):
    """FP64 rate measured here: torch.matmul float64 4096^3 (cuBLAS DGEMM), best of 5."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    b = torch.randn(n, n, dtype=torch.float64, device=dev)
    for _ in range(2):
        a @ b
    best = 1e9
    for _ in range(5):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        a @ b
        e.record()
        e.synchronize()
        best = min(best, s.elapsed_time(e) / 1e3)
    return 2.0 * n ** 3 / best / 1e12


# FP64 operations of one (receiver, source) pair of the assembly kernel
# (both unit slips, 6 entries): 318 add + 403 mul + 5 div + 3 sqrt, counted by
# oracle/count_gf_flops.cpp on the kernel's own device math.
GF_FLOP_PER_PAIR = 729
# The same pair with the published angular-dislocation expressions
# (src/TDstressFS_C.cpp:51-121) evaluated term by term and rotated tensor by
# tensor (src/TDstressFS_C.cpp:185-256), both slips sharing the geometry and
# 11 divisions: 1,016, counted by the same tool (the kernel's first form).
GF_FLOP_PER_PAIR_TERM_BY_TERM = 1016
# The same for the half-space kernel (main + image dislocation, the
# free-surface correction of the three sides in dual numbers): 5,412.7 add +
# 8,793.4 mul + 66.9 div + 18.0 sqrt per pair (and 18.0 transcendental calls),
# counted by oracle/count_hs_flops.cpp over every pair of the 40 x 20 km,
# N = 2,500 mesh of bench_halfspace (the count depends weakly on the mesh
# through the branches of the angular dislocations).
HS_FLOP_PER_PAIR = 14291
# Stores per pair: 6 FP64 + 6 FP32 entries.
GF_BYTES_PER_PAIR = 72


def gf_flops_per_pair():
    return GF_FLOP_PER_PAIR


def cpu_gf_sample(nodes, tris, seconds=12.0, kind=None):
    """Time the host CPU on a bounded sample (source columns) of the assembly."""
    import oracle
    N = tris.shape[0]
    cores = os.cpu_count() or 1
    ref_so = os.path.join(HERE, "oracle", "_ref", "libTDstressFS_ref.so")
    use_ref = (kind != "port") and os.path.exists(ref_so)
    if use_ref:
        fn, kind = _ref_assemble(ref_so, cores, nodes, tris), "reference"
    else:
        fn, kind = (lambda c0, c1: oracle.assemble_dense(nodes, tris, MU, LAM, cols=(c0, c1), nthreads=cores)), "port"
    # calibrate on a small slice (twice: the first call warms up), then size
    # the sample to ~`seconds`
    c1 = min(N, 4 * cores)
    for _ in range(2):
        t0 = time.perf_counter()
        fn(0, c1)
        dt = time.perf_counter() - t0
    ncols = int(min(N, max(c1, c1 * seconds / max(dt, 1e-3))))
    t0 = time.perf_counter()
    fn(0, ncols)
    dt = time.perf_counter() - t0
    entries = 6.0 * N * ncols
    return {"value": entries / dt, "unit": "GF entries/s", "cores": cores, "kind": kind,
            "sample": "%d of %d source columns x all %d receivers (%.3g entries, %.1f s)" % (ncols, N, N, entries, dt)}


def _ref_assemble(path, cores, nodes, tris):
    """Reference TDstressFS_C (built from its source) driven column by column
    from a thread pool (ctypes releases the GIL), strike and dip unit slip,
    then the traction projection -- the work of src/QDsim_gpu.py:1745-1785."""
    import concurrent.futures as cf
    from pyquake3d_gb300 import mesh
    lib = ctypes.CDLL(path)
    D = ctypes.POINTER(ctypes.c_double)
    lib.TDstressFS_C.argtypes = [D, D, D, ctypes.c_size_t, D, D, D] + [ctypes.c_double] * 5 + [ctypes.c_bool, D, D]
    lib.TDstressFS_C.restype = None
    fr, xg = mesh.element_frames(nodes, tris)
    X, Y, Z = (np.ascontiguousarray(xg[:, k]) for k in range(3))
    e1, e2, n = fr[:, 0:3], fr[:, 3:6], fr[:, 6:9]
    N = tris.shape[0]
    p = lambda a: a.ctypes.data_as(D)

    def column(j):
        P = [np.ascontiguousarray(nodes[tris[j, k] - 1]) for k in range(3)]
        out = []
        for Ss, Ds in ((1.0, 0.0), (0.0, 1.0)):
            s = np.empty((N, 6))
            e = np.empty((N, 6))
            lib.TDstressFS_C(p(X), p(Y), p(Z), N, p(P[0]), p(P[1]), p(P[2]), Ss, Ds, 0.0, MU, LAM, False, p(s), p(e))
            t = np.stack([s[:, 0] * n[:, 0] + s[:, 3] * n[:, 1] + s[:, 4] * n[:, 2],
                          s[:, 3] * n[:, 0] + s[:, 1] * n[:, 1] + s[:, 5] * n[:, 2],
                          s[:, 4] * n[:, 0] + s[:, 5] * n[:, 1] + s[:, 2] * n[:, 2]], axis=1)
            out.append(np.stack([np.sum(t * e1, 1), np.sum(t * e2, 1), np.sum(t * n, 1)]))
        return out

    def run(c0, c1):
        with cf.ThreadPoolExecutor(max_workers=cores) as ex:
            list(ex.map(column, range(c0, c1)))
    return run


def bench_reference(args):
    """The reference algorithm on the host cores.  One step = the GF assembly
    of a fixed sample of source columns (all receivers), sized in the warm-up
    to ~``--ref-step-seconds``; ``value`` = GF entries/s of that work (the
    rate a full assembly runs at: every source column costs the same), and
    ``ms_per_step`` is the time of the sample actually computed."""
    import oracle
    name, L, W, nodes, tris = workload(args.quick)
    N = tris.shape[0]
    cores = os.cpu_count() or 1
    ref_so = os.path.join(HERE, "oracle", "_ref", "libTDstressFS_ref.so")
    if os.path.exists(ref_so):
        fn, kind = _ref_assemble(ref_so, cores, nodes, tris), "reference"
    else:
        fn, kind = (lambda c0, c1: oracle.assemble_dense(nodes, tris, MU, LAM, cols=(c0, c1), nthreads=cores)), "port"
    # warm-up: calibration slices; the last one sizes the timed sample
    ncols = min(N, 4 * cores)
    for _ in range(max(1, args.warmup)):
        t0 = time.perf_counter()
        fn(0, ncols)
        dt = time.perf_counter() - t0
        ncols = int(min(N, max(4 * cores, ncols * args.ref_step_seconds / max(dt, 1e-3))))
    times = []
    for k in range(max(1, args.steps)):
        c0 = (k * ncols) % max(1, N - ncols + 1)
        t0 = time.perf_counter()
        fn(c0, c0 + ncols)
        times.append(time.perf_counter() - t0)
    entries = 6.0 * N * ncols
    val = entries * len(times) / sum(times)
    cb = {"value": val, "unit": "GF entries/s", "cores": cores, "kind": kind,
          "sample": "each step: %d of %d source columns x all %d receivers (%.3g GF entries), %d steps, "
                    "%.1f s in all" % (ncols, N, N, entries, len(times), sum(times))}
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": "GF entries/s", "n_gpus": args.gpus,
            "steps": len(times), "warmup": args.warmup, "ms_per_step": sum(times) / len(times) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": name, "N": N, "sample_columns": ncols, "entries_per_step": int(entries),
                       "full_assembly_entries": 6 * N * N, "halfspace": False,
                       "note": "a step is a sample of the assembly (ms_per_step is its time); value is the rate, "
                               "the same for the whole assembly"},
            "cpu_baseline": cb, "e2e": {"value": val, "unit": "GF entries/s", "h2d_bytes_per_step": 0,
                                         "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def bench_ours(args):
    import torch
    from pyquake3d_gb300 import _lib, gf, mesh
    from pyquake3d_gb300.QDsim_gpu import DenseDeviceSim, initial_state

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    L_ = _lib.load()
    name, Lkm, Wkm, nodes, tris = workload(args.quick)
    N = tris.shape[0]
    nodes_t, tris_t = gf.mesh_to_device(nodes, tris, dev)
    K64 = torch.empty((3 * N, 2 * N), dtype=torch.float64, device=dev)
    K32 = torch.empty((3 * N, 2 * N), dtype=torch.float32, device=dev)
    ws = torch.empty(L_.pq3d_gf_workspace_bytes(N), dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    def one():
        gf.assemble_dense(nodes_t, tris_t, MU, LAM, out64=K64, out32=K32, workspace=ws)

    for _ in range(args.warmup):
        one()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    with Clocks(local) as clk:
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for k in range(args.steps):
            starts[k].record(stream)
            one()
            ends[k].record(stream)
        t1.record(stream)
        torch.cuda.synchronize()
    total = t0.elapsed_time(t1) / 1e3
    per_launch = [s.elapsed_time(e) / 1e3 for s, e in zip(starts, ends)]
    if dist:
        t = torch.tensor([total], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total = float(t.item())
        if args.steps and dist:
            dist.barrier()
    entries = 6.0 * N * N * args.steps * world
    value = entries / total

    out = {}
    if rank == 0:
        peaks, peak_src = measured_peaks()
        fp64 = fp64_peak_tflops(torch, dev)
        fpp = gf_flops_per_pair()
        avg = sum(per_launch) / len(per_launch)
        roof = {"bound": "fp64", "unit": "TFLOP/s", "peak": fp64,
                "peak_source": "measured here: cuBLAS DGEMM (torch.matmul float64 4096^3); "
                               "MEASURED_PEAKS.json has no FP64 figure",
                "traffic": None, "launch_s": avg}
        if fpp:
            ach = fpp * N * N / avg / 1e12
            roof.update({"achieved": ach, "frac": ach / fp64, "flops_per_pair": fpp})
            # the same work counted as the published expressions term by term
            # (profiles/gf_flops.md): a rate that does not fall when the kernel
            # needs fewer operations
            tbt = GF_FLOP_PER_PAIR_TERM_BY_TERM * N * N / avg / 1e12
            roof["term_by_term"] = {"flops_per_pair": GF_FLOP_PER_PAIR_TERM_BY_TERM, "achieved": tbt,
                                    "frac": tbt / fp64}
        else:
            roof.update({"achieved": None, "frac": None})
        # DRAM bytes of one launch: ncu on the N=6,000 case (2.6 GB of stores,
        # 20x the L2) measured 70.7 B/pair (2.532 GB written + 13 MB read for
        # 3.6e7 pairs; ~60 MB of the 2.592 GB of stores still dirty in L2 at
        # kernel end); scaled to this launch by pairs.
        # the FP64 pipe is the bound: DGEMM issues only 2-flop DFMAs, this
        # kernel averages ~1.33 flops per FP64-pipe instruction (550 per
        # pair); ncu on the N = 6,000 case: FP64 pipe 90 % busy (active cycles)
        roof["fp64_pipe_active_pct"] = 89.8
        roof["pipe_note"] = ("ncu sm__inst_executed_pipe_fp64 pct_of_peak_sustained_active, capture of the N=6000 "
                             "case (bench.py --case gf_assembly)")
        roof["traffic"] = 70.7 * N * N
        roof["traffic_note"] = ("ncu dram__bytes_read+write at N=6000 (70.7 B/pair, 2.6 GB of stores, 20x the L2) "
                                "scaled by pairs (bench.py --case gf_assembly); algorithmic stores are %d B/pair"
                                % GF_BYTES_PER_PAIR)
        out["roofline"] = roof
        out["clocks"] = clk.summary()
        # -- end to end: host mesh in, FP64 operator out to pinned host memory
        host64 = torch.empty((3 * N, 2 * N), dtype=torch.float64, pin_memory=True)
        gf.assemble_dense_host(nodes, tris, MU, LAM, out64=host64)
        e2e_steps = max(1, min(args.steps, 3))
        t_e = time.perf_counter()
        for _ in range(e2e_steps):
            gf.assemble_dense_host(nodes, tris, MU, LAM, out64=host64)
        t_e = time.perf_counter() - t_e
        out["e2e"] = {"value": 6.0 * N * N * e2e_steps / t_e, "unit": "GF entries/s",
                      "h2d_bytes_per_step": int(nodes.nbytes + tris.astype(np.int64).nbytes),
                      "d2h_bytes_per_step": int(host64.numel() * 8), "steps": e2e_steps,
                      "path": "pq3d_assemble_dense_host (C-ABI): mesh copied in, the kernel stores the FP64 operator straight into the pinned host buffer (mapped)",
                      "outputs": "the FP64 operator only (the reference's dense path produces FP64 only); the "
                                 "device-timed value also writes the FP32 copy"}
        del host64
        # -- stepping on the assembled operator
        out["stepping"] = bench_stepping(torch, dev, K64, K32, nodes, tris, Lkm, Wkm, args, dict(peaks, fp64_tflops=fp64))
        if not args.no_batch:
            out["batched"] = bench_batched(torch, dev, args, peaks)
        if not args.no_hmat:
            out["hmatrix"] = bench_hmatrix(torch, dev, args, peaks)
        out["halfspace"] = bench_halfspace(torch, dev, args, fp64)
        if not args.no_serve:
            out["serving"] = bench_serving(torch, dev, args)
        if not args.no_cpu:
            out["cpu_baseline"] = cpu_gf_sample(nodes, tris, seconds=args.ref_seconds)
    line = {"metric": METRIC, "value": value, "unit": "GF entries/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": name, "N": N, "entries_per_step": 6 * N * N,
                       "operator_bytes_per_step": int(K64.numel() * 12), "halfspace": False,
                       "l2": "output operator (%.1f GB FP64 + FP32 per step) streams through L2; inputs are the "
                             "mesh only" % (K64.numel() * 12 / 1e9),
                       "parallelism": "replicas" if world > 1 else "single"},
            "gpu_launches": 3 * args.steps}
    line.update(out)
    if "batched" in out:
        # the primary metric's numbers in one compact key, last in the line
        line["batched_summary"] = batched_summary(out["batched"])
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def batched_summary(bt):
    """RK stages/s of the batched arms over the plain FP64 stepper on the same
    mesh, with how long each holds the 1e-5 slip bar against FP64 (lockstep)."""
    acc = bt.get("accuracy_vs_fp64", {})
    plain = bt["plain_fp64_single"]["rk_stages_per_s"]
    arms = {}
    for key, arm, acc_key, gemm in (("bf16x18_ff_attempt", "bf16x18", "bf16x18_ff_attempt", "bf16x18"),
                                    ("bf16x18_fp64_attempt", "bf16x18_fp64", "bf16x18_fp64_attempt", "bf16x18"),
                                    ("bf16x6_mixed_attempt", "bf16x6", "bf16x6", "bf16x6"),
                                    ("fp32_mixed_attempt", "fp32", "fp32", None)):
        if arm not in bt:
            continue
        a = {"rk_stages_per_s": round(bt[arm]["rk_stages_per_s"]),
             "ratio_vs_plain_fp64": round(bt[arm]["rk_stages_per_s"] / plain, 2)}
        if acc_key in acc:
            a["steps_within_1e-5"] = acc[acc_key]["steps_within_1e-5"]
        if gemm and "gemm" in bt.get(gemm, {}):
            a["product_hbm_frac"] = round(bt[gemm]["gemm"]["roofline"]["frac"], 3)
        if "e2e" in bt[arm]:
            a["e2e_rk_stages_per_s"] = round(bt[arm]["e2e"]["rk_stages_per_s"])
        arms[key] = a
    out = {"N": bt.get("N"), "B": bt.get("B"), "plain_fp64_rk_stages_per_s": round(plain), "arms": arms}
    if acc:
        out["lockstep"] = {"runs": acc.get("runs"), "accepted_steps": acc.get("accepted_steps"),
                           "fp64_perturbed_1e-12_steps_within_1e-5":
                               acc.get("fp64_perturbed_1e-12", {}).get("steps_within_1e-5")}
    return out


def bench_stepping(torch, dev, K64, K32, nodes, tris, Lkm, Wkm, args, peaks):
    """Plain FP64 and FP32-operator stepping on the assembled operator."""
    from pyquake3d_gb300 import mesh
    from pyquake3d_gb300.QDsim_gpu import DenseDeviceSim, initial_state
    N = tris.shape[0]
    _, xg = mesh.element_frames(nodes, tris)
    tab = mesh.friction_table(xg, Lkm * 1e3, Wkm * 1e3, seed=0)
    res = {"workload": "plain RK45 stepping on the same mesh (N=%d), %d accepted steps timed" % (N, args.rk_steps)}
    for label, K in (("fp64", K64), ("fp32_operator", K32)):
        sim = DenseDeviceSim(K, initial_state(tab, 1e-6, 1e-9), mu=MU, Cs=3464.0, V0=1e-6, Vpl=1e-9)
        sim.step(3)
        c0 = sim.read_ctrl()
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        sim.launch(args.rk_steps)
        e.record()
        e.synchronize()
        dt = s.elapsed_time(e) / 1e3
        c1 = sim.read_ctrl()
        att = c1.attempts - c0.attempts
        acc = c1.steps_done - c0.steps_done
        bytes_step = K.numel() * K.element_size()
        res[label] = {"rk_stages_per_s": 7.0 * att / dt, "accepted_steps_per_s": acc / dt,
                      "attempted": int(att), "accepted": int(acc), "ms_per_step": dt / max(acc, 1) * 1e3,
                      "status": int(c1.status),
                      "matvec_roofline": {"bound": "hbm", "unit": "GB/s",
                                          "achieved": bytes_step * acc / dt / 1e9, "peak": peaks["hbm_gbs"],
                                          "frac": bytes_step * acc / dt / 1e9 / peaks["hbm_gbs"],
                                          "note": "operator bytes per accepted step / step time (whole step)"}}
    res["product"] = bench_dense_product(torch, dev, K64, K32, peaks)
    if not args.no_cpu:
        res["cpu_baseline"] = cpu_stepping_sample(torch, K64, tab, seconds=min(args.ref_seconds, 12.0))
    return res


def bench_dense_product(torch, dev, K64, K32, peaks):
    """The stepping's traction product K.v' alone (pq3d_dense_matvec_f64 /
    _f32, the kernels' own launches, CUDA events, operator larger than L2):
    FP64 against the FP64 peak (GB300's FP64 rate, 1 DFMA per 8-byte entry,
    is below its HBM rate), FP32 against HBM."""
    from pyquake3d_gb300 import _lib
    L_ = _lib.load()
    N = K64.shape[1] // 2
    st = torch.cuda.current_stream(dev).cuda_stream
    g = torch.Generator(device=dev).manual_seed(0)
    v = torch.randn(2 * N, dtype=torch.float64, device=dev, generator=g)
    hi = v.float()
    vs = torch.stack([hi[0::2], hi[1::2], (v - hi.double()).float()[0::2], (v - hi.double()).float()[1::2]], 1)
    vs = vs.contiguous()
    out = torch.empty(3 * N, dtype=torch.float64, device=dev)
    res = {}
    for label, call, nbytes in (
            ("fp64", lambda: L_.pq3d_dense_matvec_f64(K64.data_ptr(), N, v.data_ptr(), out.data_ptr(), st),
             K64.numel() * 8),
            ("fp32", lambda: L_.pq3d_dense_matvec_f32(K32.data_ptr(), N, vs.data_ptr(), out.data_ptr(), st),
             K32.numel() * 4)):
        for _ in range(2):
            _lib.check(call())
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n = 5
        s.record()
        for _ in range(n):
            _lib.check(call())
        e.record()
        e.synchronize()
        t = s.elapsed_time(e) / 1e3 / n
        gbs = nbytes / t / 1e9
        r = {"launch_s": t, "hbm": {"achieved": gbs, "peak": peaks["hbm_gbs"], "frac": gbs / peaks["hbm_gbs"],
                                    "unit": "GB/s", "algorithmic_bytes": int(nbytes)}}
        if label == "fp64":
            tf = 2.0 * K64.numel() / t / 1e12
            r["bound"] = "fp64"
            r["fp64"] = {"achieved": tf, "peak": peaks["fp64_tflops"], "frac": tf / peaks["fp64_tflops"],
                         "unit": "TFLOP/s", "flops": 2.0 * K64.numel()}
        else:
            r["bound"] = "hbm"
        res[label] = r
    return res


def cpu_stepping_sample(torch, K64, tab, seconds=12.0):
    """The reference's CPU stepping algorithm (the oracle's NumPy
    restatement, bit for bit equal to QDsim_gpu.simu_forward) on the same
    operator and table, BLAS on all host threads, for about `seconds`."""
    import oracle
    from oracle.stepping import DenseStepper
    from pyquake3d_gb300 import gf
    ops = {k: np.ascontiguousarray(v.cpu().numpy()) for k, v in gf.split_ops(K64).items()}
    st = DenseStepper(ops, tab, mu=MU, density=MU / 3464.0 ** 2)
    st.run(1)
    t0 = time.perf_counter()
    att = 0
    steps = 0
    dttry = 1e-3
    while time.perf_counter() - t0 < seconds:
        h, dttry, a = st.simu_forward(dttry)
        att += a
        steps += 1
    dt = time.perf_counter() - t0
    return {"value": 7.0 * att / dt, "unit": "RK stages/s", "cores": os.cpu_count(), "kind": "port",
            "sample": "%d accepted steps (%d attempts) of the N=%d stepping, %.1f s" % (steps, att, tab.shape[0], dt)}


def bench_batched(torch, dev, args, peaks):
    """Config: batched ensemble, B runs on one planar N=10,000 mesh (100 x 50 km,
    1 km squares), per-run friction draws (seed 0).  Arms, each against the
    plain FP64 single-simulation stepper on the same mesh:
      bf16x6   three-piece BF16 product on tcgen05, FP32 mixed attempt (fast);
      bf16x18  exact fixed-point slices on tcgen05 (the FP64 product to ~1e-9
               normwise), float-float attempt: the arm that tracks the FP64
               trajectory;
      bf16x18_fp64  the same product with the reference-arithmetic FP64
               attempt;
      fp32     FP32 operator on CUDA cores, FP32 mixed attempt."""
    from pyquake3d_gb300 import _lib, autotune, gf, mesh
    from pyquake3d_gb300.ensemble import Ensemble, PackedFixOperator, PackedOperator
    from pyquake3d_gb300.QDsim_gpu import DenseDeviceSim, initial_state
    L_ = _lib.load()
    Lkm, Wkm, nx, nz = (100.0, 50.0, 100, 50) if not args.quick else (40.0, 20.0, 40, 20)
    B = args.batch
    nodes, tris = mesh.planar_fault(Lkm, Wkm, nx, nz)
    N = tris.shape[0]
    _, xg = mesh.element_frames(nodes, tris)
    tabs = mesh.ensemble_tables(xg, Lkm * 1e3, Wkm * 1e3, B=B, seed=0, v_nuc=1e-3)
    K64, K32 = gf.assemble_dense(nodes, tris, MU, LAM, device=dev)
    P = PackedOperator(K64)
    # the mesh's own cell order: on this planar workload it held 1e-5 longer
    # than the cluster tree's compact order (16 runs in lockstep: 106 against
    # 94 accepted steps with either attempt)
    PF = PackedFixOperator(K64)
    # launch shapes of the tensor-core products from the project's autotuner,
    # before anything is timed
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    shape = autotune.tune_bf16x6(P, B)
    shape_fix = autotune.tune_bf16x18(PF, min(B, 64))
    tune_s = time.perf_counter() - t0
    res = {"workload": "batched ensemble: planar %dx%d km, N=%d, B=%d runs, per-run a-b, Dc, sigma_n, nucleation "
                       "patch from seed 0; RK stages = 7 x attempted steps, all runs" % (Lkm, Wkm, N, B),
           "N": N, "B": B}
    out = {}
    st = torch.cuda.current_stream(dev).cuda_stream
    # (key, product, operator, attempt); the product alone is timed with the
    # first arm of each tensor-core product
    arms = [("bf16x6", "bf16x6", P, "mixed"), ("bf16x18", "bf16x18", PF, "ff"),
            ("bf16x18_fp64", "bf16x18", PF, "fp64"), ("fp32", "fp32", K32, "mixed")]
    for key, prec, K, attempt in arms:
        if prec == "bf16x18" and B > 64:
            continue
        ens = Ensemble(K, tabs, mu=MU, Cs=3464.0, precision=prec, attempt=attempt,
                       nsplit=args.nsplit if prec == "bf16x6" else None)
        ens.iterate(2)
        torch.cuda.synchronize()
        ens.capture(args.graph_iters)
        ens.replay(1)
        torch.cuda.synchronize()
        st0 = ens.stages()
        reps = max(1, args.batch_iters // args.graph_iters)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with Clocks(dev.index or 0) as clk:
            s.record()
            ens.replay(reps)
            e.record()
            e.synchronize()
        dt = s.elapsed_time(e) / 1e3
        st1 = ens.stages()
        c = ens.read_ctrl()
        out[key] = {"product": prec, "attempt": attempt, "rk_stages_per_s": (st1 - st0) / dt,
                    "iterations": reps * args.graph_iters, "ms_per_iteration": dt / (reps * args.graph_iters) * 1e3,
                    "accepted_steps": int(sum(x.steps for x in c)), "failed_runs": int(sum(x.status != 0 for x in c)),
                    "clocks": clk.summary(), "error_word": ens.error_word() if prec != "fp32" else 0}
        if key == "bf16x18":
            # end to end through the public API: the runs' tables from host
            # memory into a fresh ensemble (state set-up on the device), the
            # same number of graph-replayed iterations, the slips read back
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            e2 = Ensemble(K, tabs, mu=MU, Cs=3464.0, precision=prec, attempt=attempt, nsplit=ens.nsplit)
            e2.iterate(2)
            e2.capture(args.graph_iters)
            e2.replay(reps + 1)
            slips = (e2.t["slip1"].cpu(), e2.t["slip2"].cpu())
            t_e2e = time.perf_counter() - t0
            out[key]["e2e"] = {"rk_stages_per_s": e2.stages() / t_e2e, "seconds": t_e2e,
                               "iterations": 2 + (reps + 1) * args.graph_iters,
                               "h2d_bytes": int(tabs.nbytes), "d2h_bytes": int(sum(x.numel() * 8 for x in slips)),
                               "note": "Ensemble(...) from the host tables, iterate + graph capture + replays, the "
                                       "slips copied back: wall clock of the public API calls"}
            del e2, slips
        if key in ("bf16x6", "bf16x18"):
            # the tensor-core product alone, CUDA events over repeated launches
            if prec == "bf16x6":
                launch = lambda: L_.pq3d_batch_gemm_bf16x6(P.data.data_ptr(), ens.vop.data_ptr(), N, B, ens.nsplit,
                                                           ens.tc_ctas, ens.t["rates"].data_ptr(), ens.ws.data_ptr(),
                                                           ens.ws.numel(), st)
                op_bytes = P.data.numel()
                flops = 6 * 2.0 * (3 * N) * (2 * N) * ens.Bp
                note = "packed BF16 3-piece operator streamed once per product"
                fnote = "6 BF16 products x 2 x 3N x 2N x Bp"
            else:
                launch = lambda: L_.pq3d_batch_gemm_bf16x18(PF.data.data_ptr(), ens.vop.data_ptr(), N, B, ens.nsplit,
                                                            ens.t["rates"].data_ptr(), ens.ws.data_ptr(),
                                                            ens.ws.numel(), st)
                op_bytes = PF.data.numel()
                flops = 18 * 2.0 * (3 * N) * (2 * N) * ((B + 31) // 32 * 32)
                note = "packed fixed-point operator (4 BF16 slices, 8 B per entry) streamed once per product"
                fnote = "18 BF16 slice products x 2 x 3N x 2N x runs (rounded up to 32)"
            for _ in range(3):
                launch()
            nl = 20
            s.record()
            for _ in range(nl):
                launch()
            e.record()
            e.synchronize()
            tg = s.elapsed_time(e) / 1e3 / nl
            sh = shape if prec == "bf16x6" else shape_fix
            out[key]["gemm"] = {"launch_s": tg, "nsplit": ens.nsplit, "ctas_per_sm": ens.tc_ctas,
                                 "autotune": dict(sh, tune_s=tune_s),
                                 "roofline": {"bound": "hbm", "unit": "GB/s", "achieved": op_bytes / tg / 1e9,
                                              "peak": peaks["hbm_gbs"], "frac": op_bytes / tg / 1e9 / peaks["hbm_gbs"],
                                              "algorithmic_bytes": op_bytes, "note": note},
                                 "tensor": {"achieved_tflops": flops / tg / 1e12, "peak_tflops": peaks["bf16_tflops"],
                                            "frac": flops / tg / 1e12 / peaks["bf16_tflops"], "flops": flops,
                                            "note": fnote}}
            if ens.error_word() != 0:
                out[key]["error_word"] = ens.error_word()
        del ens
        torch.cuda.empty_cache()
    # plain FP64 single simulation on the same mesh (run 0's parameters)
    sim = DenseDeviceSim(K64, initial_state(tabs[0], 1e-6, 1e-9), mu=MU, Cs=3464.0, V0=1e-6, Vpl=1e-9)
    sim.step(3)
    c0 = sim.read_ctrl()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    sim.launch(args.rk_steps)
    e.record()
    e.synchronize()
    dt = s.elapsed_time(e) / 1e3
    c1 = sim.read_ctrl()
    plain = 7.0 * (c1.attempts - c0.attempts) / dt
    out["plain_fp64_single"] = {"rk_stages_per_s": plain, "accepted_steps": int(c1.steps_done - c0.steps_done),
                                "ms_per_step": dt / max(1, c1.steps_done - c0.steps_done) * 1e3}
    for key, _, _, _ in arms:
        if key in out:
            out["ratio_%s_vs_plain_fp64" % key] = out[key]["rk_stages_per_s"] / plain
    if args.acc_runs > 0:
        out["accuracy_vs_fp64"] = batched_accuracy(torch, K64, K32, P, PF, tabs[:args.acc_runs], args.acc_steps)
    res.update(out)
    del K64, K32, P, PF
    torch.cuda.empty_cache()
    return res


def batched_accuracy(torch, K64, K32, P, PF, tabs, max_steps, every=5):
    """Slip error of the mixed-precision ensembles against the FP64 batched
    stepper (the reference arithmetic, FP64 operator) on the same runs, in
    lockstep (pyquake3d_gb300.ensemble.lockstep: same step sizes and
    decisions, so the differences are the arithmetic's alone).  Beside them
    runs the FP64 stepper itself with each run's initial slip rates perturbed
    by 1e-12 (relative, random sign): the floor set by the sensitivity of the
    trajectories (nucleation amplifies any perturbation by orders of
    magnitude).  Per variant: the accepted steps up to which the normwise
    relative slip error of every run stays within 1e-5, and the error at fixed
    step counts."""
    import numpy as np
    from pyquake3d_gb300.ensemble import Ensemble, lockstep
    pert = tabs.copy()
    pert[:, :, 7] *= 1.0 + 1e-12 * np.random.default_rng(7).choice([-1.0, 1.0], size=pert[:, :, 7].shape)
    kw = dict(mu=MU, Cs=3464.0, max_steps=max_steps)
    ref = Ensemble(K64, tabs, precision="fp64", **kw)
    others = {"bf16x18_ff_attempt": Ensemble(PF, tabs, precision="bf16x18", attempt="ff", **kw),
              "bf16x18_fp64_attempt": Ensemble(PF, tabs, precision="bf16x18", attempt="fp64", **kw),
              "bf16x18_mixed_attempt": Ensemble(PF, tabs, precision="bf16x18", attempt="mixed", **kw),
              "bf16x6": Ensemble(P, tabs, precision="bf16x6", **kw),
              "fp32": Ensemble(K32, tabs, precision="fp32", **kw),
              "fp64_perturbed_1e-12": Ensemble(K64, pert, precision="fp64", **kw)}
    r = lockstep(ref, others, max_steps, every=every)
    info = r.pop("_ref")
    out = {"runs": tabs.shape[0], **info, "bar": 1e-5,
           "method": "lockstep with the FP64 batched stepper (same step sizes and decisions: the FP64 error norms "
                     "handed over between the halves of each iteration); checkpoints every %d iterations" % every}
    for k, v in r.items():
        out[k] = {"steps_within_1e-5": v["steps_within"], "slip_rel_err_at_steps": v["slip_rel_err_at_steps"],
                  "max_slip_rate_rel_err_within": v["max_slip_rate_err_within"], "failed_runs": v["failed_runs"]}
    return out


def bench_hmatrix(torch, dev, args, peaks):
    """Config: H-matrix path.  Rough fault 200 x 40 km, 500 x 100 cells ->
    N = 100,000; cluster leaf 64, block leaf 64, eta = 2, ACA tolerance 1e-4,
    FP32 factors.  RK45 stepping with the H-matrix product for a bounded
    number of stages; product error against dense FP64 rows (assembly kernel)
    at 1,000 seeded receivers."""
    from pyquake3d_gb300 import gf, mesh
    from pyquake3d_gb300.ensemble import Ensemble
    from pyquake3d_gb300.hmatrix import HMatrix
    Lkm, Wkm, nx, nz = (200.0, 40.0, 500, 100) if not args.quick else (40.0, 20.0, 80, 40)
    nodes, tris = mesh.rough_fault(Lkm, Wkm, nx, nz, hurst=0.8, ratio=1e-3, seed=0)
    N = tris.shape[0]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    H = HMatrix(nodes, tris, MU, LAM, min_size=64, mini_leaf=64, eta=2.0, tol=1e-4, device=dev)
    torch.cuda.synchronize()
    t_build = time.perf_counter() - t0
    res = {"workload": "H-matrix: rough %dx%d km, N=%d, leaf 64, eta 2, ACA tol 1e-4, FP32 factors" % (Lkm, Wkm, N),
           "build_s": t_build, "build_phases_s": H.build_phases, "partition": H.partition_info, "stats": H.stats}
    # product timing (B = 1)
    v = torch.randn(1, 2 * N, dtype=torch.float64, device=dev)
    ws = torch.empty(H.workspace_bytes(1), dtype=torch.uint8, device=dev)
    out = torch.empty(1, 3 * N, dtype=torch.float64, device=dev)
    for _ in range(3):
        H.apply(v, out, ws)
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(10):
        H.apply(v, out, ws)
    e.record()
    e.synchronize()
    ta = s.elapsed_time(e) / 10 / 1e3
    res["apply_ms"] = ta * 1e3
    res["apply_roofline"] = {"bound": "hbm", "unit": "GB/s", "achieved": H.stats["bytes"] / ta / 1e9,
                             "peak": peaks["hbm_gbs"], "frac": H.stats["bytes"] / ta / 1e9 / peaks["hbm_gbs"],
                             "algorithmic_bytes": H.stats["bytes"], "note": "dense blocks + U + V (FP32) once"}
    # error against dense FP64 rows at 1000 seeded receivers
    rng = np.random.default_rng(0)
    recv = np.sort(rng.choice(N, size=min(1000, N), replace=False))
    vv = v[0]
    y = out[0]
    num = den = 0.0
    nodes_t, tris_t = gf.mesh_to_device(nodes, tris, dev)
    row = torch.empty((3, 2 * N), dtype=torch.float64, device=dev)
    wsg = torch.empty(L_ws_bytes(N), dtype=torch.uint8, device=dev)
    for i in recv:
        gf.assemble_dense(nodes_t, tris_t, MU, LAM, fp32_copy=False, rows=(int(i), int(i) + 1), out64=row, workspace=wsg)
        ref = row @ vv
        num += float(torch.sum((ref - y[3 * i:3 * i + 3]) ** 2))
        den += float(torch.sum(ref ** 2))
    res["error_vs_dense_rows"] = {"rel_l2": (num / den) ** 0.5, "receivers": int(len(recv)), "seed": 0}
    # stepping with the H-matrix product
    _, xg = mesh.element_frames(nodes, tris)
    tab = mesh.friction_table(xg, Lkm * 1e3, Wkm * 1e3, seed=0, v_nuc=1e-3)
    ens = Ensemble(H, tab[None], mu=MU, Cs=3464.0, precision="hmat")
    ens.iterate(2)
    torch.cuda.synchronize()
    st0 = ens.stages()
    iters = max(1, args.hmat_stages // 7)
    s.record()
    ens.iterate(iters)
    e.record()
    e.synchronize()
    dt = s.elapsed_time(e) / 1e3
    st1 = ens.stages()
    res["stepping"] = {"rk_stages_per_s": (st1 - st0) / dt, "stages": int(st1 - st0), "seconds": dt,
                       "status": int(ens.read_ctrl()[0].status)}
    del ens
    if not args.no_cpu:
        res["cpu_baseline"] = hmat_cpu_baseline(H, nodes, tris, res["apply_ms"] / 1e3, t_build)
    del H
    torch.cuda.empty_cache()
    return res


def hmat_cpu_baseline(H, nodes, tris, gpu_apply_s, gpu_build_s, n_lowrank=96, n_dense=48):
    """The reference's CPU H-matrix path restated (oracle/hmat_cpu.py), one
    host core: the product as blocks_process_MVM's per-block loop over this
    H-matrix's own storage (FP32 factors as stored), timed whole; the build
    as the reference's generator calls (one receiver x n sources, one source x
    m receivers) under partial-pivot ACA on a seeded sample of the low-rank
    blocks and dense evaluation of a sample of the dense blocks, extrapolated
    to all blocks by pair evaluations (the ACA ones at the device's ranks)."""
    from oracle import hmat_cpu
    blocks = H.blocks_host
    rank = H.rank.cpu().numpy()
    off = H.off.cpu().numpy()
    data = H.data.cpu().numpy()
    x = np.random.default_rng(0).standard_normal(2 * H.N).astype(np.float32)
    t0 = time.perf_counter()
    hmat_cpu.matvec(blocks[:, :4], data, off, rank, x)
    t_mv = time.perf_counter() - t0
    del data
    frames, xg = hmat_cpu.element_frames(nodes, tris)
    perm = H.perm_host
    m = (blocks[:, 1] - blocks[:, 0]).astype(np.int64)
    n = (blocks[:, 3] - blocks[:, 2]).astype(np.int64)
    lr = np.nonzero(blocks[:, 4] == 1)[0]
    dn = np.nonzero(blocks[:, 4] == 0)[0]
    rng = np.random.default_rng(0)
    out = {"unit": "s", "cores": 1, "kind": "port",
           "product": {"value": t_mv, "gpu_s": gpu_apply_s, "ratio": t_mv / gpu_apply_s,
                       "sample": "one whole product (all %d blocks), FP32 factors" % len(blocks)}}
    t_lr = ev_lr = 0.0
    for b in rng.choice(lr, size=min(len(lr), n_lowrank), replace=False):
        r0, r1, c0, c1 = (int(v) for v in blocks[b, :4])
        gen = hmat_cpu.BlockGen(nodes, tris, frames, xg, perm[r0:r1], perm[c0:c1], MU, LAM)
        t0 = time.perf_counter()
        hmat_cpu.aca_block(gen, int(min(128, 3 * m[b], 2 * n[b])), 1e-4)
        t_lr += time.perf_counter() - t0
        ev_lr += gen.evals
    t_dn = ev_dn = 0.0
    for b in rng.choice(dn, size=min(len(dn), n_dense), replace=False):
        r0, r1, c0, c1 = (int(v) for v in blocks[b, :4])
        gen = hmat_cpu.BlockGen(nodes, tris, frames, xg, perm[r0:r1], perm[c0:c1], MU, LAM)
        t0 = time.perf_counter()
        hmat_cpu.dense_block(gen)
        t_dn += time.perf_counter() - t0
        ev_dn += gen.evals
    rk = np.where(rank[lr] >= 0, rank[lr], np.minimum(128, np.minimum(3 * m[lr], 2 * n[lr])))
    total_lr = float(np.sum((rk + 1) * (2 * n[lr] + m[lr])))   # a row (2n) and a column (m) per term
    total_dn = float(np.sum(2 * m[dn] * n[dn]))
    est = total_lr * t_lr / max(ev_lr, 1.0) + total_dn * t_dn / max(ev_dn, 1.0)
    out["build"] = {"value": est, "gpu_s": gpu_build_s, "ratio": est / gpu_build_s,
                    "sample": "%d low-rank blocks (%.3g pair evaluations, %.1f s) and %d dense blocks (%.3g, %.1f s), "
                              "extrapolated by pair evaluations to %.3g (ACA at the device's ranks) + %.3g (dense)"
                              % (min(len(lr), n_lowrank), ev_lr, t_lr, min(len(dn), n_dense), ev_dn, t_dn,
                                 total_lr, total_dn)}
    return out


def bench_halfspace(torch, dev, args, fp64_tflops=None):
    """Half-space GF assembly (image dislocation + free-surface correction):
    rough fault 40 x 20 km reaching the free surface, 50 x 25 cells ->
    N = 2,500 (1 km cells), FP64 operator + FP32 copy, against the full-space
    assembly of the same mesh."""
    from pyquake3d_gb300 import gf, mesh
    nodes, tris = mesh.rough_fault(40.0, 20.0, 50, 25, hurst=0.8, ratio=1e-3, seed=0)
    N = tris.shape[0]
    nodes_t, tris_t = gf.mesh_to_device(nodes, tris, dev)
    K64 = torch.empty((3 * N, 2 * N), dtype=torch.float64, device=dev)
    K32 = torch.empty((3 * N, 2 * N), dtype=torch.float32, device=dev)
    ws = torch.empty(L_ws_bytes(N), dtype=torch.uint8, device=dev)
    res = {"workload": "half-space GF assembly: rough 40x20 km to the surface, N=%d" % N}
    for half in (False, True):
        for _ in range(2):
            gf.assemble_dense(nodes_t, tris_t, MU, LAM, halfspace=half, out64=K64, out32=K32, workspace=ws)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = 3
        s.record()
        for _ in range(reps):
            gf.assemble_dense(nodes_t, tris_t, MU, LAM, halfspace=half, out64=K64, out32=K32, workspace=ws)
        e.record()
        e.synchronize()
        t = s.elapsed_time(e) / reps / 1e3
        res["halfspace" if half else "fullspace"] = {"s": t, "pairs_per_s": N * N / t, "entries_per_s": 6 * N * N / t}
    res["cost_ratio"] = res["halfspace"]["s"] / res["fullspace"]["s"]
    if not args.no_cpu:
        # the oracle's C restatement of the half-space path on all host cores,
        # a bounded sample of source columns (calibrated on 16, then ~3 s)
        import oracle
        cores = os.cpu_count() or 1
        ncol = min(N, 16)
        t0 = time.perf_counter()
        oracle.assemble_dense(nodes, tris, MU, LAM, halfspace=True, cols=(0, ncol), nthreads=cores)
        dt = time.perf_counter() - t0
        ncol = int(min(N, max(ncol, ncol * 3.0 / max(dt, 1e-3))))
        t0 = time.perf_counter()
        oracle.assemble_dense(nodes, tris, MU, LAM, halfspace=True, cols=(0, ncol), nthreads=cores)
        dt = time.perf_counter() - t0
        res["halfspace"]["cpu_baseline"] = {"value": N * ncol / dt, "unit": "pairs/s", "cores": cores, "kind": "port",
                                            "sample": "%d of %d source columns x all receivers, %.1f s"
                                                      % (ncol, N, dt),
                                            "gpu_ratio": res["halfspace"]["pairs_per_s"] / (N * ncol / dt)}
    if fp64_tflops:
        hs = res["halfspace"]
        ach = HS_FLOP_PER_PAIR * N * N / hs["s"] / 1e12
        hs["roofline"] = {"bound": "fp64", "unit": "TFLOP/s", "flops_per_pair": HS_FLOP_PER_PAIR,
                          "achieved": ach, "peak": fp64_tflops, "frac": ach / fp64_tflops,
                          "peak_source": "cuBLAS DGEMM measured in this run",
                          "flop_ratio_vs_fullspace": HS_FLOP_PER_PAIR / GF_FLOP_PER_PAIR}
    del K64, K32
    torch.cuda.empty_cache()
    return res


SERVE_MESHES = [(2000, 50, 20), (4000, 80, 25), (6000, 100, 30), (8000, 100, 40), (12000, 150, 40),
                (20000, 200, 50), (30000, 250, 60), (40000, 250, 80)]


def bench_serving(torch, dev, args):
    """Config: serving loop.  8 meshes, N = 2k..40k (0.5 km cells, planar and
    rough alternating; dense BF16x6 operator for N <= 20k, H-matrix above),
    requests by a seeded Poisson process (4/s), per-request friction draw and
    simulated span U(1, 20) years, 16 slots per mesh, HBM budget 150 GB."""
    from pyquake3d_gb300 import gf, mesh
    from pyquake3d_gb300.ensemble import Ensemble
    from pyquake3d_gb300.QDsim_gpu import DenseDeviceSim, initial_state
    from pyquake3d_gb300.serving import YEAR, Request, Server, poisson_arrivals
    sizes = SERVE_MESHES if not args.quick else [(n // 8, nx // 4, nz // 2) for n, nx, nz in SERVE_MESHES[:4]]
    meshes = []
    for k, (_, nx, nz) in enumerate(sizes):
        f = mesh.planar_fault if k % 2 == 0 else mesh.rough_fault
        L, W = nx * 0.5, nz * 0.5
        nodes, tris = f(L, W, nx, nz)
        meshes.append({"nodes": nodes, "tris": tris, "L": L * 1e3, "W": W * 1e3})
    srv = Server(meshes, mu=MU, lam=LAM, cs=3464.0, slots=16, budget_bytes=150e9, graph_iters=8,
                 max_steps=args.serve_max_steps, device=dev, dense_precision=args.serve_precision)
    nreq = args.serve_requests
    arr = poisson_arrivals(nreq, 4.0, seed=0)
    rng = np.random.default_rng(0)
    reqs = []
    for i in range(nreq):
        m = int(rng.integers(len(meshes)))
        _, xg = mesh.element_frames(meshes[m]["nodes"], meshes[m]["tris"])
        tab = mesh.ensemble_tables(xg, meshes[m]["L"], meshes[m]["W"], B=1, seed=int(rng.integers(1 << 30)),
                                   v_nuc=1e-3)[0]
        reqs.append(Request(rid=i, mesh=m, arrival_s=float(arr[i]), table=tab,
                            span_s=float(rng.uniform(1.0, 20.0)) * YEAR))
    res = srv.run(reqs, time_limit_s=args.serve_time_limit)
    res["meshes"] = [{"N": int(sp["tris"].shape[0]), "kind": srv.kind[m], "operator_GB": srv.op_bytes[m] / 1e9,
                      "build_s": srv.build_s[m]} for m, sp in enumerate(meshes)]
    # one at a time on the plain path, measured: each request (its own table
    # and span) run alone, in arrival order, on the plain FP64 stepper (dense
    # meshes) or a single-run H-matrix ensemble with the FP64 attempt, until
    # its span or the step cap, while the measuring budget lasts; requests
    # past the budget take their mesh's measured plain rate x their own
    # served attempt count (stated in the result).  Time to result = FIFO.
    del srv
    torch.cuda.empty_cache()
    durations, how = {}, {}
    budget_end = time.perf_counter() + args.serve_plain_seconds
    order = sorted([r for r in reqs if r.done_s is not None], key=lambda r: r.arrival_s)
    rate = {}
    for m, sp in enumerate(meshes):
        mine = [r for r in order if r.mesh == m]
        if not mine:
            continue
        N = int(sp["tris"].shape[0])
        if res["meshes"][m]["kind"].startswith("dense"):
            K64, _ = gf.assemble_dense(sp["nodes"], sp["tris"], MU, LAM, fp32_copy=False, device=dev)
            H = None
        else:
            from pyquake3d_gb300.hmatrix import HMatrix
            K64, H = None, HMatrix(sp["nodes"], sp["tris"], MU, LAM, device=dev, min_size=64, mini_leaf=64, eta=2.0,
                                   tol=1e-4)
        st_all, t_all = 0, 0.0
        for r in mine:
            if time.perf_counter() > budget_end and st_all > 0:
                continue
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            if H is None:
                sim = DenseDeviceSim(K64, initial_state(r.table, 1e-6, 1e-9), mu=MU, Cs=3464.0, V0=1e-6, Vpl=1e-9)
                while True:
                    sim.step(10)
                    c = sim.read_ctrl()
                    if c.time >= r.span_s or c.steps_done >= args.serve_max_steps or c.status != 0:
                        break
                att = int(c.attempts)
                del sim
            else:
                ens = Ensemble(H, r.table[None], mu=MU, Cs=3464.0, precision="hmat", attempt="fp64", t_end=r.span_s,
                               max_steps=args.serve_max_steps)
                while ens.read_ctrl()[0].active:
                    ens.iterate(50)
                att = int(ens.read_ctrl()[0].attempts)
                del ens
            torch.cuda.synchronize()
            durations[r.rid] = time.perf_counter() - t0
            how[r.rid] = "measured"
            st_all += 7 * att
            t_all += durations[r.rid]
        rate[m] = st_all / t_all if t_all > 0 else float("nan")
        for r in mine:
            if r.rid not in durations:
                durations[r.rid] = 7.0 * r.attempts / rate[m]
                how[r.rid] = "extrapolated"
        del K64, H
        torch.cuda.empty_cache()
    t_free = 0.0
    ttr = []
    for r in order:
        start = max(r.arrival_s, t_free)
        t_free = start + durations[r.rid]
        ttr.append(t_free - r.arrival_s)
    nmeas = sum(1 for v in how.values() if v == "measured")
    res["sequential_plain"] = {"p50_time_to_result_s": float(np.percentile(ttr, 50)) if ttr else None,
                               "p99_time_to_result_s": float(np.percentile(ttr, 99)) if ttr else None,
                               "requests_measured": nmeas, "requests_extrapolated": len(how) - nmeas,
                               "plain_rk_stages_per_s": {str(int(meshes[m]["tris"].shape[0])): v
                                                         for m, v in rate.items()},
                               "method": "each request run alone in arrival order on the plain FP64 path (dense: "
                                         "the FP64 stepper; H-matrix meshes: one H-matrix run with the FP64 "
                                         "attempt) to its span or the step cap, wall-clocked, within a %.0f s "
                                         "budget; the rest at their mesh's measured plain rate x their served "
                                         "attempt count; FIFO one at a time from arrival" % args.serve_plain_seconds}
    res["workload"] = ("serving: %d requests, Poisson 4/s seed 0, 8 meshes N=%s, 16 slots/mesh, 150 GB budget, "
                       "span U(1,20) yr, max %d steps/run" % (nreq, [m[0] for m in sizes], args.serve_max_steps))
    res["arithmetic"] = {
        "dense_bf16x18": "exact fixed-point BF16x18 product + float-float Dormand-Prince attempt: slip within 1e-5 "
                         "of the FP64 stepper for ~100 accepted steps (lockstep, N=10,000; the batched section's "
                         "bf16x18_ff_attempt), the FP64 stepper's own 1e-12-perturbation floor ~120",
        "dense_bf16x6": "BF16x6 product + mixed attempt: within 1e-5 for ~25 accepted steps",
        "hmatrix": "FP32 ACA factors (tol 1e-4) + mixed attempt: the H-matrix approximation of the operator",
        "runs_beyond_the_horizon": "past its horizon a run follows another trajectory of the same chaotic "
                                   "system, as the FP64 stepper does past ~120 steps under a 1e-12 perturbation"}
    return res


def L_ws_bytes(N):
    from pyquake3d_gb300 import _lib
    return _lib.load().pq3d_gf_workspace_bytes(N)


def profile_case(case):
    """Small single-kernel cases for ncu captures (no timing, no JSON):
    gf_assembly  full-space assembly, rough 60x25 km, N=6,000, FP64 + FP32 copy
                 (2.6 GB of stores, 20x the L2; 2 launches)
    hs_assembly  half-space assembly, rough 20x10 km to the surface, N=1,600 (2 launches)
    hmat_product H-matrix product, rough 200x40 km, N=100,000, B=1 (13 products)
    hmat_product_40k  the same, rough 100x40 km, N=40,000 (build scratch released
                 before the products; ~2 GB resident)
    tc_gemm      batched iterations (tcgen05 BF16x6 product, attempt, decision, update),
                 planar 60x50 km, N=6,000, B=64 (12 iterations)
    f32_gemm     batched iterations with the plain FP32 product on CUDA cores, same
                 mesh and runs (6 iterations)
    fix_gemm     batched iterations with the fixed-point BF16x18 product and the FP64
                 attempt, same mesh and runs (6 iterations)
    ff_attempt   the same with the float-float attempt (6 iterations)
    batch_small  the CUDA-core batched products (FP64 and FP32, 16 runs, 3 iterations
                 each, planar 40 x 25 km, N = 2,000) and the dense matvec entry
                 points (pq3d_dense_matvec_f64 / _f32)
    points       the reference-shaped point entry points (TDstressFS_C full and half
                 space: 200,000 receivers x 1 source; TDstressEachSourceAtReceiver_C:
                 1 receiver x 20,000 sources, full and half space)
    aca          H-matrix build (partition, ACA, dense blocks), rough 100x25 km, N=20,000,
                 leaf 64, eta 2, tol 1e-4 (one ACA launch over all low-rank blocks)"""
    import torch
    from pyquake3d_gb300 import gf, mesh
    if case == "gf_assembly":
        nodes, tris = mesh.rough_fault(60.0, 25.0, 100, 30, hurst=0.8, ratio=1e-3, seed=0)
        K64, K32 = gf.assemble_dense(nodes, tris, MU, LAM)
        gf.assemble_dense(nodes, tris, MU, LAM, out64=K64, out32=K32)
    elif case == "hs_assembly":
        nodes, tris = mesh.rough_fault(20.0, 10.0, 40, 20, seed=0)
        K64, K32 = gf.assemble_dense(nodes, tris, MU, LAM, halfspace=True)
        gf.assemble_dense(nodes, tris, MU, LAM, halfspace=True, out64=K64, out32=K32)
    elif case in ("hmat_product", "hmat_product_40k"):
        from pyquake3d_gb300.hmatrix import HMatrix
        if case == "hmat_product":
            nodes, tris = mesh.rough_fault(200.0, 40.0, 500, 100, seed=0)
        else:
            nodes, tris = mesh.rough_fault(100.0, 40.0, 250, 80, seed=0)
        H = HMatrix(nodes, tris, MU, LAM, min_size=64, mini_leaf=64, tol=1e-4)
        torch.cuda.empty_cache()
        v = torch.randn(1, 2 * H.N, dtype=torch.float64, device="cuda")
        ws = torch.empty(H.workspace_bytes(1), dtype=torch.uint8, device="cuda")
        out = torch.empty(1, 3 * H.N, dtype=torch.float64, device="cuda")
        for _ in range(13):
            H.apply(v, out, ws)
    elif case == "tc_gemm":
        from pyquake3d_gb300.ensemble import Ensemble, PackedOperator
        nodes, tris = mesh.planar_fault(60.0, 50.0, 60, 50)
        K64, _ = gf.assemble_dense(nodes, tris, MU, LAM, fp32_copy=False)
        P = PackedOperator(K64)
        del K64
        torch.cuda.empty_cache()
        _, xg = mesh.element_frames(nodes, tris)
        tabs = mesh.ensemble_tables(xg, 60e3, 50e3, B=64, seed=0, v_nuc=1e-3)
        # a fixed launch shape (no tuning launches before the captured ones)
        Ensemble(P, tabs, mu=MU, Cs=3464.0, precision="bf16x6", nsplit=8, tc_ctas=2).iterate(12)
    elif case == "f32_gemm":
        from pyquake3d_gb300.ensemble import Ensemble
        nodes, tris = mesh.planar_fault(60.0, 50.0, 60, 50)
        K64, K32 = gf.assemble_dense(nodes, tris, MU, LAM)
        del K64
        torch.cuda.empty_cache()
        _, xg = mesh.element_frames(nodes, tris)
        tabs = mesh.ensemble_tables(xg, 60e3, 50e3, B=64, seed=0, v_nuc=1e-3)
        Ensemble(K32, tabs, mu=MU, Cs=3464.0, precision="fp32").iterate(6)
    elif case == "batch_small":
        from pyquake3d_gb300 import _lib
        from pyquake3d_gb300.ensemble import Ensemble
        nodes, tris = mesh.planar_fault(40.0, 25.0, 40, 25)
        N = tris.shape[0]
        K64, K32 = gf.assemble_dense(nodes, tris, MU, LAM)
        _, xg = mesh.element_frames(nodes, tris)
        tabs = mesh.ensemble_tables(xg, 40e3, 25e3, B=16, seed=0, v_nuc=1e-3)
        Ensemble(K64, tabs, mu=MU, Cs=3464.0, precision="fp64").iterate(3)
        Ensemble(K32, tabs, mu=MU, Cs=3464.0, precision="fp32").iterate(3)
        L = _lib.load()
        v = torch.randn(2 * N, dtype=torch.float64, device="cuda")
        out = torch.empty(3 * N, dtype=torch.float64, device="cuda")
        st = torch.cuda.current_stream().cuda_stream
        _lib.check(L.pq3d_dense_matvec_f64(K64.data_ptr(), N, v.data_ptr(), out.data_ptr(), st))
        hi = v.float()
        v32 = torch.cat([hi.view(N, 2), (v - hi.double()).float().view(N, 2)], 1).contiguous()   # [N][4]
        _lib.check(L.pq3d_dense_matvec_f32(K32.data_ptr(), N, v32.data_ptr(), out.data_ptr(), st))
    elif case == "points":
        import ctypes as _ct
        from pyquake3d_gb300 import _lib
        rng = np.random.default_rng(0)
        n = 200000
        X, Y = rng.uniform(-20e3, 20e3, n), rng.uniform(-20e3, 20e3, n)
        Z = rng.uniform(-20e3, -100.0, n)
        P = [np.array([0.0, 0.0, -1000.0]), np.array([1000.0, 0.0, -1000.0]), np.array([300.0, -577.35, -2000.0])]
        gf.TDstressFS(X, Y, Z, *P, 1.0, 0.0, 0.0, MU, LAM)
        gf.TDstressHS(X, Y, Z, *P, 1.0, 0.0, 0.0, MU, LAM)
        ns = 20000
        c = rng.uniform(-20e3, 20e3, (ns, 3))
        c[:, 2] = -np.abs(c[:, 2]) - 1500.0
        P1 = np.ascontiguousarray(c + [0.0, 0.0, 500.0])
        P2 = np.ascontiguousarray(c + [800.0, 0.0, 0.0])
        P3 = np.ascontiguousarray(c + [0.0, 600.0, -400.0])
        L = _lib.load()
        s = np.empty((ns, 6))
        e = np.empty((ns, 6))
        dp = lambda a: a.ctypes.data_as(_ct.POINTER(_ct.c_double))
        for hs in (False, True):
            L.TDstressEachSourceAtReceiver_C(100.0, 200.0, -300.0, dp(P1), dp(P2), dp(P3), ns, 1.0, 0.0, 0.0,
                                             MU, LAM, hs, dp(s), dp(e))
    elif case in ("fix_gemm", "ff_attempt"):
        from pyquake3d_gb300.ensemble import Ensemble, PackedFixOperator
        nodes, tris = mesh.planar_fault(60.0, 50.0, 60, 50)
        K64, _ = gf.assemble_dense(nodes, tris, MU, LAM, fp32_copy=False)
        P = PackedFixOperator(K64)
        del K64
        torch.cuda.empty_cache()
        _, xg = mesh.element_frames(nodes, tris)
        tabs = mesh.ensemble_tables(xg, 60e3, 50e3, B=64, seed=0, v_nuc=1e-3)
        # 3 partial sums: the product's balanced grid at this size on 152 SMs
        Ensemble(P, tabs, mu=MU, Cs=3464.0, precision="bf16x18", attempt="fp64" if case == "fix_gemm" else "ff",
                 nsplit=3).iterate(6)
    elif case == "aca":
        from pyquake3d_gb300.hmatrix import HMatrix
        nodes, tris = mesh.rough_fault(100.0, 25.0, 200, 50, seed=0)
        # built twice: the first build in a process pays the device warm-up
        first = HMatrix(nodes, tris, MU, LAM, min_size=64, mini_leaf=64, tol=1e-4).build_phases
        H = HMatrix(nodes, tris, MU, LAM, min_size=64, mini_leaf=64, tol=1e-4)
        # GF pair evaluations of the ACA: per iteration one residual row (n
        # sources) and one column (m receivers); rank + 1 iterations per block
        b = H.blocks_host
        rk = H.rank.cpu().numpy()
        lr = np.nonzero(b[:, 4] == 1)[0]
        m, n = b[lr, 1] - b[lr, 0], b[lr, 3] - b[lr, 2]
        pairs = int(np.sum((np.maximum(rk[lr], 0) + 1) * (m + n)))
        print(json.dumps({"stats": H.stats, "phases_first_build": first, "phases": H.build_phases,
                          "aca_pair_evaluations": pairs,
                          "aca_kernel_pairs_per_s": pairs / H.build_phases["aca_kernels"]}))
    else:
        raise SystemExit("unknown --case " + case)
    torch.cuda.synchronize()
    print("case %s done" % case)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--quick", action="store_true", help="N=2,000 case (profiling)")
    ap.add_argument("--rk-steps", type=int, default=1000)
    ap.add_argument("--ref-seconds", type=float, default=12.0)
    ap.add_argument("--ref-step-seconds", type=float, default=2.0,
                    help="reference arm: CPU seconds of one step's assembly sample")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-hmat", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=24)
    ap.add_argument("--serve-precision", default="bf16x18", choices=["bf16x18", "bf16x6"],
                    help="product of the dense serving meshes (bf16x18: float-float attempt, the accurate arm)")
    ap.add_argument("--serve-max-steps", type=int, default=3000)
    ap.add_argument("--serve-time-limit", type=float, default=90.0)
    ap.add_argument("--serve-plain-seconds", type=float, default=60.0,
                    help="budget for measuring the one-at-a-time plain baseline of the serving stream")
    ap.add_argument("--hmat-stages", type=int, default=500)
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--nsplit", type=int, default=None)
    ap.add_argument("--graph-iters", type=int, default=25)
    ap.add_argument("--batch-iters", type=int, default=300)
    ap.add_argument("--acc-runs", type=int, default=16, help="runs of the slip-accuracy check (0: skip)")
    ap.add_argument("--acc-steps", type=int, default=200)
    ap.add_argument("--case", default=None,
                    help="profiling case only (gf_assembly, hs_assembly, hmat_product, tc_gemm, f32_gemm, fix_gemm, aca)")
    args = ap.parse_args()
    if args.case:
        profile_case(args.case)
        return
    if args.impl == "reference":
        if int(os.environ.get("RANK", "0")) != 0:
            return
        bench_reference(args)
    else:
        bench_ours(args)


if __name__ == "__main__":
    main()
