"""Batched ensemble: B simulations that share one mesh, stepped together.

Each run has its own friction, stress and nucleation (its own per-cell table)
and its own adaptive dt; one device iteration does the traction product for
all runs as one (3N x 2N) x (2N x B) product, one Dormand-Prince attempt per
run, the per-run accept/reject decision and the update of the accepted runs
(rejected runs retry with their smaller dt).  Iterations are captured into a
CUDA graph and replayed without host synchronisation.

Precisions of the traction product (``precision=``):
  "fp64"   FP64 operator on CUDA cores (reference arithmetic, slow on GB300)
  "fp32"   FP32 operator copy on CUDA cores ("plain FP32")
  "bf16x6" the operator and v' each split into three BF16 pieces, the six
           leading cross products on the tcgen05 tensor cores with FP32
           accumulation in tensor memory; K slices added in float-float;
           launch shape (K slices, CTAs per SM) from :mod:`.autotune`
  "bf16x18" the operator (32 bits) and v' (48 bits) as exact fixed-point BF16
           slices (one exponent per 1024-column chunk of an operator row, per
           256-column span of a run), the 18 slice products down to 2^-40 of
           the leading one on the tensor cores with exact accumulation per
           span, spans and K slices added in float-float: the FP64 product to
           ~1e-9 of its scale, for runs that must track the FP64 trajectory
           (with attempt="ff" or "fp64"); at most 64 runs
  "hmat"   an :class:`~pyquake3d_gb300.hmatrix.HMatrix` (large meshes)
Time, slip, the state and the RK error norm stay FP64 in every mode.

The Dormand-Prince attempt (``attempt=``): "mixed" (default for the mixed
products) runs the seven right-hand sides in FP32 on the FP64 start state
with float-float exponent arguments; "fp64" runs them in the reference FP64
arithmetic (always for precision "fp64"); "ff" runs them in float-float on
the FP32 pipes, with the large exponent arguments reduced in FP64 once per
attempt: the FP64 attempt's accuracy at a fraction of its FP64 work.  The
FP32 stages add ~1e-7 of each step's increment; during nucleation the slip
rate's exponential dependence on the traction amplifies that, so runs that
must track the FP64 trajectory closely over many steps take attempt="ff" or
"fp64" (the product keeps its precision).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib, autotune
from .QDsim_gpu import initial_state

PRECISIONS = {"fp64": _lib.PQ3D_BATCH_FP64, "fp32": _lib.PQ3D_BATCH_FP32, "bf16x6": _lib.PQ3D_BATCH_BF16X6,
              "hmat": _lib.PQ3D_BATCH_HMAT, "bf16x18": _lib.PQ3D_BATCH_BF16X18}
STATE = ("Tno", "Tt1o", "Tt2o", "state", "slipv1", "slipv2", "slipv", "slip1", "slip2")
PARAMS = ("a", "b", "dc", "f0", "shear_loading", "normal_loading", "cos_rake0", "sin_rake0")


# K slices of the FP32 CUDA-core product: its 3N x B sums alone give too few
# threads to fill the SMs.  A constant, so that the summation order (and the
# bits) is the same for every batch, mesh size and row shard.
FP32_NSPLIT = 4


def padded_runs(B: int) -> int:
    return (B + 15) // 16 * 16


class PackedOperator:
    """The tensor-core operand: FP64 operator split into 3 BF16 pieces, packed
    as shared-memory tile images (built once per mesh)."""

    def __init__(self, K64: torch.Tensor):
        L = _lib.load()
        assert K64.dtype == torch.float64 and K64.is_contiguous()
        self.N = K64.shape[1] // 2
        self.device = K64.device
        self.data = torch.empty(L.pq3d_batch_operator_bytes(self.N), dtype=torch.uint8, device=self.device)
        _lib.check(L.pq3d_batch_pack_operator(K64.data_ptr(), self.N, self.data.data_ptr(),
                                              torch.cuda.current_stream(self.device).cuda_stream))


class PackedFixOperator:
    """The operand of the fixed-point tensor-core product ("bf16x18"): the FP64
    operator as four BF16 slices per row and 1024-column chunk (built once per
    mesh).

    xg: the (N, 3) element centroids.  With them the cells are taken in the
    depth-first order of the bisection cluster tree (``order``, ``pos``), so
    that every 256-column span -- whose largest |v'| sets the fixed-point grid
    of the 128 cells' v' slices -- and every 1024-column operator chunk cover
    one compact region of the fault.  In the mesh order a span of a long fault
    runs along its length, and the slow cells that share a span with a
    nucleating patch keep only the bits of their v' below the patch's."""

    def __init__(self, K64: torch.Tensor, xg=None):
        L = _lib.load()
        assert K64.dtype == torch.float64 and K64.is_contiguous()
        self.N = K64.shape[1] // 2
        self.device = K64.device
        if xg is not None:
            from .hmatrix import cluster_order
            self.order = cluster_order(xg, 1, self.device)
            self.pos = torch.empty_like(self.order)
            self.pos[self.order] = torch.arange(self.N, dtype=torch.int64, device=self.device)
        else:
            self.order = self.pos = None
        self.data = torch.empty(L.pq3d_batch_operator_fix_bytes(self.N), dtype=torch.uint8, device=self.device)
        _lib.check(L.pq3d_batch_pack_operator_fix(K64.data_ptr(), self.N,
                                                  self.order.data_ptr() if self.order is not None else None,
                                                  self.data.data_ptr(),
                                                  torch.cuda.current_stream(self.device).cuda_stream))


class Ensemble:
    """Device state and launch structure of B runs on one mesh.

    K: the (3N, 2N) operator -- FP64 for "fp64", FP32 for "fp32", a
    :class:`PackedOperator` for "bf16x6", a :class:`PackedFixOperator` for
    "bf16x18".  tables: (B, N, 10) per-cell tables
    (``read_parameter`` layout).

    shard=(cell0, N_total): this object steps cells [cell0, cell0 + N) of an
    N_total-cell mesh ("fp64" / "fp32"); K is then the shard's (3N, 2 N_total)
    row block and :mod:`pyquake3d_gb300.shards` drives the iterations."""

    def __init__(self, K, tables, *, mu, Cs, V0=1e-6, Vpl=1e-9, precision="bf16x6", attempt="mixed", nsplit=None,
                 tc_ctas=None, dttry=1e-3, max_steps=2 ** 62, t_end=float("inf"), fix_Tn=False, shard=None):
        L = _lib.load()
        self.precision = precision
        prec = PRECISIONS[precision]
        if attempt not in ("mixed", "fp64", "ff"):
            raise ValueError("attempt must be 'mixed', 'fp64' or 'ff'")
        self.attempt = "fp64" if precision == "fp64" else attempt
        tables = np.asarray(tables, dtype=np.float64)
        B, N = tables.shape[0], tables.shape[1]
        self.B, self.N, self.Bp = B, N, padded_runs(B)
        self.cell0, self.N_total = (0, N) if shard is None else (int(shard[0]), int(shard[1]))
        if shard is not None and precision not in ("fp64", "fp32"):
            raise ValueError("row shards need the fp64 or fp32 product")
        Nt = self.N_total
        dev = K.device
        self.device = dev
        if precision == "hmat":
            assert K.N == N
            kop = None
            nsplit = 1
            self.hmat = K
        elif precision == "bf16x18":
            assert isinstance(K, PackedFixOperator) and K.N == N
            if B > 64:
                raise ValueError("the bf16x18 product takes at most 64 runs")
            kop = K.data
            self.fix_op = K
            if nsplit is None:
                nsplit = autotune.tune_bf16x18(K, B)["nsplit"]
            tc_ctas = 1
        elif precision == "bf16x6":
            assert isinstance(K, PackedOperator) and K.N == N
            kop = K.data
            if nsplit is None or tc_ctas is None:
                shape = autotune.tune_bf16x6(K, B)
                nsplit = shape["nsplit"] if nsplit is None else nsplit
                tc_ctas = shape["ctas_per_sm"] if tc_ctas is None else tc_ctas
        else:
            assert isinstance(K, torch.Tensor) and K.shape == (3 * N, 2 * Nt) and K.is_contiguous()
            assert K.dtype == (torch.float64 if precision == "fp64" else torch.float32)
            kop = K
            nsplit = 1 if precision == "fp64" else (FP32_NSPLIT if nsplit is None else int(nsplit))
        self.K = kop
        self.nsplit = int(nsplit)
        self.tc_ctas = int(tc_ctas or 0)
        inits = [initial_state(t, V0, Vpl) for t in tables]
        f64 = dict(dtype=torch.float64, device=dev)
        self.t = {}
        for k in STATE + ("a", "b", "dc", "f0", "shear_loading", "normal_loading"):
            self.t[k] = torch.as_tensor(np.stack([s[k] for s in inits]), **f64).contiguous()
        self.t["cos_rake0"] = torch.cos(torch.as_tensor(np.stack([s["rake0"] for s in inits]), **f64)).contiguous()
        self.t["sin_rake0"] = torch.sin(torch.as_tensor(np.stack([s["rake0"] for s in inits]), **f64)).contiguous()
        self.t["rates"] = torch.zeros(self.nsplit * self.Bp * 3 * N, **f64)
        self.t["cand"] = torch.zeros(B * N * 4, **f64)
        if self.attempt == "mixed":   # start-of-step constants of the mixed-precision attempt
            self.t["base"] = torch.zeros(_lib.PQ3D_BATCH_BASE_FIELDS * B * N, dtype=torch.float32, device=dev)
        if precision in ("fp64", "hmat"):
            self.vop = torch.zeros(self.Bp * 2 * Nt, **f64)
        elif precision == "fp32":
            self.vop = torch.zeros(self.Bp * 2 * Nt, dtype=torch.float32, device=dev)
        elif precision == "bf16x18":
            self.vop = torch.zeros(L.pq3d_batch_rhs_fix_bytes(N, B), dtype=torch.uint8, device=dev)
        else:
            self.vop = torch.zeros(L.pq3d_batch_rhs_bytes(N, B), dtype=torch.uint8, device=dev)
        self.ctrl_t = torch.zeros(B * ctypes.sizeof(_lib.RunCtrl), dtype=torch.uint8, device=dev)
        S = _lib.BatchSim()
        S.N, S.B, S.precision, S.nsplit, S.tc_ctas = N, B, prec, self.nsplit, self.tc_ctas
        for k in STATE + PARAMS + ("rates", "cand"):
            setattr(S, k, self.t[k].data_ptr())
        S.vop, S.ctrl = self.vop.data_ptr(), self.ctrl_t.data_ptr()
        S.base = self.t["base"].data_ptr() if "base" in self.t else None
        if precision == "bf16x18" and K.order is not None:
            S.fix_order, S.fix_pos = K.order.data_ptr(), K.pos.data_ptr()
        S.K = ctypes.addressof(self.hmat.H) if precision == "hmat" else self.K.data_ptr()
        S.V0, S.Vpl, S.eta, S.fix_Tn = float(V0), float(Vpl), float(mu) / (2.0 * float(Cs)), int(bool(fix_Tn))
        S.attempt64 = 0 if precision == "fp64" else {"mixed": 0, "fp64": 1, "ff": 2}[self.attempt]
        if shard is not None:
            S.N_total, S.cell0 = Nt, self.cell0
        self.S = S
        self.ws = torch.zeros(max(256, L.pq3d_batch_workspace_bytes(ctypes.byref(S))), dtype=torch.uint8, device=dev)
        self.set_ctrl(dttry=dttry, max_steps=max_steps, t_end=t_end)
        self.prepare()
        self.graph = None

    # -- control -----------------------------------------------------------
    def set_ctrl(self, dttry=1e-3, max_steps=2 ** 62, t_end=float("inf"), active=None):
        arr = (_lib.RunCtrl * self.B)()
        for r in range(self.B):
            c = arr[r]
            c.h, c.time, c.t_end = float(dttry), 0.0, float(t_end)
            c.max_steps = int(max_steps)
            c.active = 1 if active is None else int(bool(active[r]))
        host = torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8)
        self.ctrl_t.copy_(host)

    def read_ctrl(self):
        b = self.ctrl_t.cpu().numpy().tobytes()
        return list((_lib.RunCtrl * self.B).from_buffer_copy(b))

    def load_run(self, slot, table, *, dttry=1e-3, t_end=float("inf"), max_steps=2 ** 62, V0=1e-6, Vpl=1e-9):
        """Put a new run into `slot` (stream-ordered on the current stream):
        its initial state from the per-cell table, a fresh control record, and
        the operator right-hand side of every slot recomputed."""
        init = initial_state(np.asarray(table, dtype=np.float64), V0, Vpl)
        dev = self.device
        for k in STATE + ("a", "b", "dc", "f0", "shear_loading", "normal_loading"):
            self.t[k][slot].copy_(torch.as_tensor(init[k], dtype=torch.float64), non_blocking=False)
        r0 = torch.as_tensor(init["rake0"], dtype=torch.float64, device=dev)
        self.t["cos_rake0"][slot].copy_(torch.cos(r0))
        self.t["sin_rake0"][slot].copy_(torch.sin(r0))
        c = _lib.RunCtrl()
        c.h, c.time, c.t_end, c.max_steps, c.active = float(dttry), 0.0, float(t_end), int(max_steps), 1
        sz = ctypes.sizeof(_lib.RunCtrl)
        self.ctrl_t[slot * sz:(slot + 1) * sz].copy_(torch.frombuffer(bytearray(bytes(c)), dtype=torch.uint8))
        self.prepare()

    def deactivate(self, slot):
        c = _lib.RunCtrl()
        sz = ctypes.sizeof(_lib.RunCtrl)
        self.ctrl_t[slot * sz:(slot + 1) * sz].copy_(torch.frombuffer(bytearray(bytes(c)), dtype=torch.uint8))

    def traction_rates(self):
        """(B, 3N) FP64 traction rates K.v' of the last product: the FP32
        K-slice partials of the tensor-core product added, or the one FP64
        partial of the other products."""
        n = self.nsplit * self.Bp * 3 * self.N
        if self.precision == "bf16x18":
            f = self.t["rates"].view(torch.float32)[:2 * n].view(self.nsplit, self.Bp, 3 * self.N, 2).double()
            r = f.sum(3).sum(0)
            if self.fix_op.order is not None:   # rows come in the operator's cell order
                r = r.view(self.Bp, self.N, 3)[:, self.fix_op.pos].reshape(self.Bp, 3 * self.N)
        elif self.precision == "bf16x6":
            r = self.t["rates"].view(torch.float32)[:n].view(self.nsplit, self.Bp, 3 * self.N).double().sum(0)
        else:
            r = self.t["rates"][:n].view(self.nsplit, self.Bp, 3 * self.N).sum(0)
        return r[:self.B]

    def state_bytes(self):
        """Device bytes of the per-run state, rates, right-hand side and control."""
        return sum(t.numel() * t.element_size() for t in self.t.values()) + self.vop.numel() * self.vop.element_size() \
            + self.ctrl_t.numel() + self.ws.numel()

    def prepare(self):
        L = _lib.load()
        _lib.check(L.pq3d_batch_prepare(ctypes.byref(self.S), torch.cuda.current_stream(self.device).cuda_stream))

    # -- stepping ----------------------------------------------------------
    def iterate(self, n=1):
        """Queue n iterations (asynchronous)."""
        L = _lib.load()
        st = torch.cuda.current_stream(self.device).cuda_stream
        for _ in range(n):
            _lib.check(L.pq3d_batch_iterate(ctypes.byref(self.S), self.ws.data_ptr(), self.ws.numel(), st))

    def capture(self, n_iter):
        """Capture n_iter iterations into a CUDA graph (after one warm-up
        iteration has configured the kernels)."""
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.iterate(n_iter)
        self.graph = g
        self.graph_iters = n_iter
        return g

    def replay(self, times=1):
        for _ in range(times):
            self.graph.replay()

    # -- row-shard phases (driven by pyquake3d_gb300.shards) ----------------
    def begin(self):
        """Operator product of this shard's rows and one attempt (the runs'
        error norms of this shard are left in the control records)."""
        L = _lib.load()
        st = torch.cuda.current_stream(self.device).cuda_stream
        _lib.check(L.pq3d_batch_iterate_begin(ctypes.byref(self.S), self.ws.data_ptr(), self.ws.numel(), st))

    def end(self):
        """Accept/reject decision and update of this shard's cells."""
        L = _lib.load()
        _lib.check(L.pq3d_batch_iterate_end(ctypes.byref(self.S), torch.cuda.current_stream(self.device).cuda_stream))

    _ERR = _lib.RunCtrl.err1_bits.offset // 8

    def error_words(self):
        """(B, 2) int64: the FP64 bit patterns of the runs' error norms (err1,
        err2); MAX over shards of these words is MAX of the norms."""
        return self.ctrl_t.view(torch.int64).view(self.B, -1)[:, self._ERR:self._ERR + 2].clone()

    def set_error_words(self, w):
        self.ctrl_t.view(torch.int64).view(self.B, -1)[:, self._ERR:self._ERR + 2].copy_(w)

    def vprime(self):
        """(Bp, 2 N_total) view of v' of all cells (this shard writes columns
        [2 cell0, 2 (cell0 + N)))."""
        return self.vop.view(self.Bp, 2 * self.N_total)

    def error_word(self):
        return int(self.ws[:4].view(torch.int32).item())

    def stages(self):
        """Right-hand-side evaluations so far: 7 per attempted step, all runs."""
        return 7 * sum(c.attempts for c in self.read_ctrl())


def lockstep(ref: Ensemble, others: dict, max_steps: int, every: int = 5, bar: float = 1e-5,
             marks=(10, 25, 50, 100, 150, 200, 300, 400)) -> dict:
    """Step ``ref`` and the ensembles of ``others`` ({name: Ensemble}, the same
    runs in other arithmetics) in lockstep and measure how far each departs
    from ``ref`` in slip.

    Every iteration runs as its two halves (pq3d_batch_iterate_begin / _end);
    between them each other ensemble takes ``ref``'s error norms -- the hand-
    over that row shards use for their reduced norms -- so all take the same
    accept/reject decisions and step sizes and reach the same times, and the
    differences are the arithmetic's alone (left to their own step control,
    two arithmetics take different step sequences, and the Dormand-Prince
    tolerance of 1e-4 per step separates them far more than the arithmetic
    does).  Every ``every`` iterations the normwise relative slip error of
    each run, ||s - s_ref|| / ||s_ref|| over its (slip1, slip2), is taken;
    per name the result holds the accepted steps up to which the maximum over
    runs stays within ``bar`` ("steps_within"), the largest such error and
    slip-rate error within that window, the error at the ``marks`` step
    counts (None once a run forced to accept a step its own arithmetic would
    reject has gone non-finite) and the failed runs."""
    names = list(others)
    out = {k: {"steps_within": 0, "max_slip_err_within": 0.0, "max_slip_rate_err_within": 0.0,
               "slip_rel_err_at_steps": {}} for k in names}
    ok = {k: True for k in names}
    marks = [m for m in marks if m <= max_steps]
    done = False
    cr = ref.read_ctrl()
    for _ in range(40 * max_steps // every + 1):
        for _ in range(every):
            ref.begin()
            for k in names:
                others[k].begin()
            wr = ref.error_words()
            for k in names:
                others[k].set_error_words(wr)
            ref.end()
            for k in names:
                others[k].end()
        cr = ref.read_ctrl()
        steps = min(c.steps for c in cr)
        s_ref = torch.cat([ref.t["slip1"], ref.t["slip2"]], 1)
        v_ref = torch.cat([ref.t["slipv1"], ref.t["slipv2"]], 1)
        for k in names:
            e = others[k]
            s = torch.cat([e.t["slip1"], e.t["slip2"]], 1)
            v = torch.cat([e.t["slipv1"], e.t["slipv2"]], 1)
            es = ((s - s_ref).norm(dim=1) / s_ref.norm(dim=1)).max().item()
            ev = ((v - v_ref).norm(dim=1) / v_ref.norm(dim=1)).max().item()
            O = out[k]
            if ok[k] and es <= bar:
                O["steps_within"] = steps
                O["max_slip_err_within"] = max(O["max_slip_err_within"], es)
                O["max_slip_rate_err_within"] = max(O["max_slip_rate_err_within"], ev)
            else:
                ok[k] = False
            for m in marks:
                if steps >= m and str(m) not in O["slip_rel_err_at_steps"]:
                    O["slip_rel_err_at_steps"][str(m)] = es if es == es and es < float("inf") else None
        if done:
            break
        done = not any(c.active for c in cr)
    for k in names:
        out[k]["failed_runs"] = int(sum(c.status != 0 for c in others[k].read_ctrl()))
        if ok[k]:
            out[k]["steps_within"] = min(c.steps for c in cr)
    out["_ref"] = {"runs": ref.B, "accepted_steps": int(min(c.steps for c in cr)),
                   "rk_stages_per_run": int(7 * max(c.attempts for c in cr)),
                   "simulated_time_s": float(max(c.time for c in cr))}
    return out
