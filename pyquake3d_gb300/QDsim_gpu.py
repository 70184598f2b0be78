"""Drop-in for the dense simulator of PyQuake3D (``src/QDsim_gpu.py``).

``QDsim(elelst, nodelst, fnamePara)`` reads the same ``key: value`` parameter
file and the same per-cell parameter file, assembles the dense traction
operator on the GPU (FP64, plus an FP32 copy) and steps on the GPU:

* ``initGPUvariable()``          -- moves the state to the device
                                    (src/QDsim_gpu.py:893-940)
* ``simu_forwardGPU(dttry)``     -- one accepted step, returns (h, dtnext)
                                    (src/QDsim_gpu.py:942-1027)
* ``simu_forward(dttry)``        -- the same, and refreshes the host NumPy
                                    attributes the reference's CPU path keeps
                                    (src/QDsim_gpu.py:1029-1122)
* ``simu_forward_many(dttry, n)`` -- n accepted steps in one device launch

Device attributes keep the reference names with the ``_gpu`` suffix
(``slipv1_gpu``, ``Tno_gpu`` ...), as torch tensors.  Where the reference
exits (dt < 1e-15 or > 20 rejected attempts, src/QDsim_gpu.py:983-985) this
raises :class:`StepError`.

Supported inputs: per-cell parameter files (``InputHetoparamter: True``,
layout of src/QDsim_gpu.py:714-770), full- or half-space (``Half space``),
pore-pressure dilatancy (``If Dilatancy``; dense stepper).  Other
parameter-file options raise ``NotImplementedError`` rather than silently
computing something else.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np
import torch

from . import _lib, gf
from .mesh import element_frames

OPS = gf.OPS


class StepError(RuntimeError):
    """The step-size control failed (dt < 1e-15 or more than 20 rejections)."""


def readPara0(fname):
    """``key: value`` parameter file -> dict of stripped strings (src/QDsim_gpu.py:90-99)."""
    para = {}
    with open(fname) as f:
        for line in f:
            if ":" in line:
                k, v = line.split(":", 1)
                para[k.strip()] = v.strip()
    return para


def initial_state(table, V0, Vpl, P=None):
    """Initial state from a per-cell table (src/QDsim_gpu.py:714-770).

    Setup only (once per run, host side).  Returns a dict of NumPy arrays."""
    N = table.shape[0]
    P = np.zeros(N) if P is None else P
    slipvC = np.ones(N) * Vpl
    s = {}
    s["rake"] = table[:, 0].copy()
    s["a"] = table[:, 1].copy()
    s["b"] = table[:, 2].copy()
    s["dc"] = table[:, 3].copy()
    s["f0"] = table[:, 4].copy()
    s["Tno"] = table[:, 6].copy()
    s["slipv"] = table[:, 7].copy()
    s["shear_loading"] = table[:, 8].copy()
    s["normal_loading"] = table[:, 9].copy()
    x = np.cos(s["rake"])
    y = np.sin(s["rake"])
    s["slipv1"] = s["slipv"] * x + 1e-16
    s["slipv2"] = s["slipv"] * y + 1e-16
    a, b, f0, Tno = s["a"], s["b"], s["f0"], s["Tno"]
    Tt = (Tno - P * 1e-6) * a * np.arcsinh(s["slipv"] / (2.0 * V0) * np.exp((f0 + b * np.log(V0 / slipvC)) / a))
    s["Tt"] = Tt
    s["Tt1o"] = Tt * x
    s["Tt2o"] = Tt * y
    s["fric"] = Tt / (Tno - P * 1e-6)
    s["state"] = np.log(np.sinh(Tt / (Tno - P * 1e-6) / a) * 2.0 * V0 / s["slipv"]) * a
    s["rake0"] = s["rake"].copy()
    s["slip1"] = np.zeros(N)
    s["slip2"] = np.zeros(N)
    s["slip"] = np.zeros(N)
    return s


STATE_FIELDS = ("Tno", "Tt1o", "Tt2o", "state", "slipv1", "slipv2", "slipv", "rake", "slip1", "slip2", "slip",
                "Tt", "fric")
PARAM_FIELDS = ("a", "b", "dc", "f0", "shear_loading", "normal_loading", "rake0")


DILATANCY_KEYS = ("Dilatancy coefficient", "Hydraulic diffusivity", "Actively shearing zone thickness",
                  "Effective compressibility", "Constant porepressure", "Initial porepressure")


def dilatancy_depths(num=60, c=1e-2):
    """Fault-normal nodes of the pore-pressure profile (src/QDsim_gpu.py:342-343)."""
    yp = np.logspace(start=-3, stop=10, num=num, base=10)
    return np.log(1 + yp / c)


class DenseDeviceSim:
    """Device state of one dense simulation + the launch structure of
    ``pq3d_dense_step``.  ``K`` is the (3N, 2N) FP64 or FP32 operator.
    ``dilatancy``: None, or a dict of the parameter-file values
    (DILATANCY_KEYS, pressures in MPa) -- pore pressure P (initial value,
    also in ``init``'s initial state) and the per-cell diffusion profile."""

    def __init__(self, K, init, *, mu, Cs, V0, Vpl, fix_Tn=False, dttry=1e-3, device=None, dilatancy=None):
        self.device = K.device if device is None else device
        N = K.shape[1] // 2
        self.N = N
        self.K = K
        dev = self.device
        f64 = torch.float64
        self.t = {}
        for name in STATE_FIELDS + PARAM_FIELDS:
            self.t[name] = torch.as_tensor(np.ascontiguousarray(init[name], dtype=np.float64), device=dev).clone()
        self.t["rates"] = torch.zeros(3 * N, dtype=f64, device=dev)
        self.t["vprime"] = torch.zeros(2 * N, dtype=f64, device=dev)
        self.t["cand"] = torch.zeros(4 * N, dtype=f64, device=dev)
        self.ctrl_t = torch.zeros(ctypes.sizeof(_lib.StepCtrl), dtype=torch.uint8, device=dev)
        self.V0, self.Vpl, self.eta = float(V0), float(Vpl), float(mu) / (2.0 * float(Cs))
        self.fix_Tn = bool(fix_Tn)
        self.set_ctrl(dttry=dttry, time=0.0)
        S = _lib.DenseSim()
        S.N = N
        for name in STATE_FIELDS + PARAM_FIELDS + ("rates", "vprime", "cand"):
            setattr(S, name, self.t[name].data_ptr())
        if K.dtype == torch.float64:
            S.K64, S.K32 = K.data_ptr(), None
        elif K.dtype == torch.float32:
            S.K64, S.K32 = None, K.data_ptr()
        else:
            raise TypeError("operator must be float64 or float32")
        S.ctrl = self.ctrl_t.data_ptr()
        S.V0, S.Vpl, S.eta, S.fix_Tn = self.V0, self.Vpl, self.eta, int(self.fix_Tn)
        if dilatancy is not None:
            L = _lib.load()
            z = dilatancy_depths()
            nd = len(z) - 1
            P0 = float(dilatancy["Constant porepressure"]) * 1e6
            Pin = float(dilatancy["Initial porepressure"]) * 1e6
            tab = np.zeros(L.pq3d_dilatancy_table_len(nd))
            _lib.check(L.pq3d_dilatancy_table(z.ctypes.data, nd, float(dilatancy["Hydraulic diffusivity"]),
                                              float(dilatancy["Dilatancy coefficient"]),
                                              float(dilatancy["Actively shearing zone thickness"]),
                                              float(dilatancy["Effective compressibility"]), P0, tab.ctypes.data))
            self.t["dila"] = torch.as_tensor(tab, device=dev)
            self.t["P"] = torch.full((N,), Pin, dtype=f64, device=dev)
            self.t["dPdt"] = torch.zeros(N, dtype=f64, device=dev)
            self.t["Parr"] = torch.full((nd + 1, N), Pin, dtype=f64, device=dev)   # [depth node][cell]
            S.ndepth = nd
            S.P, S.dPdt, S.Parr, S.dila = (self.t[k].data_ptr() for k in ("P", "dPdt", "Parr", "dila"))
        self.S = S

    def set_ctrl(self, dttry, time):
        c = _lib.StepCtrl()
        c.dttry, c.time, c.status = float(dttry), float(time), 0
        host = torch.frombuffer(bytearray(bytes(c)), dtype=torch.uint8)
        self.ctrl_t.copy_(host)

    def read_ctrl(self):
        b = self.ctrl_t.cpu().numpy().tobytes()
        return _lib.StepCtrl.from_buffer_copy(b)

    def launch(self, nsteps, h_hist=None, t_hist=None, h_force=None, stream=None):
        """Queue nsteps accepted steps (asynchronous)."""
        L = _lib.load()
        st = torch.cuda.current_stream(self.device).cuda_stream if stream is None else stream
        rc = L.pq3d_dense_step(ctypes.byref(self.S), int(nsteps),
                               h_hist.data_ptr() if h_hist is not None else None,
                               t_hist.data_ptr() if t_hist is not None else None,
                               h_force.data_ptr() if h_force is not None else None, st)
        _lib.check(rc)

    def step(self, nsteps=1, h_force=None):
        """nsteps accepted steps; returns (h[n], t[n], ctrl) on the host.
        ``h_force`` (sequence of nsteps step sizes) replays a step sequence."""
        dev = self.device
        h = torch.empty(nsteps, dtype=torch.float64, device=dev)
        t = torch.empty(nsteps, dtype=torch.float64, device=dev)
        hf = None
        if h_force is not None:
            hf = torch.as_tensor(np.asarray(h_force, dtype=np.float64)[:nsteps], device=dev).contiguous()
            assert hf.numel() == nsteps
        self.launch(nsteps, h, t, hf)
        c = self.read_ctrl()
        if c.status == _lib.PQ3D_ERR_STEP:
            raise StepError("error: dt is too small (after %d accepted steps)" % c.steps_done)
        if c.status != _lib.PQ3D_OK:
            raise _lib.PQ3DError(c.status, "stepper status %d" % c.status)
        return h.cpu().numpy(), t.cpu().numpy(), c


class QDsim:
    """Dense quasi-dynamic simulator with the reference's constructor and
    stepping API (src/QDsim_gpu.py:119-1122)."""

    def __init__(self, elelst, nodelst, fnamePara, device=None, operator_dtype=torch.float64):
        i = fnamePara.rfind("/")
        self.dirname = fnamePara[:i] if i != -1 else fnamePara
        self.Para0 = readPara0(fnamePara)
        self.elelst = np.asarray(elelst, dtype=np.int64)
        self.nodelst = np.asarray(nodelst, dtype=np.float64)
        self.eleVec, self.xg = element_frames(self.nodelst, self.elelst)
        P = self.Para0
        self.mu = float(P["Shear modulus"])
        self.lambda_ = float(P["Lame constants"])
        self.density = float(P["Rock density"])
        self.htry = 1e-3
        self.Cs = np.sqrt(self.mu / self.density)
        self.time = 0
        self.halfspace_jud = P.get("Half space", "False") == "True"
        self.InputHetoparamter = P.get("InputHetoparamter", "False") == "True"
        self.Ifdila = P.get("If Dilatancy", "False") == "True"
        self.fix_Tn = P.get("Fix_Tn", "False") == "True"
        self.V0 = float(P["Reference slip rate"])
        self.Vpl_con = float(P["Plate loading rate"])
        if not self.InputHetoparamter:
            raise NotImplementedError("only per-cell parameter files (InputHetoparamter: True) are supported")
        self.device = torch.device(device) if device is not None else torch.device("cuda")
        self.operator_dtype = operator_dtype
        self.read_parameter(P["Inputparamter file"])
        self.calc_corefunc()

    def read_parameter(self, fname):
        path = fname if os.path.isabs(fname) else os.path.join(self.dirname, fname)
        values = np.loadtxt(path, ndmin=2)
        N = self.eleVec.shape[0]
        # pore pressure (Pa): the initial value with dilatancy, else 0 (src/QDsim_gpu.py:332-348)
        self.dilatancy = {k: float(self.Para0[k]) for k in DILATANCY_KEYS} if self.Ifdila else None
        self.P = np.ones(N) * self.dilatancy["Initial porepressure"] * 1e6 if self.Ifdila else np.zeros(N)
        self.init = initial_state(values[:N], self.V0, self.Vpl_con, P=self.P)
        for k, v in self.init.items():
            setattr(self, k, v.copy())
        self.maxslipv0 = np.max(self.slipv)

    def calc_corefunc(self):
        """Load the six operators from the cache directory when all six .npy
        files exist, else assemble on the GPU (src/QDsim_gpu.py:188-245)."""
        d = self.Para0.get("Corefunc directory")
        cached = d is not None and all(os.path.exists(os.path.join(d, k + ".npy")) for k in OPS)
        if cached:
            ops = {k: np.load(os.path.join(d, k + ".npy")) for k in OPS}
            K64 = torch.as_tensor(gf.join_ops(ops), device=self.device)
            K32 = K64.float()
        else:
            K64, K32 = gf.assemble_dense(self.nodelst, self.elelst, self.mu, self.lambda_,
                                         halfspace=self.halfspace_jud, device=self.device)
            if d is not None and self.Para0.get("save Corefunc", "False") == "True":
                os.makedirs(d, exist_ok=True)
                for k, v in gf.split_ops(K64).items():
                    np.save(os.path.join(d, k), v.cpu().numpy())
        self.K64, self.K32 = K64, K32

    def ops(self):
        """The six reference matrices as device views."""
        return gf.split_ops(self.K64)

    def initGPUvariable(self):
        K = self.K64 if self.operator_dtype == torch.float64 else self.K32
        self.dev = DenseDeviceSim(K, self.init, mu=self.mu, Cs=self.Cs, V0=self.V0, Vpl=self.Vpl_con,
                                  fix_Tn=self.fix_Tn, dttry=self.htry, device=self.device, dilatancy=self.dilatancy)
        for k, v in self.dev.t.items():
            setattr(self, k + "_gpu", v)

    def simu_forwardGPU(self, dttry):
        h, dtnext = self.simu_forward_many(dttry, 1)
        return float(h[0]), dtnext

    def simu_forward_many(self, dttry, nsteps):
        """nsteps accepted steps; returns (h per step, dtnext)."""
        if not hasattr(self, "dev"):
            self.initGPUvariable()
        self.dev.set_ctrl(dttry=dttry, time=self.time)
        h, t, c = self.dev.step(nsteps)
        self.time = c.time
        self.maxslipv0 = c.maxv
        return h, c.dttry

    def simu_forward(self, dttry):
        h, dtnext = self.simu_forwardGPU(dttry)
        for k in STATE_FIELDS:
            setattr(self, k, self.dev.t[k].cpu().numpy())
        return h, dtnext

    def ouputVTK(self, fname):
        """Snapshot as legacy VTK (the reference's method name, fields and
        layout, src/QDsim_gpu.py:1927-2073): the device state is staged into
        one pinned host buffer by a single copy, then written."""
        import torch
        from .mesh import write_vtk
        if hasattr(self, "dev"):
            keys = STATE_FIELDS + ("a", "b", "dc")
            staged = torch.stack([self.dev.t[k] for k in keys])
            host = torch.empty(staged.shape, dtype=staged.dtype, pin_memory=True)
            host.copy_(staged)
            fields = {k: host[i].numpy() for i, k in enumerate(keys)}
        else:
            fields = {k: np.asarray(getattr(self, k)) for k in STATE_FIELDS + ("a", "b", "dc")}
        write_vtk(fname, self.nodelst, self.elelst, fields)
