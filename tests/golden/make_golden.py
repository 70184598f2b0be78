"""Generate the golden fixtures under tests/golden/ from the reference itself.

Run in a checkout where the reference tree is available (default
/root/reference, override with PQ3D_REFERENCE):

    python tests/golden/make_golden.py

What it records:
  gf_kat.npz        inputs and outputs of the reference C-ABI TDstressFS_C and
                    TDstressEachSourceAtReceiver_C (built from
                    src/TDstressFS_C.cpp by oracle/Makefile `ref`) on random
                    and hand-picked geometries: far and near field, self terms
                    (centroids), receivers on in-plane side lines, steep and
                    dipping sources; full- and half-space.
  dense_small.npz   the six traction operators A1s..Bd the reference Python
                    assembles (QDsim_gpu.get_coreAB_mulproess, pure NumPy GF)
                    for a small planar and a small rough mesh.
  traj_small.npz    a stepping trajectory of the reference CPU path
                    (QDsim_gpu.simu_forward, src/QDsim_gpu.py:1029-1122) on the
                    small planar mesh: step sizes, times and the state at
                    checkpoints.
  traj_config1.npz  the same for the planar N = 1,600 workload (40 x 20 km
                    vertical strike-slip fault, 1 km squares, velocity-
                    weakening rectangle, 4 x 4 km nucleation square at
                    0.03 m/s): 300 accepted steps (``--config1-only``).

The reference Python imports matplotlib, mpi4py, h5py, pyvista and vtk, which
are not installed; empty stand-in modules are injected into sys.modules before
importing it.  Nothing here runs at test time.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("PQ3D_REFERENCE", "/root/reference")
sys.path.insert(0, REPO)

from pyquake3d_gb300 import mesh  # noqa: E402

MU = 32038120320.0
LAM = 32038120320.0
D = ctypes.POINTER(ctypes.c_double)


def _ptr(a):
    return a.ctypes.data_as(D)


def load_ref_lib():
    subprocess.check_call(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref",
                           "REF_SRC=" + os.path.join(REF, "src", "TDstressFS_C.cpp")])
    lib = ctypes.CDLL(os.path.join(REPO, "oracle", "_ref", "libTDstressFS_ref.so"))
    lib.TDstressFS_C.argtypes = [D, D, D, ctypes.c_size_t, D, D, D] + [ctypes.c_double] * 5 + [ctypes.c_bool, D, D]
    lib.TDstressFS_C.restype = None
    lib.TDstressEachSourceAtReceiver_C.argtypes = [ctypes.c_double] * 3 + [D, D, D, ctypes.c_size_t] + \
        [ctypes.c_double] * 5 + [ctypes.c_bool, D, D]
    lib.TDstressEachSourceAtReceiver_C.restype = None
    return lib


def gf_cases(rng):
    """(P1, P2, P3, receivers[n,3], Ss, Ds, Ts, halfspace) cases."""
    cases = []
    for k in range(24):
        # random source triangle at depth, random orientation
        c = np.array([0.0, 0.0, -8000.0]) + rng.normal(size=3) * [2000, 2000, 1000]
        P = c + rng.normal(size=(3, 3)) * 800
        far = c + rng.normal(size=(12, 3)) * 6000
        near = c + rng.normal(size=(12, 3)) * 300
        cen = P.mean(axis=0)[None, :]
        R = np.concatenate([far, near, cen])
        R[:, 2] = np.minimum(R[:, 2], -10.0)
        half = bool(k % 3 == 2)
        if half:
            P[:, 2] = np.minimum(P[:, 2], -50.0)
        Ss, Ds, Ts = [(1.0, 0.0, 0.0), (0.0, 1.0, 0.0), (0.3, -0.7, 0.2)][k % 3]
        cases.append((P[0], P[1], P[2], R, Ss, Ds, Ts, half))
    # steep (vertical) and gently dipping sources, with in-plane side-line receivers
    for dip in (90.0, 60.0, 15.0):
        d = np.deg2rad(dip)
        P1 = np.array([0.0, 0.0, -5000.0])
        P2 = P1 + [1000.0, 0.0, 0.0]
        P3 = P1 + [300.0, 1000.0 * np.cos(d), -1000.0 * np.sin(d)]
        # points on the line through P1, P2 (in-plane, outside the triangle)
        on_line = np.stack([P1 + t * (P2 - P1) for t in (-0.5, 1.5, 2.0)])
        inside = np.stack([(P1 + P2 + P3) / 3.0, 0.6 * P1 + 0.2 * P2 + 0.2 * P3])
        off = (P1 + P2 + P3) / 3.0 + np.array([[0, 0, 0], [100, 100, -100], [-3000, 2000, -2000]])
        R = np.concatenate([on_line, inside, off])
        for (Ss, Ds) in ((1.0, 0.0), (0.0, 1.0)):
            cases.append((P1, P2, P3, R, Ss, Ds, 0.0, False))
    # exactly representable vertical triangle in the x-z plane: receivers on its
    # edges and vertices are in-plane side-line points (configuration 0)
    P1 = np.array([0.0, 0.0, -5000.0])
    P2 = np.array([1000.0, 0.0, -5000.0])
    P3 = np.array([400.0, 0.0, -4000.0])
    R = np.array([[500.0, 0.0, -5000.0], [200.0, 0.0, -4500.0], [700.0, 0.0, -4500.0],
                  [1500.0, 0.0, -5000.0], [300.0, 0.0, -4700.0], [300.0, 50.0, -4700.0]])
    for (Ss, Ds) in ((1.0, 0.0), (0.0, 1.0)):
        cases.append((P1, P2, P3, R, Ss, Ds, 0.0, False))
    # the reference's own smoke inputs (src/TDstressFS_C.cpp:2035-2078): half-space
    R = np.array([[29387.75593897, 0., -38297.33922684],
                  [-48489.89772099, 0., -37991.33142056],
                  [-48479.08845632, 0., -14039.49925884]])
    cases.append((np.array([48120.9759287, 0., -6947.86435537]),
                  np.array([49133.9746038, 0., -7500.00001313]),
                  np.array([49133.97459622, 0., -6500.]), R, 1.0, 0.5, 0.0, True))
    return cases


def make_gf_kat(lib, rng):
    out = {"n_cases": 0}
    cases = gf_cases(rng)
    for i, (P1, P2, P3, R, Ss, Ds, Ts, half) in enumerate(cases):
        R = np.ascontiguousarray(R, dtype=np.float64)
        n = R.shape[0]
        x, y, z = (np.ascontiguousarray(R[:, k]) for k in range(3))
        s = np.zeros((n, 6))
        e = np.zeros((n, 6))
        P1c, P2c, P3c = (np.ascontiguousarray(p, dtype=np.float64) for p in (P1, P2, P3))
        lib.TDstressFS_C(_ptr(x), _ptr(y), _ptr(z), n, _ptr(P1c), _ptr(P2c), _ptr(P3c),
                         Ss, Ds, Ts, MU, LAM, half, _ptr(s), _ptr(e))
        out[f"c{i}_P"] = np.stack([P1c, P2c, P3c])
        out[f"c{i}_R"] = R
        out[f"c{i}_b"] = np.array([Ss, Ds, Ts, float(half)])
        out[f"c{i}_stress"] = s
        out[f"c{i}_strain"] = e
    out["n_cases"] = len(cases)
    # one receiver, many sources
    nodes, tris = mesh.rough_fault(6.0, 3.0, 6, 3, seed=3)
    P1 = np.ascontiguousarray(nodes[tris[:, 0] - 1])
    P2 = np.ascontiguousarray(nodes[tris[:, 1] - 1])
    P3 = np.ascontiguousarray(nodes[tris[:, 2] - 1])
    ns = P1.shape[0]
    recv = np.array([120.0, 35.0, -1400.0])
    for half in (False, True):
        s = np.zeros((ns, 6))
        e = np.zeros((ns, 6))
        lib.TDstressEachSourceAtReceiver_C(recv[0], recv[1], recv[2], _ptr(P1), _ptr(P2), _ptr(P3), ns,
                                           0.0, 1.0, 0.0, MU, LAM, half, _ptr(s), _ptr(e))
        out[f"each_h{int(half)}_stress"] = s
        out[f"each_h{int(half)}_strain"] = e
    out["each_P1"], out["each_P2"], out["each_P3"], out["each_recv"] = P1, P2, P3, recv
    np.savez_compressed(os.path.join(HERE, "gf_kat.npz"), **out)
    print("gf_kat.npz:", out["n_cases"], "cases")


def import_reference_python():
    """Import the reference's Python with stand-ins for absent packages."""
    for name in ("matplotlib", "matplotlib.pyplot", "matplotlib.colors", "h5py", "pyvista", "vtk"):
        m = types.ModuleType(name)
        if name == "matplotlib.pyplot":
            m.rcParams = {}
            m.rcParams = types.SimpleNamespace(update=lambda *a, **k: None)
        if name == "matplotlib.colors":
            m.ListedColormap = object
        sys.modules[name] = m
    sys.modules["matplotlib"].pyplot = sys.modules["matplotlib.pyplot"]
    sys.modules["matplotlib"].colors = sys.modules["matplotlib.colors"]
    mpi = types.ModuleType("mpi4py")

    class _Comm:
        def Get_rank(self):
            return 0

        def Get_size(self):
            return 1

    mpi.MPI = types.SimpleNamespace(COMM_WORLD=_Comm())
    sys.modules["mpi4py"] = mpi
    sys.path.insert(0, os.path.join(REF, "src"))
    import QDsim_gpu  # noqa: F401
    return QDsim_gpu


PARAM_TXT = """Corefunc directory: {core}
save Corefunc: True
Node_order: False
Scale_km: True
Max_thread workers: 2
Batch_size: 1000
GPU:False
Lame constants: {lam}
Shear modulus: {mu}
Rock density: {rho}
InputHetoparamter: True
Inputparamter file: cells.dat
If Dilatancy:{dila}
Dilatancy coefficient: 3e-4
Hydraulic diffusivity: 1e-5
Actively shearing zone thickness: 3e-3
Effective compressibility: 8e-11
Constant porepressure: 2
Initial porepressure: 2
Half space: {half}
Fix_Tn:False
ssv_scale: 1.0
ssh1_scale: 1.6
ssh2_scale: 0.6
Angle between ssh1 and X-axis: 30
Vertical principal stress value: 2.5e7
Vertical principal stress value varies with depth: False
Turnning depth: 15000
Shear traction solved from stress tensor: False
Normal traction solved from stress tensor: False
Rake solved from stress tensor: False
Fix_rake: 0
Widths of VS region: 10000
Widths of surface VS region: 2000
Transition region from VS to VW region: 2000
Reference slip rate: 1e-6
Reference friction coefficient: 0.6
Plate loading rate: 1e-9
"""

RHO = MU / 3464.0 ** 2  # cs = 3.464 km/s


def reference_sim(QDsim_gpu, nodes, tris, table, workdir, half=False, dila=False):
    core = os.path.join(workdir, "core")
    with open(os.path.join(workdir, "parameter.txt"), "w") as f:
        f.write(PARAM_TXT.format(core=core, lam=LAM, mu=MU, rho=RHO, half="True" if half else "False",
                                 dila="True" if dila else "False"))
    mesh.write_parameter_file(os.path.join(workdir, "cells.dat"), table)
    cwd = os.getcwd()
    os.chdir(workdir)
    try:
        sim = QDsim_gpu.QDsim(tris, nodes, os.path.join(workdir, "parameter.txt"))
    finally:
        os.chdir(cwd)
    return sim


def make_hmatrix_golden(nodes, tris, mini_leaf, seed=0):
    """Leaf blocks of the reference's H-matrix (src/Hmatrix.py:2147-2196) and
    its ACA products for one seeded x, from a scratch directory whose
    src/TDstressFS_C.so is the reference built from source."""
    import shutil
    out = {}
    with tempfile.TemporaryDirectory() as td:
        os.mkdir(os.path.join(td, "src"))
        shutil.copy(os.path.join(REPO, "oracle", "_ref", "libTDstressFS_ref.so"), os.path.join(td, "src", "TDstressFS_C.so"))
        cwd = os.getcwd()
        os.chdir(td)
        try:
            import Hmatrix
            import readmsh
            eleVec, xg = readmsh.get_eleVec(nodes, tris, False)
            para = {"GPU": False, "Shear modulus": MU, "Lame constants": LAM, "Half space": False,
                    "Hmatrix_mpi_plot": False, "Using C++ green function": True}
            tree = Hmatrix.createHmatrix(xg, nodes, tris, eleVec, para, mini_leaf=mini_leaf)
            np.random.seed(seed)
            # calc_Hmatrix_ACA collects the leaf blocks itself (src/Hmatrix.py:1603-1616)
            blocks = tree.calc_Hmatrix_ACA(td, save_corefunc=False)
            rows = [np.asarray(b.row_cluster, dtype=np.int64) for b in blocks]
            cols = [np.asarray(b.col_cluster, dtype=np.int64) for b in blocks]
            out["row_ptr"] = np.cumsum([0] + [len(r) for r in rows])
            out["col_ptr"] = np.cumsum([0] + [len(c) for c in cols])
            out["rows"] = np.concatenate(rows)
            out["cols"] = np.concatenate(cols)
            x = np.random.default_rng(seed).standard_normal(len(xg))
            out["x"] = x
            for typ in ("A1s", "A2s", "Bs", "A1d", "A2d", "Bd"):
                out["y_" + typ] = tree.blocks_process_MVM(x, blocks, typ)
            out["aca"] = np.array([bool(getattr(b, "judaca", False)) for b in blocks])
        finally:
            os.chdir(cwd)
    out["nodes"], out["tris"], out["mini_leaf"] = nodes, tris, mini_leaf
    return out


def main_hmatrix_only():
    import_reference_python()
    nodes, tris = mesh.rough_fault(24.0, 12.0, 40, 20, seed=2, ratio=5e-3)
    hm = make_hmatrix_golden(nodes, tris, mini_leaf=32)
    np.savez_compressed(os.path.join(HERE, "hmatrix_small.npz"), **hm)
    print("hmatrix_small.npz: %d leaf blocks, %d ACA" % (len(hm["row_ptr"]) - 1, int(hm["aca"].sum())))


def dipping_fault(dip_deg=60.0):
    """8 x 4 km planar fault dipping dip_deg, 1 km cells, top edge on the free
    surface -> N = 64."""
    nodes, tris = mesh.planar_fault(8.0, 4.0, 8, 4)
    nodes = nodes.copy()
    nodes[:, 1] = nodes[:, 2] / np.tan(np.radians(dip_deg))
    return nodes, tris


def _hs_reference_ops(lib, nodes, tris, ev, xg):
    """Dense half-space traction operators from the reference C++
    TDstressFS_C (jud_halfspace), projected as QDsim_gpu.GetTtstress does."""
    N = tris.shape[0]
    X, Y, Z = (np.ascontiguousarray(xg[:, q]) for q in range(3))
    cpp = {k: np.zeros((N, N)) for k in ("A1s", "A2s", "Bs", "A1d", "A2d", "Bd")}
    for j in range(N):
        P = [np.ascontiguousarray(nodes[tris[j, q] - 1]) for q in range(3)]
        for sl, (Ss, Ds) in (("s", (1.0, 0.0)), ("d", (0.0, 1.0))):
            st = np.zeros((N, 6))
            sn = np.zeros((N, 6))
            lib.TDstressFS_C(_ptr(X), _ptr(Y), _ptr(Z), N, _ptr(P[0]), _ptr(P[1]), _ptr(P[2]), Ss, Ds, 0.0, MU, LAM,
                             True, _ptr(st), _ptr(sn))
            S = np.stack([np.stack([st[:, 0], st[:, 3], st[:, 4]], 1), np.stack([st[:, 3], st[:, 1], st[:, 5]], 1),
                          np.stack([st[:, 4], st[:, 5], st[:, 2]], 1)], 1)
            t = np.einsum("nij,nj->ni", S, ev[:, 6:9])
            cpp["A1" + sl][:, j] = np.einsum("ni,ni->n", t, ev[:, 0:3])
            cpp["A2" + sl][:, j] = np.einsum("ni,ni->n", t, ev[:, 3:6])
            cpp["B" + sl][:, j] = np.einsum("ni,ni->n", t, ev[:, 6:9])
    return cpp


def main_halfspace_only():
    """Half-space dense operators: a dipping fault reaching the surface, from
    the reference's own dense path (QDsim_gpu.get_coreAB_mulproess with
    "Half space: True", NumPy GF) and from the reference C++ TDstressFS_C
    (jud_halfspace); and a rough vertical fault reaching the surface (C++),
    whose near-vertical sides make the formula ill-conditioned."""
    lib = load_ref_lib()
    QDsim_gpu = import_reference_python()
    nodes, tris = dipping_fault()
    _, xg = mesh.element_frames(nodes, tris)
    table = mesh.friction_table(xg, 8e3, 4e3, v_nuc=1e-3, seed=0)
    out = {"nodes": nodes, "tris": tris, "mu": MU, "lam": LAM}
    with tempfile.TemporaryDirectory() as td:
        sim = reference_sim(QDsim_gpu, nodes, tris, table, td, half=True)
        for k in ("A1s", "A2s", "Bs", "A1d", "A2d", "Bd"):
            out["py_" + k] = getattr(sim, k)
        ev, xgr = sim.eleVec, sim.xg
    cpp = _hs_reference_ops(lib, nodes, tris, ev, xgr)
    for k, v in cpp.items():
        out["cpp_" + k] = v
    d = max(np.abs(out["py_" + k] - cpp[k]).max() / np.abs(cpp[k]).max() for k in cpp)
    # rough vertical fault, 6 x 3 km, 0.75 km cells -> N = 64, top edge at z = 0
    rn, rt = mesh.rough_fault(6.0, 3.0, 8, 4, seed=3)
    frames, rxg = mesh.element_frames(rn, rt)
    for k, v in _hs_reference_ops(lib, rn, rt, frames, rxg).items():
        out["rough_cpp_" + k] = v
    out["rough_nodes"], out["rough_tris"] = rn, rt
    # 40-digit values of the 8 entries where the oracle and the reference C++
    # disagree most (ill-conditioned pairs): the yardstick for FP64 evaluations
    import oracle
    from pyquake3d_gb300.gf import join_ops
    from tests.hs_highprec import fsc_strain
    ref = join_ops({k: out["rough_cpp_" + k] for k in oracle.OPS})
    orc = join_ops(dict(zip(oracle.OPS, oracle.assemble_dense(rn, rt, MU, LAM, halfspace=True))))
    idx = np.argsort(np.abs(orc - ref).ravel())[-8:]
    vals = []
    for flat in idx:
        r, c = divmod(int(flat), ref.shape[1])
        i, j, comp, slip = r // 3, c // 2, r % 3, c % 2
        P = [rn[rt[j, q] - 1] for q in range(3)]
        x = rxg[i]
        Ss, Ds = (1.0, 0.0) if slip == 0 else (0.0, 1.0)
        X = (x[:1].copy(), x[1:2].copy(), x[2:3].copy())
        _, e_fs = oracle.tdstress(*X, *P, Ss, Ds, 0.0, MU, LAM, False)
        Q = [np.array([p[0], p[1], -p[2]]) for p in P]
        _, e_im = oracle.tdstress(*X, *Q, Ss, Ds, 0.0, MU, LAM, False)
        e = e_fs[0] + e_im[0] + fsc_strain(*P, Ss, Ds, 0.0, x)
        tr = e[0] + e[1] + e[2]
        S = 2 * MU * np.array([[e[0], e[3], e[4]], [e[3], e[1], e[5]], [e[4], e[5], e[2]]]) + LAM * tr * np.eye(3)
        n = frames[i, 6:9]
        t = S @ n
        vals.append([t @ frames[i, 0:3], t @ frames[i, 3:6], t @ n][comp])
    out["rough_true_idx"] = idx.astype(np.int64)
    out["rough_true_val"] = np.array(vals)
    np.savez_compressed(os.path.join(HERE, "hs_dense_small.npz"), **out)
    print("hs_dense_small.npz: N = %d, reference NumPy vs C++ max rel %.2e" % (tris.shape[0], d))


DILA = {"Dilatancy coefficient": 3e-4, "Hydraulic diffusivity": 1e-5, "Actively shearing zone thickness": 3e-3,
        "Effective compressibility": 8e-11, "Constant porepressure": 2.0, "Initial porepressure": 2.0}


def main_dilatancy_only():
    """The reference CPU stepper with pore-pressure dilatancy (If Dilatancy:
    True, the parameter values of PARAM_TXT) on the planar N=64 mesh: 200
    accepted steps with checkpoints of the state, P and dPdt."""
    QDsim_gpu = import_reference_python()
    nodes, tris = mesh.planar_fault(8.0, 4.0, 8, 4)
    _, xg = mesh.element_frames(nodes, tris)
    table = mesh.friction_table(xg, 8e3, 4e3, v_nuc=3e-2, seed=0)   # fast nucleation: dilatant weakening
    out = {"nodes": nodes, "tris": tris, "table": table, "mu": MU, "rho": RHO}
    for k, v in DILA.items():
        out["dila_" + k.replace(" ", "_")] = v
    with tempfile.TemporaryDirectory() as td:
        sim = reference_sim(QDsim_gpu, nodes, tris, table, td, dila=True)
        out["P_init"] = np.array(sim.P)
        out["state_init"] = np.array(sim.state)
        hs, ts = [], []
        dttry = sim.htry
        for i in range(200):
            h, dttry = sim.simu_forward(dttry)
            hs.append(h)
            ts.append(sim.time)
            if (i + 1) in (1, 10, 50, 100, 200):
                for k in ("Tno", "Tt1o", "state", "slipv", "slip1", "P", "dPdt0"):
                    out[f"s{i + 1}_{k}"] = np.array(getattr(sim, k))
        out["h"], out["t"] = np.array(hs), np.array(ts)
        out["Parr_200"] = np.array(sim.Parr)
    np.savez_compressed(os.path.join(HERE, "traj_dila.npz"), **out)
    print("traj_dila.npz: t_end = %.6e s, P range %.6e .. %.6e" % (ts[-1], out["s200_P"].min(), out["s200_P"].max()))


def main_config1_only():
    """The reference CPU stepping on the N = 1,600 planar workload: 300
    accepted steps from the reference's own dense operators (its Python GF)."""
    QDsim_gpu = import_reference_python()
    nodes, tris = mesh.planar_fault(40.0, 20.0, 40, 20)
    _, xg = mesh.element_frames(nodes, tris)
    table = mesh.friction_table(xg, 40e3, 20e3, seed=0)
    out = {"nodes": nodes, "tris": tris, "table": table, "mu": MU, "rho": RHO}
    with tempfile.TemporaryDirectory() as td:
        sim = reference_sim(QDsim_gpu, nodes, tris, table, td)
        hs, ts = [], []
        dttry = sim.htry
        for i in range(300):
            h, dttry = sim.simu_forward(dttry)
            hs.append(h)
            ts.append(sim.time)
            if (i + 1) in (1, 25, 50, 100, 150, 200, 250, 300):
                for k in ("Tno", "Tt1o", "state", "slipv1", "slipv", "slip1", "slip"):
                    out[f"s{i + 1}_{k}"] = np.array(getattr(sim, k))
        out["h"], out["t"] = np.array(hs), np.array(ts)
    np.savez_compressed(os.path.join(HERE, "traj_config1.npz"), **out)
    print("traj_config1.npz: t_end = %.6e s, max V = %.3e" % (ts[-1], np.max(sim.slipv)))


def main():
    rng = np.random.default_rng(20251203)
    lib = load_ref_lib()
    make_gf_kat(lib, rng)

    QDsim_gpu = import_reference_python()
    dense = {}
    traj = {}
    with tempfile.TemporaryDirectory() as td:
        # small planar mesh: 8 km x 4 km, 1 km cells -> N = 64
        nodes, tris = mesh.planar_fault(8.0, 4.0, 8, 4)
        _, xg = mesh.element_frames(nodes, tris)
        table = mesh.friction_table(xg, 8e3, 4e3, v_nuc=1e-3, seed=0)
        w1 = os.path.join(td, "planar")
        os.mkdir(w1)
        sim = reference_sim(QDsim_gpu, nodes, tris, table, w1)
        for k in ("A1s", "A2s", "Bs", "A1d", "A2d", "Bd"):
            dense["planar_" + k] = getattr(sim, k)
        dense["planar_nodes"], dense["planar_tris"] = nodes, tris
        dense["planar_eleVec"], dense["planar_xg"] = sim.eleVec, sim.xg
        traj["nodes"], traj["tris"], traj["table"] = nodes, tris, table
        traj["mu"], traj["rho"] = MU, RHO
        # trajectory of the reference CPU stepping
        hs, ts, ckpt = [], [], {}
        dttry = sim.htry
        nsteps = 400
        for i in range(nsteps):
            h, dttry = sim.simu_forward(dttry)
            hs.append(h)
            ts.append(sim.time)
            if (i + 1) in (1, 10, 30, 60, 100, 200, 400):
                for k in ("Tno", "Tt1o", "Tt2o", "state", "slipv1", "slipv2", "slipv", "slip1", "slip2", "slip", "rake"):
                    ckpt[f"s{i + 1}_{k}"] = np.array(getattr(sim, k))
        traj["h"], traj["t"] = np.array(hs), np.array(ts)
        traj.update(ckpt)
        print("trajectory: t_end = %.6e s, max V = %.3e" % (ts[-1], np.max(sim.slipv)))

        # small rough mesh: 6 km x 3 km, 0.5 km cells -> N = 144
        nodes, tris = mesh.rough_fault(6.0, 3.0, 12, 6, seed=1, ratio=1e-2)
        _, xg = mesh.element_frames(nodes, tris)
        table = mesh.friction_table(xg, 6e3, 3e3, seed=1)
        w2 = os.path.join(td, "rough")
        os.mkdir(w2)
        sim = reference_sim(QDsim_gpu, nodes, tris, table, w2)
        for k in ("A1s", "A2s", "Bs", "A1d", "A2d", "Bd"):
            dense["rough_" + k] = getattr(sim, k)
        dense["rough_nodes"], dense["rough_tris"] = nodes, tris
        dense["rough_eleVec"], dense["rough_xg"] = sim.eleVec, sim.xg
    dense["mu"], dense["lam"] = MU, LAM
    np.savez_compressed(os.path.join(HERE, "dense_small.npz"), **dense)
    # reference H-matrix: rough 24 x 12 km fault, 0.6 km cells -> N = 1600
    nodes, tris = mesh.rough_fault(24.0, 12.0, 40, 20, seed=2, ratio=5e-3)
    hm = make_hmatrix_golden(nodes, tris, mini_leaf=32)
    np.savez_compressed(os.path.join(HERE, "hmatrix_small.npz"), **hm)
    print("hmatrix_small.npz: %d leaf blocks, %d ACA" % (len(hm["row_ptr"]) - 1, int(hm["aca"].sum())))
    np.savez_compressed(os.path.join(HERE, "traj_small.npz"), **traj)
    print("dense_small.npz, traj_small.npz written")


if __name__ == "__main__":
    if "--hmatrix-only" in sys.argv:
        main_hmatrix_only()
    elif "--halfspace-only" in sys.argv:
        main_halfspace_only()
    elif "--dilatancy-only" in sys.argv:
        main_dilatancy_only()
    elif "--config1-only" in sys.argv:
        main_config1_only()
    else:
        main()
