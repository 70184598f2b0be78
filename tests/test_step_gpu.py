"""GPU stepping parity: the persistent FP64 stepper against the reference CPU
trajectory (golden) and against the NumPy oracle; the traction-product
kernels against NumPy; the failure path."""
import numpy as np
import pytest
import torch

import oracle
from oracle.stepping import DenseStepper
from pyquake3d_gb300 import _lib, gf, mesh
from pyquake3d_gb300.QDsim_gpu import DenseDeviceSim, StepError, initial_state
from tests.util import normwise_rel

pytestmark = pytest.mark.gpu
MU = 32038120320.0
RHO = MU / 3464.0 ** 2


def test_matvec_f64_f32_match_numpy(cuda):
    rng = np.random.default_rng(0)
    for N in (1, 31, 33, 100, 257):
        K = rng.standard_normal((3 * N, 2 * N))
        v = rng.standard_normal(2 * N)
        Kt = torch.as_tensor(K, device=cuda)
        vt = torch.as_tensor(v, device=cuda)
        out = torch.empty(3 * N, dtype=torch.float64, device=cuda)
        L = _lib.load()
        st = torch.cuda.current_stream().cuda_stream
        _lib.check(L.pq3d_dense_matvec_f64(Kt.data_ptr(), N, vt.data_ptr(), out.data_ptr(), st))
        ref = K @ v
        assert np.abs(out.cpu().numpy() - ref).max() <= 1e-13 * np.abs(K).sum(axis=1).max() * np.abs(v).max()
        K32 = Kt.float().contiguous()
        _lib.check(L.pq3d_dense_matvec_f32(K32.data_ptr(), N, vt.data_ptr(), out.data_ptr(), st))
        assert np.abs(out.cpu().numpy() - ref).max() <= 1e-5 * np.abs(K).sum(axis=1).max() * np.abs(v).max()


def _golden_sim(golden, cuda, dtype=torch.float64):
    g = golden("traj_small.npz")
    d = golden("dense_small.npz")
    K = gf.join_ops({k: d["planar_" + k] for k in oracle.OPS})
    Kt = torch.as_tensor(K, device=cuda).to(dtype).contiguous()
    init = initial_state(g["table"], 1e-6, 1e-9)
    sim = DenseDeviceSim(Kt, init, mu=float(g["mu"]), Cs=np.sqrt(float(g["mu"]) / float(g["rho"])), V0=1e-6,
                         Vpl=1e-9, dttry=1e-3)
    return g, sim


def test_stepper_reproduces_reference_trajectory(cuda, golden):
    g, sim = _golden_sim(golden, cuda)
    hs = []
    done = 0
    for stop in (1, 10, 100, 200, 400):
        h, t, c = sim.step(stop - done)
        hs.extend(h)
        done = stop
        for k in ("slip1", "slipv1", "state", "Tt1o", "Tno", "slip"):
            got = sim.t[k].cpu().numpy()
            assert normwise_rel(g[f"s{stop}_{k}"], got) < 1e-9, (stop, k)
    assert np.allclose(hs, g["h"], rtol=1e-9, atol=0)
    assert np.isclose(c.time, g["t"][-1], rtol=1e-9)


def test_many_steps_per_launch_equal_one_step_per_launch(cuda, golden):
    _, a = _golden_sim(golden, cuda)
    _, b = _golden_sim(golden, cuda)
    a.step(50)
    for _ in range(50):
        b.step(1)
    for k in ("slip1", "slip2", "state", "Tt1o", "Tt2o", "Tno"):
        assert torch.equal(a.t[k], b.t[k]), k


def test_stepper_vs_oracle_config1_mesh(cuda):
    """N = 1600 planar fault (40 x 20 km, 1 km squares), 300 accepted steps,
    GPU-assembled operator vs the oracle operator and oracle stepping."""
    nodes, tris = mesh.planar_fault(40.0, 20.0, 40, 20)
    _, xg = mesh.element_frames(nodes, tris)
    tab = mesh.friction_table(xg, 40e3, 20e3, seed=0)
    K64, _ = gf.assemble_dense(nodes, tris, MU, MU, fp32_copy=False)
    Ko = oracle.assemble_dense(nodes, tris, MU, MU, nthreads=8)
    ops = {name: Ko[k] for k, name in enumerate(oracle.OPS)}
    ref = DenseStepper(ops, tab, mu=MU, density=RHO)
    sim = DenseDeviceSim(K64, initial_state(tab, 1e-6, 1e-9), mu=MU, Cs=3464.0, V0=1e-6, Vpl=1e-9)
    hist = ref.run(300)
    h, t, c = sim.step(300)
    assert np.allclose(h, hist[:, 0], rtol=1e-6)
    for k in ("slip1", "slip"):
        assert normwise_rel(getattr(ref, k), sim.t[k].cpu().numpy()) < 1e-5, k
    assert normwise_rel(ref.slipv, sim.t["slipv"].cpu().numpy()) < 1e-5


def test_fp32_operator_stays_close(cuda, golden):
    _, a = _golden_sim(golden, cuda)
    _, b = _golden_sim(golden, cuda, dtype=torch.float32)
    a.step(100)
    b.step(100)
    assert normwise_rel(a.t["slip1"].cpu().numpy(), b.t["slip1"].cpu().numpy()) < 1e-4


def test_nan_state_reports_step_failure(cuda, golden):
    _, sim = _golden_sim(golden, cuda)
    sim.t["state"][3] = float("nan")   # host-side injection: every attempt is rejected
    with pytest.raises(StepError):
        sim.step(1)
    c = sim.read_ctrl()
    assert c.status == _lib.PQ3D_ERR_STEP
    assert c.attempts == 21
    # the context is still usable
    _, ok = _golden_sim(golden, cuda)
    ok.step(2)
