"""The float-float Dormand-Prince attempt (attempt="ff", pq3d_batch_sim
attempt64 = 2) against the FP64 attempt on the same BF16x18 product: one
iteration agrees to rounding, free-running steps agree closely, and in
lockstep with the FP64 stepper it holds the slip bar as long as the FP64
attempt does."""
import numpy as np
import pytest
import torch

from pyquake3d_gb300 import gf, mesh
from pyquake3d_gb300.ensemble import Ensemble, PackedFixOperator, lockstep
from tests.util import normwise_rel

pytestmark = pytest.mark.gpu
MU = 32038120320.0
CS = 3464.0


def _physical(cuda, nx=40, nz=20, B=8, seed=0):
    nodes, tris = mesh.planar_fault(float(nx), float(nz), nx, nz)
    K64, _ = gf.assemble_dense(nodes, tris, MU, MU, fp32_copy=False, device=cuda)
    _, xg = mesh.element_frames(nodes, tris)
    tabs = mesh.ensemble_tables(xg, nx * 1e3, nz * 1e3, B=B, seed=seed, v_nuc=1e-3)
    return K64, tabs, xg


def _pair(K64, tabs, xg, **kw):
    P = PackedFixOperator(K64, xg)
    a = Ensemble(P, tabs, mu=MU, Cs=CS, precision="bf16x18", attempt="fp64", nsplit=2, **kw)
    b = Ensemble(P, tabs, mu=MU, Cs=CS, precision="bf16x18", attempt="ff", nsplit=2, **kw)
    assert a.S.attempt64 == 1 and b.S.attempt64 == 2 and "base" not in b.t
    return a, b


def test_ff_attempt_one_iteration_equals_fp64_attempt(cuda):
    """Planar N = 1,600, 8 runs with nucleation patches: after one iteration
    (the same product, then the attempt, decision and update) the states agree
    to 1e-13 and the slip rates to 1e-10 (relative, normwise per run), every
    run takes the same decision, and the next step sizes agree to 1e-9."""
    K64, tabs, xg = _physical(cuda)
    a, b = _pair(K64, tabs, xg)
    a.iterate(1)
    b.iterate(1)
    ca, cb = a.read_ctrl(), b.read_ctrl()
    for r in range(tabs.shape[0]):
        assert (ca[r].steps, ca[r].attempts) == (cb[r].steps, cb[r].attempts), r
        assert abs(ca[r].h - cb[r].h) <= 1e-9 * abs(ca[r].h), r
        for k in ("Tno", "Tt1o", "Tt2o", "state", "slip1", "slip2"):
            assert normwise_rel(a.t[k][r].cpu().numpy(), b.t[k][r].cpu().numpy()) < 1e-13, (k, r)
        for k in ("slipv1", "slipv2"):
            assert normwise_rel(a.t[k][r].cpu().numpy(), b.t[k][r].cpu().numpy()) < 1e-10, (k, r)
    assert b.error_word() == 0


def test_ff_attempt_free_running_close_to_fp64_attempt(cuda):
    """Free-running (each ensemble its own step sizes) for 40 accepted steps
    through the nucleation: the two attempts' slips stay within 1e-9."""
    K64, tabs, xg = _physical(cuda)
    a, b = _pair(K64, tabs, xg, max_steps=40)
    a.iterate(200)
    b.iterate(200)
    assert all(c.steps == 40 and c.status == 0 for c in a.read_ctrl())
    assert all(c.steps == 40 and c.status == 0 for c in b.read_ctrl())
    for r in range(tabs.shape[0]):
        assert normwise_rel(a.t["slip1"][r].cpu().numpy(), b.t["slip1"][r].cpu().numpy()) < 1e-9, r


@pytest.mark.parametrize("order", ["compact", "mesh"])
def test_ff_attempt_tracks_fp64_through_nucleation(cuda, order):
    """Lockstep with the FP64 batched stepper on planar N = 1,600, 8 runs,
    120 accepted steps: within 2e-6 in slip, the bar the FP64 attempt on the
    same product meets.  In the mesh's own cell order the update kernel packs
    v' itself; in the compact order the pack kernel does."""
    K64, tabs, xg = _physical(cuda)
    kw = dict(mu=MU, Cs=CS, max_steps=120)
    ref = Ensemble(K64, tabs, precision="fp64", **kw)
    ff = Ensemble(PackedFixOperator(K64, xg if order == "compact" else None), tabs, precision="bf16x18",
                  attempt="ff", **kw)
    r = lockstep(ref, {"ff": ff}, 120, bar=2e-6)["ff"]
    assert r["failed_runs"] == 0 and ff.error_word() == 0
    assert r["steps_within"] >= 120, r


@pytest.mark.parametrize("order", ["compact", "mesh"])
def test_ff_attempt_horizon_on_the_batched_workload(cuda, order):
    """The batched workload (planar 100 x 50 km, N = 10,000, nucleation
    patches at 1e-3 m/s), 8 runs in lockstep with the FP64 batched stepper:
    the BF16x18 product with the float-float attempt keeps every run's slip
    within 1e-5 of FP64 for 80 accepted steps, like the FP64 attempt (the
    mesh order is the benchmark's)."""
    K64, tabs, xg = _physical(cuda, nx=100, nz=50, B=8)
    kw = dict(mu=MU, Cs=CS, max_steps=80)
    ref = Ensemble(K64, tabs, precision="fp64", **kw)
    ff = Ensemble(PackedFixOperator(K64, xg if order == "compact" else None), tabs, precision="bf16x18",
                  attempt="ff", nsplit=5, **kw)
    r = lockstep(ref, {"ff": ff}, 80, bar=1e-5)["ff"]
    assert r["failed_runs"] == 0 and ff.error_word() == 0
    assert r["steps_within"] >= 80, r


def test_ff_attempt_rejected_for_bad_value():
    with pytest.raises(ValueError):
        Ensemble(torch.zeros((3, 2), dtype=torch.float64), np.zeros((1, 1, 10)), mu=MU, Cs=CS, precision="fp64",
                 attempt="fp128")


@pytest.mark.parametrize("precision", ["hmat", "fp32"])
def test_ff_attempt_with_other_products(cuda, precision):
    """The float-float attempt behind the H-matrix and the plain FP32
    products (FP64 partial sums, split on the device): one iteration equals
    the FP64 attempt on the same product to 1e-13 in the states."""
    from pyquake3d_gb300.hmatrix import HMatrix
    nodes, tris = mesh.planar_fault(40.0, 20.0, 40, 20)
    _, xg = mesh.element_frames(nodes, tris)
    tabs = mesh.ensemble_tables(xg, 40e3, 20e3, B=4, seed=2, v_nuc=1e-3)
    if precision == "hmat":
        K = HMatrix(nodes, tris, MU, MU, min_size=32, mini_leaf=32, tol=1e-6, device=cuda)
    else:
        K = gf.assemble_dense(nodes, tris, MU, MU, device=cuda)[1]
    a = Ensemble(K, tabs, mu=MU, Cs=CS, precision=precision, attempt="fp64")
    b = Ensemble(K, tabs, mu=MU, Cs=CS, precision=precision, attempt="ff")
    assert b.S.attempt64 == 2
    a.iterate(1)
    b.iterate(1)
    for r in range(4):
        for k in ("Tt1o", "Tt2o", "state", "slip1"):
            assert normwise_rel(a.t[k][r].cpu().numpy(), b.t[k][r].cpu().numpy()) < 1e-13, (k, r)
    assert [c.steps for c in a.read_ctrl()] == [c.steps for c in b.read_ctrl()]


def test_ff_attempt_small_mesh_and_odd_run_count(cuda, golden):
    """The golden mesh (N = 64: one 256-column span, padded operator tiles)
    with 3 runs: 30 free-running accepted steps of the float-float attempt
    stay within 1e-9 in slip of the FP64 attempt on the same product."""
    from tests.test_batch_gpu import CS as CS_G, _golden, _tables
    g, K = _golden(golden, cuda)
    tabs = _tables(g, 3, seed=6)
    P = PackedFixOperator(K)
    kw = dict(mu=float(g["mu"]), Cs=CS_G, max_steps=30, nsplit=1)
    a = Ensemble(P, tabs, precision="bf16x18", attempt="fp64", **kw)
    b = Ensemble(P, tabs, precision="bf16x18", attempt="ff", **kw)
    a.iterate(150)
    b.iterate(150)
    assert all(c.steps == 30 and c.status == 0 for c in b.read_ctrl())
    assert [c.steps for c in a.read_ctrl()] == [c.steps for c in b.read_ctrl()]
    for r in range(3):
        assert normwise_rel(a.t["slip1"][r].cpu().numpy(), b.t["slip1"][r].cpu().numpy()) < 1e-9, r
    assert b.error_word() == 0
