"""Batched ensemble on the GPU: the tcgen05 BF16x6 traction product against
FP64, batched runs against the single-simulation stepper, bitwise equality of
a run alone and in a mix, CUDA-graph replay, per-run failure isolation."""
import ctypes

import numpy as np
import pytest
import torch

import oracle
from pyquake3d_gb300 import _lib, gf, mesh
from pyquake3d_gb300.ensemble import Ensemble, PackedOperator
from pyquake3d_gb300.QDsim_gpu import DenseDeviceSim, initial_state
from tests.util import normwise_rel

pytestmark = pytest.mark.gpu
MU = 32038120320.0
CS = 3464.0


def _golden(golden, cuda):
    d = golden("dense_small.npz")
    g = golden("traj_small.npz")
    K = torch.as_tensor(gf.join_ops({k: d["planar_" + k] for k in oracle.OPS}), device=cuda).contiguous()
    return g, K


def _tables(g, B, seed=0):
    """B variants of the golden table: sigma, Dc and initial V per run."""
    rng = np.random.default_rng(seed)
    out = []
    for r in range(B):
        t = g["table"].copy()
        t[:, 6] *= rng.uniform(0.8, 1.2)
        t[:, 3] *= rng.uniform(0.8, 1.2)
        t[:, 7] = np.where(t[:, 7] > 1e-9, t[:, 7] * rng.uniform(0.5, 2.0), t[:, 7])
        out.append(t)
    return np.stack(out)


def _rates(ens):
    r = ens.t["rates"].view(ens.nsplit, ens.Bp, 3 * ens.N).sum(0)
    return r[:ens.B].cpu().numpy()


@pytest.mark.parametrize("N,B,nsplit", [(64, 16, 1), (64, 5, 3), (700, 64, 2), (1000, 40, 7)])
def test_tensor_core_product_matches_fp64(cuda, N, B, nsplit):
    """rates = K.v' for all runs: BF16x6 on tcgen05 vs FP64 (torch).  The split
    products carry ~2^-24; the FP32 accumulation in tensor memory over up to
    2N terms adds ~1e-6 on random data (measured 1.1e-6 .. 1.6e-6), so the bar
    is 5e-6 normwise per run."""
    rng = np.random.default_rng(N + B)
    K = torch.as_tensor(rng.standard_normal((3 * N, 2 * N)) * 1e9, device=cuda)
    tabs = np.zeros((B, N, 10))
    tabs[:, :, 1] = 0.01; tabs[:, :, 2] = 0.015; tabs[:, :, 3] = 0.1; tabs[:, :, 4] = 0.6; tabs[:, :, 6] = 30.0
    tabs[:, :, 7] = 10 ** rng.uniform(-12, -1, size=(B, N))
    tabs[:, :, 0] = rng.uniform(-0.3, 0.3, size=(B, N))
    ens = Ensemble(PackedOperator(K), tabs, mu=MU, Cs=CS, precision="bf16x6", nsplit=nsplit)
    L = _lib.load()
    st = torch.cuda.current_stream().cuda_stream
    _lib.check(L.pq3d_batch_gemm_bf16x6(ens.K.data_ptr(), ens.vop.data_ptr(), N, B, nsplit,
                                        ens.t["rates"].data_ptr(), ens.ws.data_ptr(), ens.ws.numel(), st))
    torch.cuda.synchronize()
    assert ens.error_word() == 0
    v = torch.empty((B, 2 * N), dtype=torch.float64, device=cuda)
    v[:, 0::2] = ens.t["slipv1"] - 1e-9 * ens.t["cos_rake0"]
    v[:, 1::2] = ens.t["slipv2"] - 1e-9 * ens.t["sin_rake0"]
    ref = (K @ v.T).T.cpu().numpy()
    got = _rates(ens)
    for r in range(B):
        assert normwise_rel(ref[r], got[r]) < 5e-6, r


def test_batched_fp64_matches_single_simulation(cuda, golden):
    g, K = _golden(golden, cuda)
    tabs = _tables(g, 3)
    ens = Ensemble(K, tabs, mu=float(g["mu"]), Cs=CS, precision="fp64", max_steps=30)
    ens.iterate(200)
    ctrl = ens.read_ctrl()
    for r in range(3):
        assert ctrl[r].steps == 30 and ctrl[r].active == 0 and ctrl[r].status == 0
        one = DenseDeviceSim(K, initial_state(tabs[r], 1e-6, 1e-9), mu=float(g["mu"]), Cs=CS, V0=1e-6, Vpl=1e-9)
        one.step(30)
        for k in ("slip1", "state", "Tt1o", "Tno"):
            assert normwise_rel(one.t[k].cpu().numpy(), ens.t[k][r].cpu().numpy()) < 1e-9, (r, k)
        assert np.isclose(ctrl[r].time, one.read_ctrl().time, rtol=1e-9)


def test_bf16x6_traction_rates_and_early_trajectory(cuda, golden):
    """Same states: BF16x6 traction rates within 1e-6 of FP64; over the first
    30 accepted steps (before step-control divergence) slip within 1e-5."""
    g, K = _golden(golden, cuda)
    tabs = _tables(g, 4, seed=1)
    a = Ensemble(K, tabs, mu=float(g["mu"]), Cs=CS, precision="fp64", max_steps=30)
    b = Ensemble(PackedOperator(K), tabs, mu=float(g["mu"]), Cs=CS, precision="bf16x6", max_steps=30)
    a.iterate(1)
    b.iterate(1)
    ra, rb = _rates(a), _rates(b)
    for r in range(4):
        assert normwise_rel(ra[r], rb[r]) < 1e-6, r
    a.iterate(150)
    b.iterate(150)
    for r in range(4):
        assert normwise_rel(a.t["slip1"][r].cpu().numpy(), b.t["slip1"][r].cpu().numpy()) < 1e-5, r
    assert b.error_word() == 0


def test_fp32_batched_product_close_to_fp64(cuda, golden):
    g, K = _golden(golden, cuda)
    tabs = _tables(g, 3, seed=2)
    a = Ensemble(K, tabs, mu=float(g["mu"]), Cs=CS, precision="fp64")
    b = Ensemble(K.float().contiguous(), tabs, mu=float(g["mu"]), Cs=CS, precision="fp32")
    a.iterate(1)
    b.iterate(1)
    ra, rb = _rates(a), _rates(b)
    for r in range(3):
        assert normwise_rel(ra[r], rb[r]) < 1e-5, r


def test_run_alone_equals_run_in_mix_bitwise(cuda, golden):
    """Serving determinism: a run's trajectory does not depend on which other
    runs share the batch (per-element accumulation order is fixed)."""
    g, K = _golden(golden, cuda)
    P = PackedOperator(K)
    tabs = _tables(g, 20, seed=3)
    mix = Ensemble(P, tabs, mu=float(g["mu"]), Cs=CS, precision="bf16x6", max_steps=40)
    alone = Ensemble(P, tabs[7:8], mu=float(g["mu"]), Cs=CS, precision="bf16x6", max_steps=40)
    mix.iterate(120)
    alone.iterate(120)
    for k in ("slip1", "slip2", "state", "Tt1o", "Tno", "slipv"):
        assert torch.equal(mix.t[k][7], alone.t[k][0]), k
    assert mix.read_ctrl()[7].time == alone.read_ctrl()[0].time


def test_graph_replay_equals_eager(cuda, golden):
    g, K = _golden(golden, cuda)
    P = PackedOperator(K)
    tabs = _tables(g, 6, seed=4)
    e = Ensemble(P, tabs, mu=float(g["mu"]), Cs=CS, precision="bf16x6")
    c = Ensemble(P, tabs, mu=float(g["mu"]), Cs=CS, precision="bf16x6")
    e.iterate(31)
    c.iterate(1)
    c.capture(10)
    c.replay(3)
    torch.cuda.synchronize()
    for k in ("slip1", "state", "Tt1o"):
        assert torch.equal(e.t[k], c.t[k]), k


def test_failing_run_is_retired_alone(cuda, golden):
    """A run whose state is NaN (host-side injection) ends with PQ3D_ERR_STEP
    after 21 rejected attempts; the other runs keep stepping."""
    g, K = _golden(golden, cuda)
    tabs = _tables(g, 3, seed=5)
    e = Ensemble(PackedOperator(K), tabs, mu=float(g["mu"]), Cs=CS, precision="bf16x6", max_steps=25)
    e.t["state"][1, 5] = float("nan")
    e.iterate(60)
    c = e.read_ctrl()
    assert c[1].status == _lib.PQ3D_ERR_STEP and c[1].active == 0 and c[1].attempts == 21
    for r in (0, 2):
        assert c[r].status == 0 and c[r].steps == 25
