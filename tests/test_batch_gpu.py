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
    return ens.traction_rates().cpu().numpy()


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
    _lib.check(L.pq3d_batch_gemm_bf16x6(ens.K.data_ptr(), ens.vop.data_ptr(), N, B, nsplit, ens.tc_ctas,
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


def test_autotuned_launch_shape_and_ctas_do_not_change_bits(cuda):
    """The autotuner returns a valid launch shape, caches it per mesh size
    (nsplit) and per run count (CTAs per SM), and the CTA count is the launch
    shape only: the product's bits are the same for 1, 2 and 3 CTAs per SM."""
    from pyquake3d_gb300 import autotune
    autotune.clear()
    N, B = 600, 20
    rng = np.random.default_rng(5)
    K = torch.as_tensor(rng.standard_normal((3 * N, 2 * N)), device=cuda)
    P = PackedOperator(K)
    shape = autotune.tune_bf16x6(P, B)
    assert shape["tuned"] and 1 <= shape["nsplit"] <= 16 and shape["ctas_per_sm"] in (1, 2, 3)
    again = autotune.tune_bf16x6(P, 30)      # same padded width (32)
    assert not again["tuned"] and again["nsplit"] == shape["nsplit"]
    wide = autotune.tune_bf16x6(P, 200)      # another width: same nsplit, its own CTA count
    assert wide["nsplit"] == shape["nsplit"]
    tabs = np.zeros((B, N, 10))
    tabs[:, :, 1] = 0.01; tabs[:, :, 2] = 0.015; tabs[:, :, 3] = 0.1; tabs[:, :, 4] = 0.6; tabs[:, :, 6] = 30.0
    tabs[:, :, 7] = 10 ** rng.uniform(-12, -1, size=(B, N))
    ens = Ensemble(P, tabs, mu=MU, Cs=CS, precision="bf16x6")
    assert (ens.nsplit, ens.tc_ctas) == (shape["nsplit"], shape["ctas_per_sm"])
    L = _lib.load()
    st = torch.cuda.current_stream().cuda_stream
    outs = []
    for c in (1, 2, 3):
        ens.t["rates"].zero_()
        _lib.check(L.pq3d_batch_gemm_bf16x6(ens.K.data_ptr(), ens.vop.data_ptr(), N, B, ens.nsplit, c,
                                            ens.t["rates"].data_ptr(), ens.ws.data_ptr(), ens.ws.numel(), st))
        outs.append(ens.t["rates"].clone())
    torch.cuda.synchronize()
    assert ens.error_word() == 0
    assert torch.equal(outs[0], outs[1]) and torch.equal(outs[0], outs[2])
    plan = np.zeros(2, dtype=np.int32)
    _lib.check(L.pq3d_batch_gemm_bf16x6_plan(256, 3, plan.ctypes.data))
    assert plan[0] in (1, 2) and plan[1] >= 2     # 3 CTAs of 256 runs do not fit tensor memory


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


def test_bf16x6_product_with_fp64_attempt(cuda, golden):
    """attempt="fp64": the tensor-core product with the reference FP64
    Dormand-Prince arithmetic (no start-of-step constants); over the first 30
    accepted steps slip within 1e-5 of the FP64 batched stepper, like the
    mixed attempt."""
    g, K = _golden(golden, cuda)
    tabs = _tables(g, 4, seed=1)
    a = Ensemble(K, tabs, mu=float(g["mu"]), Cs=CS, precision="fp64", max_steps=30)
    b = Ensemble(PackedOperator(K), tabs, mu=float(g["mu"]), Cs=CS, precision="bf16x6", attempt="fp64", max_steps=30)
    assert "base" not in b.t and b.S.attempt64 == 1
    a.iterate(150)
    b.iterate(150)
    for r in range(4):
        assert normwise_rel(a.t["slip1"][r].cpu().numpy(), b.t["slip1"][r].cpu().numpy()) < 1e-5, r
    assert all(c.steps == 30 and c.status == 0 for c in b.read_ctrl())
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


@pytest.mark.parametrize("nsplit", [1, 4, 9])
def test_fp32_product_k_slices(cuda, golden, nsplit):
    """The split-K FP32 product with 1, 4 and 9 K slices.  The golden mesh
    has 2N = 128 columns = 4 chunks of 32, so with 9 slices five get an empty
    K range and must write zeros.  The partials are NaN before the product,
    so a slice that writes nothing shows.  Each result is within 1e-5 of the
    FP64 product and within 1e-6 of the one-slice result (only the order of
    the FP32 chunk sums differs)."""
    g, K = _golden(golden, cuda)
    tabs = _tables(g, 3, seed=2)
    a = Ensemble(K, tabs, mu=float(g["mu"]), Cs=CS, precision="fp64")
    K32 = K.float().contiguous()
    one = Ensemble(K32, tabs, mu=float(g["mu"]), Cs=CS, precision="fp32", nsplit=1)
    b = Ensemble(K32, tabs, mu=float(g["mu"]), Cs=CS, precision="fp32", nsplit=nsplit)
    assert b.nsplit == nsplit
    b.t["rates"].fill_(float("nan"))
    for e in (a, one, b):
        e.iterate(1)
    ra, r1, rb = _rates(a), _rates(one), _rates(b)
    assert np.all(np.isfinite(rb))
    for r in range(3):
        assert normwise_rel(ra[r], rb[r]) < 1e-5, r
        assert normwise_rel(r1[r], rb[r]) < 1e-6, r


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


# Cells recorded from RK45 stepping of the 200 x 40 km rough fault (N = 100,000,
# H-matrix product, nucleation patch at 1e-3 m/s) at t = 26.2 s:
# (a, b, dc, f0, Tno, Tt1o, Tt2o, state, V, AdotV1, AdotV2, dsigma/dt).  With
# dt = 9.2124 s, stage 5 of the Dormand-Prince attempt overshoots the first
# four cells' shear stress by ~11 MPa, i.e. the slip-rate exponent by ~100:
# FP64 stays finite there (the step is rejected with a moderate error); FP32
# e^x overflows unless the right-hand side is kept in scale.
STAGE_OVERSHOOT_DT = 9.212423770310084
STAGE_OVERSHOOT_CELLS = np.array([
    (0.004, 0.03, 0.14, 0.6, 25.10468272887533, 20.86252722459316, -0.002760444839195026, 0.7992124489447135,
     0.002841888671875, 71096.96010955973, -5694.026039135735, 6560.18839958655),
    (0.004, 0.03, 0.14, 0.6, 25.01407476670933, 20.789991456525662, -0.0022071424474962094, 0.7989258258571602,
     0.003138430908203125, 94074.79105999242, -6539.926320837528, 821.216190121016),
    (0.004, 0.03, 0.14, 0.6, 25.010806663905637, 20.783066464523046, -0.003983947056773062, 0.7986710025369866,
     0.00320707470703125, 71442.20331160886, -4145.00307035588, 765.1998111441719),
    (0.004, 0.03, 0.14, 0.6, 24.979281731662297, 20.754842854125048, -0.0017027261935954384, 0.7982971840641563,
     0.0034505085449218747, 78594.30492606362, -4672.568136799041, -1424.6719326721313),
    (0.007839999999999993, 0.03, 0.14, 0.6, 25.00000776405218, 18.827723270419693, -3.647291134394441e-05,
     0.8072326583603793, 1.0041975183412432e-09, -43.931460405325566, 1.9563141481575645, 0.42981355991842674),
    (0.02656, 0.03, 0.14, 0.6, 25.000243771293796, 15.601184432203162, 0.0024916621398196393, 0.8072326583459437,
     1.0105451801791787e-09, -351.2858186715674, -130.83729749546245, 11.993399799267007),
    (0.04000000000000001, 0.03, 0.14, 0.6, 25.000001389555507, 13.273161081080296, 7.962887358376142e-06,
     0.8072326583692505, 1.000099233348689e-09, -5.346188035257384, -0.4267521966803598, 0.0764763278500351),
    (0.004, 0.03, 0.14, 0.6, 24.999990713881537, 19.50592064913241, 0.0011329691141147916, 0.8072326580016972,
     1.1721852933987974e-09, -803.5071173343583, -67.20042687143759, -1.0927068774489872)])


def _recorded_cells_ensemble(cuda, precision, h, rows, attempt="mixed"):
    """One run over the recorded cells: state written directly, and a
    (3n x 2n) operator with one non-zero column per cell so that K.v'
    reproduces the recorded traction rates."""
    cells = STAGE_OVERSHOOT_CELLS[rows]
    n = len(cells)
    tab = np.zeros((1, n, 10))
    tab[0, :, 1:5] = cells[:, 0:4]
    tab[0, :, 6] = cells[:, 4]
    tab[0, :, 7] = cells[:, 8]
    vp = cells[:, 8] - 1e-9                     # v' = V - Vpl (rake 0)
    K = np.zeros((3 * n, 2 * n))
    for i in range(n):
        K[3 * i:3 * i + 3, 2 * i] = cells[i, 9:12] / vp[i]
    Kt = torch.as_tensor(K, device=cuda)
    if precision == "fp32":
        Kt = Kt.float().contiguous()
    ens = Ensemble(Kt, tab, mu=MU, Cs=CS, precision=precision, dttry=h, attempt=attempt)
    for k, col in (("Tno", 4), ("Tt1o", 5), ("Tt2o", 6), ("state", 7), ("slipv", 8), ("slipv1", 8)):
        ens.t[k][0].copy_(torch.as_tensor(cells[:, col]))
    ens.t["slipv2"].zero_()
    ens.prepare()
    return ens, cells


def _oracle_attempt(cells, h):
    """The reference's FP64 attempt on the recorded cells (per cell)."""
    from oracle.stepping import DenseStepper
    s = object.__new__(DenseStepper)
    s.mu, s.Cs, s.V0 = MU, CS, 1e-6
    s.a, s.b, s.dc, s.f0 = (cells[:, k].copy() for k in range(4))
    s.Tno, s.Tt1o, s.Tt2o, s.state, s.slipv = (cells[:, k].copy() for k in range(4, 9))
    s.AdotV1, s.AdotV2, s.dsigmadt = cells[:, 9].copy(), cells[:, 10].copy(), cells[:, 11].copy()
    s.shear_loading = np.zeros(len(cells))
    s.P = np.zeros(len(cells))
    s.dPdt0 = np.zeros(len(cells))
    return s.rk_attempt_raw(h)


@pytest.mark.parametrize("rows,h", [(slice(0, 4), STAGE_OVERSHOOT_DT), (slice(0, 8), STAGE_OVERSHOOT_DT / 2),
                                    (slice(4, 8), STAGE_OVERSHOOT_DT), (slice(0, 8), 0.5)])
def test_mixed_attempt_in_range_through_stage_overshoot(cuda, rows, h):
    """The mixed-precision attempt against the FP64 one on the recorded cells:
    error norms within 1e-4 relative or 1e-8 absolute (they decide accept /
    reject and the next dt against the tolerance 1e-4), candidate state
    within 1e-6 of the step's increment, no NaN or inf from finite inputs --
    including the attempt whose stage 5 overshoots."""
    ref = _oracle_attempt(STAGE_OVERSHOOT_CELLS[rows], h)
    res = {}
    for prec in ("fp64", "fp32"):
        ens, cells = _recorded_cells_ensemble(cuda, prec, h, rows)
        ens.begin()
        w = ens.error_words()[0].cpu().numpy()
        err = w.view(np.float64)
        cand = ens.t["cand"].view(-1, 4).cpu().numpy()
        ens.end()
        res[prec] = (err, cand, ens.read_ctrl()[0])
    e64, c64, k64 = res["fp64"]
    e32, c32, k32 = res["fp32"]
    assert np.all(np.isfinite(e32)) and np.all(np.isfinite(c32))
    # FP64 arm = the reference arithmetic (the state error is a difference of
    # two states ~0.8 apart by ~1e-10: ~1e-15 of rounding)
    assert abs(e64[0] - ref[4]) <= 1e-6 * ref[4] + 1e-14
    assert abs(e64[1] - ref[5]) <= 1e-9 * ref[5] + 1e-15
    assert abs(e32[0] - e64[0]) <= 1e-4 * e64[0] + 1e-8
    assert abs(e32[1] - e64[1]) <= 1e-4 * e64[1] + 1e-8
    y0 = STAGE_OVERSHOOT_CELLS[rows][:, [4, 5, 6, 7]]
    inc = np.abs(c64 - y0)
    assert np.all(np.abs(c32 - c64) <= 1e-6 * inc + 1e-13 * np.abs(y0))
    assert k32.accepted == k64.accepted
    assert abs(k32.h - k64.h) <= 1e-4 * k64.h


@pytest.mark.parametrize("rows,h", [(slice(0, 4), STAGE_OVERSHOOT_DT), (slice(0, 8), STAGE_OVERSHOOT_DT / 2),
                                    (slice(4, 8), STAGE_OVERSHOOT_DT), (slice(0, 8), 0.5)])
def test_ff_attempt_matches_fp64_attempt_through_stage_overshoot(cuda, rows, h):
    """The float-float attempt against the FP64 attempt on the recorded cells,
    the same FP32 product under both: error norms within 1e-6 (the first, a
    difference of two states ~0.8 apart, carries the FP64 attempt's own
    rounding of ~1e-6 of it) and 1e-9 relative, candidate state within 1e-12
    of the step's increment, the same decision and next step size to 1e-9 --
    including the attempt whose stage 5 overshoots (the w-form keeps the
    float-float range)."""
    res = {}
    for att in ("fp64", "ff"):
        ens, _ = _recorded_cells_ensemble(cuda, "fp32", h, rows, attempt=att)
        ens.begin()
        err = ens.error_words()[0].cpu().numpy().view(np.float64)
        cand = ens.t["cand"].view(-1, 4).cpu().numpy()
        ens.end()
        res[att] = (err, cand, ens.read_ctrl()[0])
    e64, c64, k64 = res["fp64"]
    eff, cff, kff = res["ff"]
    assert np.all(np.isfinite(eff)) and np.all(np.isfinite(cff))
    assert abs(eff[0] - e64[0]) <= 1e-6 * e64[0] + 1e-14
    assert abs(eff[1] - e64[1]) <= 1e-9 * e64[1] + 1e-15
    y0 = STAGE_OVERSHOOT_CELLS[rows][:, [4, 5, 6, 7]]
    inc = np.abs(c64 - y0)
    assert np.all(np.abs(cff - c64) <= 1e-12 * inc + 1e-15 * np.abs(y0))
    assert kff.accepted == k64.accepted
    assert abs(kff.h - k64.h) <= 1e-9 * k64.h


def test_batched_fp64_matches_single_simulation_n10000(cuda):
    """The batched workload's mesh and runs (planar 100 x 50 km, N = 10,000,
    per-run friction draws with nucleation patches): the FP64 batched stepper
    against the single-simulation FP64 stepper run by run over 25 accepted
    steps, state and slip to 1e-9.  (The two products add in different
    orders; from step ~30 the nucleation amplifies that ulp-level difference
    -- 8e-9 at step 40 -- as it does any 1e-16 perturbation.)"""
    nodes, tris = mesh.planar_fault(100.0, 50.0, 100, 50)
    _, xg = mesh.element_frames(nodes, tris)
    tabs = mesh.ensemble_tables(xg, 100e3, 50e3, B=4, seed=0, v_nuc=1e-3)
    K64, _ = gf.assemble_dense(nodes, tris, MU, MU, fp32_copy=False, device=cuda)
    ens = Ensemble(K64, tabs, mu=MU, Cs=CS, precision="fp64", max_steps=25)
    ens.iterate(300)
    ctrl = ens.read_ctrl()
    for r in (0, 3):
        assert ctrl[r].steps == 25 and ctrl[r].status == 0
        one = DenseDeviceSim(K64, initial_state(tabs[r], 1e-6, 1e-9), mu=MU, Cs=CS, V0=1e-6, Vpl=1e-9)
        one.step(25)
        for k in ("slip1", "state", "Tt1o", "Tno"):
            assert normwise_rel(one.t[k].cpu().numpy(), ens.t[k][r].cpu().numpy()) < 1e-9, (r, k)
        assert np.isclose(ctrl[r].time, one.read_ctrl().time, rtol=1e-9)
