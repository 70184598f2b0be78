"""The fixed-point BF16x18 tensor-core product (pq3d_batch_gemm_bf16x18) and
the batched stepper built on it: exact accumulation on the integer grid, the
product against the NumPy model of its slices and against FP64, K-slice
invariance, and slip tracking of the FP64 stepper in lockstep through a
nucleation."""
import math

import numpy as np
import pytest
import torch

import oracle
from pyquake3d_gb300 import _lib, gf, mesh
from pyquake3d_gb300.ensemble import Ensemble, PackedFixOperator, lockstep
from tests import fixemul
from tests.util import normwise_rel

pytestmark = pytest.mark.gpu
MU = 32038120320.0
CS = 3464.0


def _run_product(cuda, K, V, nsplit, xg=None):
    """(nsplit, Bp, 3N, 2) float32 (hi, lo) partials (rows in the operator's
    cell order: mesh order, or the compact order of xg), the error word and
    the packed operator."""
    L = _lib.load()
    N, B = K.shape[1] // 2, V.shape[0]
    Kt = torch.as_tensor(K, device=cuda).contiguous()
    Vt = torch.as_tensor(V, device=cuda).contiguous()
    P = PackedFixOperator(Kt, xg)
    vop = torch.zeros(L.pq3d_batch_rhs_fix_bytes(N, B), dtype=torch.uint8, device=cuda)
    st = torch.cuda.current_stream().cuda_stream
    order = P.order.data_ptr() if P.order is not None else None
    _lib.check(L.pq3d_batch_pack_rhs_fix(Vt.data_ptr(), N, B, order, vop.data_ptr(), st))
    Bp = (B + 15) // 16 * 16
    out = torch.full((nsplit, Bp, 3 * N, 2), float("nan"), dtype=torch.float32, device=cuda)
    ws = torch.zeros(256, dtype=torch.uint8, device=cuda)
    _lib.check(L.pq3d_batch_gemm_bf16x18(P.data.data_ptr(), vop.data_ptr(), N, B, nsplit, out.data_ptr(),
                                         ws.data_ptr(), ws.numel(), st))
    torch.cuda.synchronize()
    return out.cpu().numpy(), int(ws[:4].view(torch.int32).item()), P


def _from_digits(rng, rows, cols, ndig, sign, chunk):
    """Values whose fixed-point digits per (row, `chunk` columns) are known:
    leading digit +-126/127 (so the chunk exponent is e), the next two random
    in [-127, 127], the rest zero.  Returns (X, digits, e)."""
    nch = (cols + chunk - 1) // chunk
    e = rng.integers(-4, 31, size=(rows, nch))
    eb = np.repeat(e, chunk, axis=1)[:, :cols]
    d = [np.zeros((rows, cols), dtype=np.int64) for _ in range(ndig)]
    d[0] = sign[:, None] * rng.integers(126, 128, size=(rows, cols))
    d[1] = rng.integers(-127, 128, size=(rows, cols))
    d[2] = rng.integers(-127, 128, size=(rows, cols))
    X = sum(np.ldexp(d[p].astype(np.float64), eb - 7 - 8 * p) for p in range(ndig))
    return X, d, e


@pytest.mark.parametrize("nsplit", [1, 3])
def test_fix_product_accumulates_exactly(cuda, nsplit):
    """Digits chosen so that the slot sums of a 256-column span come close to
    the 2^24 limit of exact FP32 integers (the level-2 slot adds three slice
    pairs of 256 products of 126..127 x 126..127 in one sign): the tensor-core
    result must equal the exact sum of the slice products (math.fsum of the
    exact integer span sums) to float-float precision.  An accumulation that
    rounded at FP32 level would be off by ~1e-7."""
    rng = np.random.default_rng(11)
    N, B = 1024, 64                      # 2N = 2048 columns: 2 operator chunks, 8 spans
    K, dK, eK = _from_digits(rng, 3 * N, 2 * N, fixemul.K_SLICES, rng.choice([-1, 1], size=3 * N),
                             fixemul.K_CHUNK)
    V, dV, eV = _from_digits(rng, B, 2 * N, fixemul.V_SLICES, rng.choice([-1, 1], size=B), fixemul.V_CHUNK)
    out, err, _ = _run_product(cuda, K, V, nsplit)
    assert err == 0
    got = out[..., 0].astype(np.float64).sum(0)[:B] + out[..., 1].astype(np.float64).sum(0)[:B]
    # exact: per span and slice pair an integer sum, scaled by a power of two
    terms = []
    for sp in range(2 * N // fixemul.V_CHUNK):
        sl = slice(sp * fixemul.V_CHUNK, (sp + 1) * fixemul.V_CHUNK)
        c = sp * fixemul.V_CHUNK // fixemul.K_CHUNK
        for p in range(3):
            for q in range(3):
                S = dV[q][:, sl].astype(np.float64) @ dK[p][:, sl].T.astype(np.float64)   # exact: |S| < 2^24
                assert np.abs(S).max() < 2 ** 24
                terms.append(np.ldexp(S, eV[:, sp][:, None] + eK[:, c][None, :] - 14 - 8 * (p + q)))
    T = np.stack(terms, -1)
    exact = np.array([[math.fsum(T[n, m]) for m in range(3 * N)] for n in range(B)])
    scale = np.abs(T).sum(-1)
    rel = np.abs(got - exact) / scale
    assert rel.max() < 1e-12, rel.max()


def _physical(cuda, N_side=(40, 20), B=8, seed=0):
    nx, nz = N_side
    nodes, tris = mesh.planar_fault(float(nx), float(nz), nx, nz)
    K64, _ = gf.assemble_dense(nodes, tris, MU, MU, device=cuda)
    N = tris.shape[0]
    _, xg = mesh.element_frames(nodes, tris)
    tabs = mesh.ensemble_tables(xg, nx * 1e3, nz * 1e3, B=B, seed=seed, v_nuc=1e-3)
    return K64, tabs, N, xg


@pytest.mark.parametrize("ordered", [False, True])
def test_fix_product_matches_model_and_fp64(cuda, ordered):
    """The physical operator (planar N=1,600, four chunks) against a slip-rate
    deficit with a nucleation patch and magnitudes over 10 decades, in the
    mesh order and in the compact cluster-tree order: equal to the NumPy model
    of the slices to 1e-12 (every slot sum is exact; what remains is the
    float-float addition of the span sums), and to the FP64 product to 5e-9
    normwise per run (the operator's 32 bits per chunk; the FP32 operator is
    ~1e-8, BF16x6 ~1e-6)."""
    K64, tabs, N, xg = _physical(cuda)
    B = tabs.shape[0]
    rng = np.random.default_rng(3)
    V = np.zeros((B, 2 * N))
    V[:, 0::2] = (tabs[:, :, 7] - 1e-9) * 10 ** rng.uniform(-3, 0, size=(B, N))
    V[:, 1::2] = 1e-9 * rng.standard_normal((B, N))
    K = K64.cpu().numpy()
    out, err, P = _run_product(cuda, K, V, 4, xg if ordered else None)
    assert err == 0
    got = (out[..., 0].astype(np.float64) + out[..., 1]).sum(0)[:B]
    if ordered:
        order = P.order.cpu().numpy()
        assert sorted(order.tolist()) == list(range(N))
        rows = (3 * order[:, None] + np.arange(3)).ravel()
        cols = (2 * order[:, None] + np.arange(2)).ravel()
        model = np.empty((B, 3 * N))
        model[:, rows] = fixemul.product(K[np.ix_(rows, cols)], V[:, cols])
        g = np.empty_like(got)
        g[:, rows] = got
        got = g
    else:
        model = fixemul.product(K, V)
    ref = V @ K.T
    for r in range(B):
        assert normwise_rel(model[r], got[r]) < 1e-12, r
        assert normwise_rel(ref[r], got[r]) < 5e-9, r


def test_fix_product_k_slices_and_padding(cuda):
    """nsplit 1, 5 and 19 (slices that cut spans) agree to float-float
    precision (the span sums are exact; only their addition order changes);
    padded runs and padded rows come out zero."""
    rng = np.random.default_rng(4)
    N, B = 700, 5
    K = rng.standard_normal((3 * N, 2 * N)) * 1e8
    V = rng.standard_normal((B, 2 * N)) * 10 ** rng.uniform(-9, 0, size=(B, 2 * N))
    res = {}
    for ns in (1, 5, 19):
        out, err, _ = _run_product(cuda, K, V, ns)
        assert err == 0
        assert np.all(out[:, B:] == 0.0)
        res[ns] = (out[..., 0].astype(np.float64) + out[..., 1]).sum(0)[:B]
    ref = V @ K.T
    for r in range(B):
        assert normwise_rel(res[1][r], res[5][r]) < 1e-12
        assert normwise_rel(res[1][r], res[19][r]) < 1e-12
        assert normwise_rel(ref[r], res[1][r]) < 1e-8


def test_fix_product_balanced_grid(cuda):
    """N = 1,600 (38 row tiles x 100 blocks): with 4 or more output slices a
    GB300's 152 SMs take the balanced grid (one CTA per SM, equal shares of
    the tile-major blocks, a tile's share per CTA in its own slice, unused
    slices zeroed); with 1 or 3 the grid of (tile, K slice) CTAs.  Every
    schedule gives the same sums to float-float precision, and padded runs
    stay zero in every slice."""
    rng = np.random.default_rng(5)
    N, B = 1600, 40
    K = rng.standard_normal((3 * N, 2 * N)) * 1e8
    V = rng.standard_normal((B, 2 * N)) * 10 ** rng.uniform(-9, 0, size=(B, 2 * N))
    res = {}
    for ns in (1, 3, 4, 8):
        out, err, _ = _run_product(cuda, K, V, ns)
        assert err == 0
        assert np.all(out[:, B:] == 0.0)
        assert np.all(np.isfinite(out))
        res[ns] = (out[..., 0].astype(np.float64) + out[..., 1]).sum(0)[:B]
    ref = V @ K.T
    for r in range(B):
        for ns in (3, 4, 8):
            assert normwise_rel(res[1][r], res[ns][r]) < 1e-12, (ns, r)
        assert normwise_rel(ref[r], res[1][r]) < 1e-8


def test_fix_rejects_bad_arguments(cuda):
    L = _lib.load()
    buf = torch.zeros(1 << 16, dtype=torch.uint8, device=cuda)
    p = buf.data_ptr()
    assert L.pq3d_batch_gemm_bf16x18(p, p, 16, 65, 1, p, p, 256, None) == _lib.PQ3D_ERR_ARG   # B > 64
    assert L.pq3d_batch_gemm_bf16x18(p, p, 16, 16, 0, p, p, 256, None) == _lib.PQ3D_ERR_ARG   # nsplit 0
    assert L.pq3d_batch_gemm_bf16x18(p, p, 16, 16, 2, p, p, 16, None) == _lib.PQ3D_ERR_ARG    # workspace
    assert L.pq3d_batch_pack_rhs_fix(p, 16, 65, None, p, None) == _lib.PQ3D_ERR_ARG


def _rates64(K64, ens):
    """K.v' in FP64 for the ensemble's current slip rates (cell order)."""
    v = torch.empty((ens.B, 2 * ens.N), dtype=torch.float64, device=K64.device)
    v[:, 0::2] = ens.t["slipv1"] - 1e-9 * ens.t["cos_rake0"]
    v[:, 1::2] = ens.t["slipv2"] - 1e-9 * ens.t["sin_rake0"]
    return (K64 @ v.T).T.cpu().numpy()


def test_batched_fix_tracks_fp64_through_nucleation(cuda):
    """Lockstep with the FP64 batched stepper (same step sizes and decisions)
    on planar N=1,600, 8 runs with nucleation patches, 120 accepted steps:
    the BF16x18 product with the FP64 attempt stays within 2e-6 in slip of the
    FP64 stepper (NumPy model of the same arithmetic: 2.3e-7 at step 80; the
    BF16x6 product leaves 1e-5 within ~45 steps here)."""
    K64, tabs, N, xg = _physical(cuda)
    kw = dict(mu=MU, Cs=CS, max_steps=120)
    ref = Ensemble(K64, tabs, precision="fp64", **kw)
    fix = Ensemble(PackedFixOperator(K64, xg), tabs, precision="bf16x18", attempt="fp64", **kw)
    # the ensemble's own product (packed v' in the compact order), read back in
    # the cell order, against FP64 on the same state
    L = _lib.load()
    _lib.check(L.pq3d_batch_gemm_bf16x18(fix.K.data_ptr(), fix.vop.data_ptr(), N, fix.B, fix.nsplit,
                                         fix.t["rates"].data_ptr(), fix.ws.data_ptr(), fix.ws.numel(),
                                         torch.cuda.current_stream().cuda_stream))
    got = fix.traction_rates().cpu().numpy()
    for ref_r, got_r in zip(_rates64(K64, ref), got):
        assert normwise_rel(ref_r, got_r) < 5e-9
    res = lockstep(ref, {"bf16x18": fix}, 120, bar=2e-6)
    r = res["bf16x18"]
    assert r["failed_runs"] == 0 and fix.error_word() == 0
    assert r["steps_within"] >= 120, r


def test_bf16x18_horizon_on_the_batched_workload(cuda):
    """The batched workload itself (planar 100 x 50 km, N = 10,000, per-run
    friction draws, nucleation patches at 1e-3 m/s), 8 runs in lockstep with
    the FP64 batched stepper: the BF16x18 product with the FP64 attempt keeps
    every run's slip within 1e-5 of FP64 for 80 accepted steps, through the
    nucleation (the BF16x6 and FP32 products leave 1e-5 at ~25 steps here; the
    FP64 stepper with its initial slip rates perturbed by 1e-12 leaves it at
    ~120 on 16 runs, the problem's own conditioning floor)."""
    nodes, tris = mesh.planar_fault(100.0, 50.0, 100, 50)
    _, xg = mesh.element_frames(nodes, tris)
    tabs = mesh.ensemble_tables(xg, 100e3, 50e3, B=8, seed=0, v_nuc=1e-3)
    K64, _ = gf.assemble_dense(nodes, tris, MU, MU, fp32_copy=False, device=cuda)
    kw = dict(mu=MU, Cs=CS, max_steps=80)
    ref = Ensemble(K64, tabs, precision="fp64", **kw)
    fix = Ensemble(PackedFixOperator(K64, xg), tabs, precision="bf16x18", attempt="fp64", nsplit=5, **kw)
    r = lockstep(ref, {"bf16x18": fix}, 80, bar=1e-5)["bf16x18"]
    assert r["failed_runs"] == 0 and fix.error_word() == 0
    assert r["steps_within"] >= 80, r


@pytest.mark.parametrize("nsplit", [2, 4])
@pytest.mark.parametrize("attempt", ["ff", "fp64", "mixed"])
def test_update_packs_rhs_like_the_pack_kernel(cuda, attempt, nsplit):
    """In the mesh's cell order the update kernel writes the fixed-point
    slices of v' itself (accepted runs only; a rejected run's slip rates, and
    so its slices, are unchanged).  After iterations with rejections, packing
    every run afresh from the slip rates (the pack kernel, through prepare)
    leaves the packed right-hand side bit for bit as it was.  N = 1,600 (the
    last 256-column span is half full), 8 runs (padded to 32); 2 partial sums
    (the (tile, K slice) grid) and 4 (the balanced grid on 152 SMs)."""
    nodes, tris = mesh.planar_fault(40.0, 20.0, 40, 20)
    K64, _ = gf.assemble_dense(nodes, tris, MU, MU, fp32_copy=False, device=cuda)
    _, xg = mesh.element_frames(nodes, tris)
    tabs = mesh.ensemble_tables(xg, 40e3, 20e3, B=8, seed=3, v_nuc=1e-3)
    ens = Ensemble(PackedFixOperator(K64), tabs, mu=MU, Cs=CS, precision="bf16x18", attempt=attempt, nsplit=nsplit)
    ens.set_ctrl(dttry=10.0)   # a first step far too long: rejections follow
    ens.iterate(30)
    torch.cuda.synchronize()
    c = ens.read_ctrl()
    assert sum(x.attempts - x.steps for x in c) > 0   # some rejections happened
    packed = ens.vop.clone()
    ens.prepare()
    torch.cuda.synchronize()
    assert torch.equal(packed, ens.vop)
    assert ens.error_word() == 0
