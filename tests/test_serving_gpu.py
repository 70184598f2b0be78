"""Serving loop on the GPU: every request completes, admission respects the
slots, and a request's result is the same alone and in the mix."""
import numpy as np
import pytest
import torch

from pyquake3d_gb300 import mesh
from pyquake3d_gb300.ensemble import Ensemble, PackedOperator
from pyquake3d_gb300.serving import YEAR, Request, Server, poisson_arrivals
from pyquake3d_gb300 import gf

pytestmark = pytest.mark.gpu
MU = 32038120320.0


def _meshes():
    out = []
    for k, (nx, nz) in enumerate(((16, 8), (24, 8))):
        L, W = nx * 0.5, nz * 0.5
        f = mesh.planar_fault if k % 2 == 0 else mesh.rough_fault
        nodes, tris = f(L, W, nx, nz)
        out.append({"nodes": nodes, "tris": tris, "L": L * 1e3, "W": W * 1e3})
    return out


def _requests(meshes, n, seed=0):
    arr = poisson_arrivals(n, 20.0, seed)
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n):
        m = i % len(meshes)
        _, xg = mesh.element_frames(meshes[m]["nodes"], meshes[m]["tris"])
        tab = mesh.ensemble_tables(xg, meshes[m]["L"], meshes[m]["W"], B=1, seed=int(rng.integers(1 << 30)),
                                   v_nuc=1e-3)[0]
        reqs.append(Request(rid=i, mesh=m, arrival_s=float(arr[i]), table=tab, span_s=float(rng.uniform(0.05, 0.2)) * YEAR))
    return reqs


def test_serving_completes_and_result_alone_equals_mix(cuda):
    meshes = _meshes()
    srv = Server(meshes, mu=MU, lam=MU, cs=3464.0, slots=4, budget_bytes=50e9, graph_iters=8, max_steps=400,
                 device=cuda, dense_max_n=10 ** 9)
    reqs = _requests(meshes, 10)
    res = srv.run(reqs, time_limit_s=120)
    assert res["completed"] == 10 and res["failed"] == 0
    assert np.isfinite(res["p99_time_to_result_s"])
    # request 3 alone, same operator, one active slot
    r = reqs[3]
    ens = srv.ens[r.mesh]
    alone = Ensemble(PackedOperator(gf.assemble_dense(meshes[r.mesh]["nodes"], meshes[r.mesh]["tris"], MU, MU,
                                                      fp32_copy=False, device=cuda)[0]),
                     r.table[None], mu=MU, Cs=3464.0, precision="bf16x6", t_end=r.span_s, max_steps=400,
                     nsplit=ens.nsplit)
    alone.iterate(r.attempts + 5)
    c = alone.read_ctrl()[0]
    assert c.steps == r.steps and c.attempts == r.attempts and c.time == r.sim_time


def test_serving_hmatrix_mesh_result_alone_equals_mix(cuda):
    """The same with the second mesh (N = 384) served through an H-matrix
    (dense_max_n below its size): its runs step through the masked H-matrix
    product (pq3d_hmat_apply_masked, free slots and finished runs skipped) in
    the mix, and a request replayed alone on the same H-matrix takes the same
    steps and attempts and reaches the same simulated time, bit for bit."""
    meshes = _meshes()
    srv = Server(meshes, mu=MU, lam=MU, cs=3464.0, slots=4, budget_bytes=50e9, graph_iters=8, max_steps=400,
                 device=cuda, dense_max_n=300, hmat_kw=dict(min_size=32, mini_leaf=32, eta=2.0, tol=1e-6))
    assert srv.kind[0] == "dense_bf16x6" and srv.kind[1] == "hmatrix"
    reqs = _requests(meshes, 10, seed=3)
    res = srv.run(reqs, time_limit_s=120)
    assert res["completed"] == 10 and res["failed"] == 0
    hreqs = [r for r in reqs if r.mesh == 1]
    assert len(hreqs) >= 3
    H = srv.ens[1].hmat
    for r in hreqs[:3]:
        alone = Ensemble(H, r.table[None], mu=MU, Cs=3464.0, precision="hmat", t_end=r.span_s, max_steps=400)
        alone.iterate(r.attempts + 5)
        c = alone.read_ctrl()[0]
        assert c.status == 0 and c.active == 0
        assert c.steps == r.steps and c.attempts == r.attempts and c.time == r.sim_time, r.rid


def test_serving_bf16x18_result_alone_equals_mix(cuda):
    """Dense meshes on the fixed-point BF16x18 product with the float-float attempt
    (dense_precision="bf16x18"): a request replayed alone on a one-run
    ensemble of the same packed operator and K slices takes the same steps
    and attempts and reaches the same simulated time, bit for bit (the v'
    exponents, slices and float-float sums are per run)."""
    from pyquake3d_gb300.ensemble import PackedFixOperator
    meshes = _meshes()
    srv = Server(meshes, mu=MU, lam=MU, cs=3464.0, slots=4, budget_bytes=50e9, graph_iters=8, max_steps=400,
                 device=cuda, dense_max_n=10 ** 9, dense_precision="bf16x18")
    assert all(k == "dense_bf16x18" for k in srv.kind.values())
    reqs = _requests(meshes, 8, seed=5)
    res = srv.run(reqs, time_limit_s=120)
    assert res["completed"] == 8 and res["failed"] == 0
    for r in reqs[:3]:
        ens = srv.ens[r.mesh]
        op = PackedFixOperator(gf.assemble_dense(meshes[r.mesh]["nodes"], meshes[r.mesh]["tris"], MU, MU,
                                                 fp32_copy=False, device=cuda)[0],
                               mesh.element_frames(meshes[r.mesh]["nodes"], meshes[r.mesh]["tris"])[1])
        alone = Ensemble(op, r.table[None], mu=MU, Cs=3464.0, precision="bf16x18", attempt="ff", t_end=r.span_s,
                         max_steps=400, nsplit=ens.nsplit)
        alone.iterate(r.attempts + 5)
        c = alone.read_ctrl()[0]
        assert c.status == 0 and c.active == 0
        assert c.steps == r.steps and c.attempts == r.attempts and c.time == r.sim_time, r.rid
