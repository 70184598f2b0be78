"""Receiver-row shards of the batched stepper on one GPU (the in-process
exchange; the collectives over torch.distributed are covered by the gloo
tests): three shards give the same bits as the unsharded ensemble, for the
FP64 and the FP32 product, on the golden mesh and on a 2,000-cell mesh."""
import numpy as np
import pytest
import torch

import oracle
from pyquake3d_gb300 import gf, mesh
from pyquake3d_gb300.ensemble import Ensemble
from pyquake3d_gb300.shards import InProcessExchange, iterate_sharded, make_shards
from tests.test_batch_gpu import CS, _tables

pytestmark = pytest.mark.gpu
MU = 32038120320.0


def _check(K, tabs, precision, world, iters, **kw):
    whole = Ensemble(K, tabs, mu=MU, Cs=CS, precision=precision, **kw)
    whole.iterate(iters)
    shards = make_shards(K, tabs, world, mu=MU, Cs=CS, precision=precision, **kw)
    iterate_sharded(shards, InProcessExchange(), iters)
    torch.cuda.synchronize()
    cw = whole.read_ctrl()
    for s in shards:
        cs = s.read_ctrl()
        for r in range(tabs.shape[0]):
            assert (cs[r].steps, cs[r].attempts, cs[r].time, cs[r].h) == \
                   (cw[r].steps, cw[r].attempts, cw[r].time, cw[r].h), r
    assert cw[0].steps > 10
    for k in ("slip1", "slip2", "Tt1o", "state", "slipv"):
        got = torch.cat([s.t[k] for s in shards], dim=1)
        assert torch.equal(got, whole.t[k]), k


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_shards_bitwise_golden(cuda, golden, precision):
    d = golden("dense_small.npz")
    g = golden("traj_small.npz")
    K = torch.as_tensor(gf.join_ops({k: d["planar_" + k] for k in oracle.OPS}), device=cuda).contiguous()
    if precision == "fp32":
        K = K.float().contiguous()
    _check(K, _tables(g, 3), precision, 3, 150)


@pytest.mark.parametrize("nsplit", [1, 9])
def test_shards_fp32_k_slices(cuda, golden, nsplit):
    """FP32 product on row shards (each shard: N = 21 or 22 of Nt = 64 cells,
    its K slices over all 2 Nt columns) with one slice and with more slices
    than the 4 column chunks: the same bits as the unsharded ensemble."""
    d = golden("dense_small.npz")
    g = golden("traj_small.npz")
    K = torch.as_tensor(gf.join_ops({k: d["planar_" + k] for k in oracle.OPS}), device=cuda).float().contiguous()
    _check(K, _tables(g, 3), "fp32", 3, 150, nsplit=nsplit)


def test_shards_bitwise_n2000(cuda):
    nodes, tris = mesh.planar_fault(40.0, 25.0, 40, 25)
    N = tris.shape[0]
    K, _ = gf.assemble_dense(nodes, tris, MU, MU, fp32_copy=False, device=cuda)
    _, xg = mesh.element_frames(nodes, tris)
    tabs = mesh.ensemble_tables(xg, 40e3, 25e3, 2, seed=1, v_nuc=1e-3)
    assert tabs.shape == (2, N, 10)
    _check(K, tabs, "fp64", 4, 80)


def test_shard_rejects_tensor_core_product(cuda, golden):
    d = golden("dense_small.npz")
    K = torch.as_tensor(gf.join_ops({k: d["planar_" + k] for k in oracle.OPS}), device=cuda).contiguous()
    tabs = _tables(golden("traj_small.npz"), 1)
    with pytest.raises(ValueError):
        Ensemble(K[:96].contiguous(), tabs[:, :32], mu=MU, Cs=CS, precision="bf16x6", shard=(0, 64))


def test_dist_exchange_over_nccl_world1(cuda, golden):
    """The torch.distributed exchange on device tensors (NCCL) with one rank
    (one GPU here): the collective calls run and the result equals the
    unsharded ensemble bitwise.  Several ranks are covered on CPU (gloo)."""
    import socket

    import torch.distributed as dist
    from pyquake3d_gb300.shards import DistExchange, receiver_partition
    if not dist.is_nccl_available():
        pytest.fail("NCCL backend missing")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    dist.init_process_group("nccl", init_method="tcp://127.0.0.1:%d" % port, rank=0, world_size=1)
    try:
        d = golden("dense_small.npz")
        g = golden("traj_small.npz")
        K = torch.as_tensor(gf.join_ops({k: d["planar_" + k] for k in oracle.OPS}), device=cuda).contiguous()
        tabs = _tables(g, 2)
        N = tabs.shape[1]
        whole = Ensemble(K, tabs, mu=MU, Cs=CS, precision="fp64")
        whole.iterate(60)
        bounds = receiver_partition(N, 1)
        shard = Ensemble(K, tabs, mu=MU, Cs=CS, precision="fp64", shard=(0, N))
        iterate_sharded([shard], DistExchange(bounds), 60)
        torch.cuda.synchronize()
        assert torch.equal(shard.t["slip1"], whole.t["slip1"])
        assert [c.steps for c in shard.read_ctrl()] == [c.steps for c in whole.read_ctrl()]
    finally:
        dist.destroy_process_group()
