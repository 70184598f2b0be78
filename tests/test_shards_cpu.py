"""Receiver-row sharding of the dense stepping on CPU: the partition, and the
collective call sites (allgather of v', allreduce MAX of the error norms) run
as gloo ranks (world sizes 2 and 3) around oracle row shards; the sharded run
must take the same steps and give the same bits as one shard holding every
cell, and follow the oracle's unsharded stepper."""
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from pyquake3d_gb300.shards import InProcessExchange, iterate_sharded, receiver_partition
from tests.shard_cpu import OracleRowShard, gloo_worker, load_case
from tests.util import normwise_rel

ITERS = 60


def test_receiver_partition():
    assert receiver_partition(10, 3) == [(0, 4), (4, 7), (7, 10)]
    assert receiver_partition(8, 2) == [(0, 4), (4, 8)]
    assert receiver_partition(5, 5) == [(q, q + 1) for q in range(5)]
    for N, w in ((1000, 7), (64, 3), (3, 1)):
        b = receiver_partition(N, w)
        assert b[0][0] == 0 and b[-1][1] == N
        assert all(b[q][1] == b[q + 1][0] for q in range(w - 1))
        sizes = [c1 - c0 for c0, c1 in b]
        assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        receiver_partition(2, 3)


def _single(iters=ITERS, world=1):
    K, table, mu, rho = load_case()
    shards = [OracleRowShard(K, table, c0, c1, mu=mu, density=rho)
              for c0, c1 in receiver_partition(table.shape[0], world)]
    iterate_sharded(shards, InProcessExchange(), iters)
    return shards


def test_in_process_shards_match_one_shard():
    one = _single()[0]
    three = _single(world=3)
    assert all(s.steps == one.steps and s.attempts == one.attempts and s.h == one.h for s in three)
    assert np.array_equal(np.concatenate([s.st.slip1 for s in three]), one.st.slip1)


def test_one_shard_follows_oracle_stepper():
    """The phase-split stepping (one attempt per iteration) takes the oracle's
    steps; only the product's summation order differs (row sums vs BLAS)."""
    from oracle.stepping import DenseStepper
    one = _single()[0]
    K, table, mu, rho = load_case()
    ref = DenseStepper(K, table, mu=mu, density=rho)
    ref.run(one.steps)
    assert abs(ref.time - one.st.time) <= 1e-9 * ref.time
    assert normwise_rel(ref.slip1, one.st.slip1) < 1e-9


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("world", [2, 3])
def test_gloo_ranks_match_one_process(tmp_path, world):
    mp.spawn(gloo_worker, args=(world, _free_port(), ITERS, str(tmp_path)), nprocs=world, join=True)
    parts = [np.load(tmp_path / ("rank%d.npz" % q)) for q in range(world)]
    one = _single()[0]
    for p in parts:
        assert int(p["steps"]) == one.steps and int(p["attempts"]) == one.attempts
        assert float(p["time"]) == one.st.time and float(p["h"]) == one.h
    assert np.array_equal(np.concatenate([p["slip1"] for p in parts]), one.st.slip1)
    assert np.array_equal(np.concatenate([p["Tt1o"] for p in parts]), one.st.Tt1o)
