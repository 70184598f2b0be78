"""The H-matrix partition (cluster tree + block tree, built on the device)
against the oracle's restatement of the reference rules and against the
reference's own partition recorded in tests/golden/hmatrix_small.npz."""
import os

import numpy as np
import pytest

from oracle import hmatrix as ohm
from pyquake3d_gb300 import mesh
from pyquake3d_gb300.hmatrix import build_partition

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "hmatrix_small.npz")


def _as_sets(perm, blocks):
    """Blocks as sorted index tuples (the renumbering orders a cluster's
    elements by depth-first leaf order, the reference by original order)."""
    return [(tuple(sorted(perm[b[0]:b[1]])), tuple(sorted(perm[b[2]:b[3]])), bool(b[4])) for b in blocks]


@pytest.mark.gpu
@pytest.mark.parametrize("which,params", [("planar", (16, 32)), ("rough", (16, 32)), ("rough", (64, 64)),
                                          ("planar", (8, 16)), ("rough", (1, 1))])
def test_partition_matches_oracle(cuda, which, params):
    if which == "planar":
        nodes, tris = mesh.planar_fault(30.0, 15.0, 30, 15)
    else:
        nodes, tris = mesh.rough_fault(24.0, 12.0, 40, 20, seed=2, ratio=5e-3)
    _, xg = mesh.element_frames(nodes, tris)
    perm, blocks, leaves = build_partition(xg, params[0], params[1], device=cuda)
    got = _as_sets(perm, blocks)
    ref = [(tuple(sorted(r)), tuple(sorted(c)), lr) for r, c, lr in ohm.leaf_blocks(xg, params[0], params[1])]
    assert got == ref
    # leaves tile [0, N), blocks tile the whole matrix
    assert leaves[0, 0] == 0 and leaves[-1, 1] == len(xg) and np.all(leaves[1:, 0] == leaves[:-1, 1])
    area = np.sum((blocks[:, 1] - blocks[:, 0]) * (blocks[:, 3] - blocks[:, 2]))
    assert area == len(xg) ** 2
    assert sorted(perm.tolist()) == list(range(len(xg)))


def test_oracle_partition_matches_reference_golden():
    if not os.path.exists(GOLDEN):
        pytest.fail("missing golden " + GOLDEN)
    g = np.load(GOLDEN)
    _, xg = mesh.element_frames(g["nodes"], g["tris"])
    ref = []
    for b in range(len(g["row_ptr"]) - 1):
        ref.append((tuple(g["rows"][g["row_ptr"][b]:g["row_ptr"][b + 1]]),
                    tuple(g["cols"][g["col_ptr"][b]:g["col_ptr"][b + 1]])))
    got = [(tuple(r), tuple(c)) for r, c, _ in ohm.leaf_blocks(xg, 16, int(g["mini_leaf"]))]
    assert got == ref
    lr = [lowrank for _, _, lowrank in ohm.leaf_blocks(xg, 16, int(g["mini_leaf"]))]
    assert np.array_equal(np.array(lr), g["aca"])


def test_low_rank_row_schedule_and_groups():
    """Host-side work lists of the low-rank product: short rows first (row
    order), long rows after; groups of up to 4 consecutive short rows of one
    block, each group one record (the first row's t_info, first row, size)."""
    import torch
    from pyquake3d_gb300.hmatrix import HMatrix
    H = HMatrix.__new__(HMatrix)
    H.device = torch.device("cpu")
    # four low-rank blocks (ids 1, 2, 4, 5 of 6): ranks 5, 3, 9, 1; block 4's rows are long
    rank = np.array([-1, 5, 3, -1, 9, 1], dtype=np.int32)
    lr = np.array([1, 2, 4, 5], dtype=np.int32)
    H.rank, H.lr_ids = torch.as_tensor(rank), torch.as_tensor(lr)
    ranks = rank[lr]
    H.t_rows = int(ranks.sum())
    Nc = np.concatenate([np.full(k, nc) for k, nc in zip(ranks, (300, 64, 20000, 8))]).astype(np.int64)
    info = np.stack([np.arange(H.t_rows, dtype=np.int64) * 1000, Nc << 32], 1)
    H._make_sched(info)
    sched = H.t_sched.numpy()
    short = np.nonzero(Nc <= H.LONG_ROW)[0]
    assert np.array_equal(sched[:len(short)], short) and H.t_nlong == 9
    assert np.array_equal(np.sort(sched[len(short):]), np.nonzero(Nc > H.LONG_ROW)[0])
    rec = H.t_grp.numpy()
    w0, g = rec[:, 1] >> 32, rec[:, 0] >> 56
    assert list(g) == [4, 1, 3, 1] and H.t_ngrp == 4
    assert np.array_equal(rec[:, 0] & (2 ** 40 - 1), info[w0, 0])
    assert np.array_equal((rec[:, 0] >> 40) & 0xffff, info[w0, 1] >> 32)
    assert np.array_equal(rec[:, 1] & 0xffffffff, info[w0, 1] & 0xffffffff)
    covered = np.concatenate([np.arange(a, a + n) for a, n in zip(w0, g)])
    assert np.array_equal(np.sort(covered), short)
    # rows of a group are consecutive rows of one block
    block_of = np.repeat(np.arange(len(lr)), ranks)
    for a, n in zip(w0, g):
        assert len(set(block_of[a:a + n])) == 1


@pytest.mark.gpu
def test_partition_reproduces_reference_golden(cuda):
    """The device partition on the mesh of the reference's own H-matrix
    (hmatrix_small.npz, min_size 16, mini_leaf 32): the same leaf blocks, in
    the same depth-first order, with the same ACA/dense split."""
    g = np.load(GOLDEN)
    _, xg = mesh.element_frames(g["nodes"], g["tris"])
    perm, blocks, _ = build_partition(xg, 16, int(g["mini_leaf"]), device=cuda)
    assert len(blocks) == len(g["row_ptr"]) - 1
    for b in range(len(blocks)):
        r0, r1, c0, c1, lr = blocks[b]
        assert sorted(perm[r0:r1]) == list(g["rows"][g["row_ptr"][b]:g["row_ptr"][b + 1]])
        assert sorted(perm[c0:c1]) == list(g["cols"][g["col_ptr"][b]:g["col_ptr"][b + 1]])
        assert bool(lr) == bool(g["aca"][b])
