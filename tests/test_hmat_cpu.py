"""The CPU restatement of the H-matrix build and product used as the CPU
baseline (oracle/hmat_cpu.py): its generators against the oracle's dense
assembly, its ACA against the dense block, its per-block product against an
explicit dense product of the same storage."""
import numpy as np

import oracle
from oracle import hmat_cpu
from pyquake3d_gb300 import gf, mesh

MU = 32038120320.0


def _mesh():
    nodes, tris = mesh.rough_fault(20.0, 5.0, 40, 10, seed=1)
    frames, xg = hmat_cpu.element_frames(nodes, tris)
    return nodes, tris, frames, xg


def test_frames_and_generators_match_the_oracle_assembly():
    nodes, tris, frames, xg = _mesh()
    f2, x2 = mesh.element_frames(nodes, tris)
    assert np.array_equal(frames, f2) and np.array_equal(xg, x2)
    N = tris.shape[0]
    ri = np.nonzero(xg[:, 0] < -7000)[0]
    sj = np.nonzero(xg[:, 0] > 5000)[0]
    K = gf.join_ops({n: a for n, a in zip(oracle.OPS, oracle.assemble_dense(nodes, tris, MU, MU))})
    Kb = K.reshape(N, 3, N, 2)[np.ix_(ri, [0, 1, 2], sj, [0, 1])].reshape(3 * len(ri), 2 * len(sj))
    gen = hmat_cpu.BlockGen(nodes, tris, frames, xg, ri, sj, MU, MU)
    D = hmat_cpu.dense_block(gen)
    assert np.abs(D - Kb).max() <= 1e-12 * np.abs(Kb).max()
    # rows through the other generator (one receiver x all sources)
    for i in (0, 7, 3 * len(ri) - 1):
        assert np.abs(gen.row(i) - Kb[i]).max() <= 1e-12 * np.abs(Kb).max()


def test_aca_of_a_far_block_is_within_tolerance():
    nodes, tris, frames, xg = _mesh()
    ri = np.nonzero(xg[:, 0] < -7000)[0]
    sj = np.nonzero(xg[:, 0] > 5000)[0]
    D = hmat_cpu.dense_block(hmat_cpu.BlockGen(nodes, tris, frames, xg, ri, sj, MU, MU))
    gen = hmat_cpu.BlockGen(nodes, tris, frames, xg, ri, sj, MU, MU)
    k, U, V = hmat_cpu.aca_block(gen, 60, 1e-4)
    assert 5 < k < 60
    A = np.array(U).T @ np.array(V)
    assert np.linalg.norm(A - D) <= 5e-4 * np.linalg.norm(D)
    assert gen.evals >= k * (2 * len(sj) + len(ri))   # a row and a column per term


def test_per_block_product_equals_dense_product():
    rng = np.random.default_rng(0)
    N = 12
    blocks = np.array([[0, 6, 0, 6], [0, 6, 6, 12], [6, 12, 0, 12]])
    rank = np.array([-1, 2, -1])
    parts, off, H = [], [], np.zeros((3 * N, 2 * N))
    o = 0
    for (r0, r1, c0, c1), k in zip(blocks, rank):
        M, Nc = 3 * (r1 - r0), 2 * (c1 - c0)
        if k < 0:
            D = rng.standard_normal((M, Nc))
            parts.append(D.T.reshape(-1))          # column-major
            H[3 * r0:3 * r1, 2 * c0:2 * c1] = D
            size = M * Nc
        else:
            U = rng.standard_normal((M, k))
            V = rng.standard_normal((k, Nc))
            parts.append(np.concatenate([U.T.reshape(-1), V.reshape(-1)]))
            H[3 * r0:3 * r1, 2 * c0:2 * c1] = U @ V
            size = k * (M + Nc)
        off.append(o)
        o += size
    data = np.concatenate(parts)
    x = rng.standard_normal(2 * N)
    y = hmat_cpu.matvec(blocks, data, np.array(off), rank, x)
    assert np.allclose(y, H @ x, rtol=1e-12, atol=1e-12)
