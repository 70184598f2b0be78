"""CPU ORACLE -- test infrastructure only.

Restatement of PyQuake3D's H-matrix partition (cluster tree and block tree),
used by the tests to check the GPU H-matrix's partition:

  * bounding box, diameter, box distance, admissibility min(diam) <= eta*dist
                                  src/Hmatrix.py:68-113 (eta = 2.0, line 2090)
  * cluster tree: bisect the longest bounding-box axis at its midpoint,
    points <= midpoint go left, order kept; a leaf when <= min_size points or
    when one side would be empty   src/Hmatrix.py:153-192
  * block tree: a leaf block when admissible or when either cluster has
    <= mini_leaf points or a cluster has no children; else the four child
    pairs (left/right x left/right)  src/Hmatrix.py:2077-2142
  * low-rank (ACA) blocks: both sides > mini_leaf; others dense
                                  src/Hmatrix.py:1292-1344

Returns leaf blocks in the reference's depth-first order as (rows, cols)
index arrays of the original element numbering.
"""
from __future__ import annotations

import numpy as np


def _bbox(points, idx):
    p = points[idx]
    return p.min(axis=0), p.max(axis=0)


def admissible(points, tau, sigma, eta=2.0):
    a_t, b_t = _bbox(points, tau)
    a_s, b_s = _bbox(points, sigma)
    d_t = np.sqrt(np.sum((b_t - a_t) ** 2))
    d_s = np.sqrt(np.sum((b_s - a_s) ** 2))
    dist = np.sqrt(np.sum(np.maximum(0, a_s - b_t) ** 2 + np.maximum(0, a_t - b_s) ** 2))
    return min(d_t, d_s) <= eta * dist


class Node:
    def __init__(self, idx):
        self.idx = idx
        self.left = None
        self.right = None


def cluster_tree(idx, points, min_size=16):
    if len(idx) <= min_size:
        return Node(idx)
    lo = points.min(axis=0)
    hi = points.max(axis=0)
    j = int(np.argmax(hi - lo))
    g = (lo[j] + hi[j]) / 2
    m1 = points[:, j] <= g
    m2 = points[:, j] > g
    if m1.sum() == 0 or m2.sum() == 0:
        return Node(idx)
    n = Node(idx)
    n.left = cluster_tree(idx[m1], points[m1], min_size)
    n.right = cluster_tree(idx[m2], points[m2], min_size)
    return n


def leaf_blocks(xg, min_size=16, mini_leaf=32, eta=2.0):
    """Leaf blocks [(rows, cols, lowrank)] in depth-first order."""
    root = cluster_tree(np.arange(len(xg)), xg, min_size)
    out = []

    def rec(r, c):
        adm = admissible(xg, r.idx, c.idx, eta)
        if adm or len(r.idx) <= mini_leaf or len(c.idx) <= mini_leaf or \
                r.left is None or r.right is None or c.left is None or c.right is None:
            out.append((r.idx, c.idx, len(r.idx) > mini_leaf and len(c.idx) > mini_leaf))
            return
        rec(r.left, c.left)
        rec(r.left, c.right)
        rec(r.right, c.left)
        rec(r.right, c.right)

    rec(root, root)
    return out
