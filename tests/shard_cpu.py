"""CPU row shard used by the sharding tests: the oracle's stepping restricted
to a range of cells, behind the phase interface of pyquake3d_gb300.shards
(begin / error words / end / v' of all cells).  Test infrastructure only."""
from __future__ import annotations

import os

import numpy as np
import torch

from oracle.stepping import DenseStepper, StepFailure

OPS = ("A1s", "A2s", "Bs", "A1d", "A2d", "Bd")


def _rowdot(A, x):
    # one pairwise sum per row: the same bits whatever rows the shard holds
    return (A * x[None, :]).sum(axis=1)


class OracleRowShard:
    def __init__(self, K, table, c0, c1, *, mu, density, dttry=1e-3, V0=1e-6, Vpl=1e-9):
        N = table.shape[0]
        self.cell0, self.N, self.N_total, self.B = c0, c1 - c0, N, 1
        self.st = DenseStepper({k: np.ascontiguousarray(K[k][c0:c1]) for k in OPS}, table[c0:c1], mu=mu,
                               density=density, V0=V0, Vpl=Vpl)
        self.vp = torch.zeros((1, 2 * N), dtype=torch.float64)
        self.words = torch.zeros((1, 2), dtype=torch.int64)
        self.h, self.nrjct, self.steps, self.attempts = float(dttry), 0, 0, 0
        self.cand = None
        self._write_vprime()

    def _write_vprime(self):
        st = self.st
        v = self.vp[0].numpy()
        a = 2 * self.cell0
        v[a:a + 2 * self.N:2] = st.slipv1 - st.Vpl_con * np.cos(st.rake0)
        v[a + 1:a + 2 * self.N:2] = st.slipv2 - st.Vpl_con * np.sin(st.rake0)

    def vprime(self):
        return self.vp

    def error_words(self):
        return self.words.clone()

    def set_error_words(self, w):
        self.words.copy_(w)

    def begin(self):
        st = self.st
        v = self.vp[0].numpy()
        v1, v2 = v[0::2], v[1::2]
        st.AdotV1 = _rowdot(st.K["A1s"], v1) + _rowdot(st.K["A1d"], v2)
        st.AdotV2 = _rowdot(st.K["A2s"], v1) + _rowdot(st.K["A2d"], v2)
        st.dsigmadt = _rowdot(st.K["Bs"], v1) + _rowdot(st.K["Bd"], v2) + st.normal_loading
        *y, m1, m2 = st.rk_attempt_raw(self.h)
        self.cand = y
        self.words[0] = torch.from_numpy(np.array([m1, m2], dtype=np.float64).view(np.int64))

    def end(self):
        m1, m2 = self.words[0].numpy().view(np.float64)
        h = self.h
        c1, c2, hn1, hn2 = DenseStepper.step_control(h, float(m1), float(m2))
        self.attempts += 1
        if max(c1, c2) < 1.0 and not (np.isnan(c1) or np.isnan(c2)):
            self.st.accept(h, *self.cand)
            self.steps += 1
            self.nrjct = 0
            self.h = min(1.5 * h, min(hn1, hn2))
            self._write_vprime()
        else:
            self.nrjct += 1
            self.h = max(0.5 * h, min(hn1, hn2))
            if self.h < 1.e-15 or self.nrjct > 20:
                raise StepFailure("dt is too small")


def load_case():
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    d = np.load(os.path.join(here, "dense_small.npz"))
    g = np.load(os.path.join(here, "traj_small.npz"))
    K = {k: d["planar_" + k] for k in OPS}
    return K, g["table"], float(g["mu"]), float(g["rho"])


def gloo_worker(rank, world, port, iters, outdir):
    """One rank of a gloo run: its shard, the collectives over torch.distributed."""
    import torch.distributed as dist

    from pyquake3d_gb300.shards import DistExchange, iterate_sharded, receiver_partition
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        K, table, mu, rho = load_case()
        bounds = receiver_partition(table.shape[0], world)
        c0, c1 = bounds[rank]
        s = OracleRowShard(K, table, c0, c1, mu=mu, density=rho)
        iterate_sharded([s], DistExchange(bounds), iters)
        np.savez(os.path.join(outdir, "rank%d.npz" % rank), slip1=s.st.slip1, slip2=s.st.slip2, Tt1o=s.st.Tt1o,
                 time=s.st.time, steps=s.steps, attempts=s.attempts, h=s.h, c0=c0, c1=c1)
    finally:
        dist.destroy_process_group()
