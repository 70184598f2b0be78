"""Bounded device waits: a wait whose partner never arrives gives up after its
iteration limit and reports PQ3D_ERR_TIMEOUT (where the reference would call
sys.exit or hang), every block returns, and the context stays usable."""
import numpy as np
import pytest
import torch

from pyquake3d_gb300 import _lib

pytestmark = pytest.mark.gpu


def test_grid_barrier_gives_up_when_a_block_never_arrives(cuda):
    L = _lib.load()
    ret = np.zeros(16, dtype=np.int32)
    rc = L.pq3d_selftest_barrier_timeout(16, 5, 2000, ret.ctypes.data)
    assert rc == _lib.PQ3D_ERR_TIMEOUT, L.pq3d_last_error()
    assert b"gave up" in L.pq3d_last_error()
    assert ret[5] == 3 and np.all(ret[np.arange(16) != 5] == 1)   # every block returned, none passed
    # all blocks arrive: the same barrier passes
    ret[:] = 0
    assert L.pq3d_selftest_barrier_timeout(16, -1, 2000, ret.ctypes.data) == _lib.PQ3D_OK
    assert np.all(ret == 2)
    torch.cuda.synchronize()
    assert float(torch.ones(4, device=cuda).sum()) == 4.0      # context still usable


def test_mbarrier_wait_gives_up_with_error_word(cuda):
    L = _lib.load()
    g = np.zeros(1, dtype=np.int32)
    rc = L.pq3d_selftest_mbar_timeout(1000, g.ctypes.data)
    assert rc == _lib.PQ3D_ERR_TIMEOUT, L.pq3d_last_error()
    assert g[0] == 128
    assert float(torch.ones(4, device=cuda).sum()) == 4.0
