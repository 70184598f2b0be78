"""The allocation-free assembly entry point, pq3d_assemble_dense_noalloc.

It serves callers that cannot call cudaMalloc (device memory owned by the host
application's own pool, or loops that must not pay cudaMalloc's implicit
synchronisation): its scratch tables live in a fixed __device__ array of the
library instead of a caller workspace.  Called through the C ABI, twice in a
row on different meshes (the second, smaller call must not see the first
call's leftovers), and checked against pq3d_assemble_dense with a workspace
within the parity tolerance of the other GF tests (1e-10 normwise; the two
paths run the same kernels, so they agree bit for bit).  This file is
collected last so that a failure here cannot stop the other tests."""
import numpy as np
import pytest
import torch

from pyquake3d_gb300 import _lib, gf, mesh
from tests.util import normwise_rel

pytestmark = pytest.mark.gpu
MU = 32038120320.0
MAX_N = 32768


def _noalloc(L, nodes_t, tris_t, N, K64, K32):
    return L.pq3d_assemble_dense_noalloc(nodes_t.data_ptr(), tris_t.data_ptr(), N, 0, N, MU, MU, 0,
                                         K64.data_ptr(), K32.data_ptr(), torch.cuda.current_stream().cuda_stream)


def test_noalloc_matches_workspace_variant_on_two_calls(cuda):
    L = _lib.load()
    cases = [mesh.rough_fault(20.0, 10.0, 20, 20, seed=11, ratio=5e-3), mesh.planar_fault(12.0, 6.0, 12, 12)]
    for nodes, tris in cases:
        N = tris.shape[0]
        nodes_t, tris_t = gf.mesh_to_device(nodes, tris, cuda)
        K64 = torch.full((3 * N, 2 * N), float("nan"), dtype=torch.float64, device=cuda)
        K32 = torch.full((3 * N, 2 * N), float("nan"), dtype=torch.float32, device=cuda)
        rc = _noalloc(L, nodes_t, tris_t, N, K64, K32)
        assert rc == _lib.PQ3D_OK, L.pq3d_last_error()
        ref64, ref32 = gf.assemble_dense(nodes, tris, MU, MU, device=cuda)
        torch.cuda.synchronize()
        assert normwise_rel(ref64.cpu().numpy(), K64.cpu().numpy(), axis=1) < 1e-10
        assert normwise_rel(ref32.cpu().numpy(), K32.cpu().numpy(), axis=1) < 1e-6
        assert not torch.isnan(K64).any()


def test_noalloc_rejects_n_beyond_its_fixed_scratch(cuda):
    L = _lib.load()
    dummy = torch.zeros(16, dtype=torch.float64, device=cuda)
    tris = torch.ones(16, dtype=torch.int64, device=cuda)
    rc = L.pq3d_assemble_dense_noalloc(dummy.data_ptr(), tris.data_ptr(), MAX_N + 1, 0, MAX_N + 1, MU, MU, 0,
                                       dummy.data_ptr(), None, torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.PQ3D_ERR_ARG
    assert b"32768" in L.pq3d_last_error()


def test_noalloc_row_range_empty_range_and_halfspace(cuda):
    """A receiver-row range [row0, row1) inside the mesh (a caller's K64 then
    holds those rows only) equals the same rows of the workspace variant;
    row0 == row1 writes nothing; the half space is refused with
    PQ3D_ERR_UNSUPPORTED (the fixed array holds the full-space tables only)."""
    L = _lib.load()
    nodes, tris = mesh.rough_fault(16.0, 8.0, 16, 16, seed=5, ratio=5e-3)
    N = tris.shape[0]
    nodes_t, tris_t = gf.mesh_to_device(nodes, tris, cuda)
    ref64, _ = gf.assemble_dense(nodes, tris, MU, MU, device=cuda)
    st = torch.cuda.current_stream().cuda_stream
    r0, r1 = 37, 301
    K64 = torch.full((3 * (r1 - r0), 2 * N), float("nan"), dtype=torch.float64, device=cuda)
    rc = L.pq3d_assemble_dense_noalloc(nodes_t.data_ptr(), tris_t.data_ptr(), N, r0, r1, MU, MU, 0, K64.data_ptr(),
                                       None, st)
    assert rc == _lib.PQ3D_OK, L.pq3d_last_error()
    torch.cuda.synchronize()
    assert normwise_rel(ref64[3 * r0:3 * r1].cpu().numpy(), K64.cpu().numpy(), axis=1) < 1e-10
    sentinel = torch.full((6,), 7.0, dtype=torch.float64, device=cuda)
    rc = L.pq3d_assemble_dense_noalloc(nodes_t.data_ptr(), tris_t.data_ptr(), N, 5, 5, MU, MU, 0,
                                       sentinel.data_ptr(), None, st)
    assert rc == _lib.PQ3D_OK
    torch.cuda.synchronize()
    assert torch.all(sentinel == 7.0)
    rc = L.pq3d_assemble_dense_noalloc(nodes_t.data_ptr(), tris_t.data_ptr(), N, 0, N, MU, MU, 1, K64.data_ptr(),
                                       None, st)
    assert rc == _lib.PQ3D_ERR_UNSUPPORTED
