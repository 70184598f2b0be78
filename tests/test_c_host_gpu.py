"""The library from a plain C host (include/pq3d.h and libpq3d.so only):
dense assembly into host buffers and the reference ABI TDstressFS_C, checked
against the CPU oracle; an error comes back as a status with a message."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from pyquake3d_gb300 import _lib, gf
from tests.util import normwise_rel

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def test_plain_c_host(cuda, tmp_path):
    lib = os.path.abspath(_lib.LIB_PATH)
    libdir = os.path.dirname(lib)
    exe = tmp_path / "c_host_check"
    subprocess.check_call(["gcc", "-O1", "-I", os.path.dirname(_lib.HEADER), os.path.join(HERE, "c_host_check.c"),
                           "-L", libdir, "-lpq3d", "-Wl,-rpath," + libdir, "-o", str(exe)])
    out = tmp_path / "out.bin"
    r = subprocess.run([str(exe), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    raw = out.read_bytes()
    N, n_nodes, bad, bad_text = np.frombuffer(raw[:32], dtype=np.int64)
    o = 32
    nodes = np.frombuffer(raw[o:o + 24 * n_nodes], dtype=np.float64).reshape(n_nodes, 3); o += 24 * n_nodes
    tris = np.frombuffer(raw[o:o + 24 * N], dtype=np.int64).reshape(N, 3); o += 24 * N
    K = np.frombuffer(raw[o:o + 48 * N * N], dtype=np.float64).reshape(3 * N, 2 * N); o += 48 * N * N
    stress = np.frombuffer(raw[o:o + 144], dtype=np.float64).reshape(3, 6); o += 144
    strain = np.frombuffer(raw[o:o + 144], dtype=np.float64).reshape(3, 6)
    mu = 3.2038120320e10
    ref = gf.join_ops({name: op for name, op in zip(oracle.OPS, oracle.assemble_dense(nodes, tris, mu, mu))})
    assert normwise_rel(ref, K) < 1e-10
    P = (np.array([0.0, 0.0, -1000.0]), np.array([1000.0, 0.0, -1000.0]), np.array([1000.0, 0.0, -2000.0]))
    so, eo = oracle.tdstress(np.array([500.0, 1500.0, -200.0]), np.array([300.0, -700.0, 50.0]),
                             np.array([-1500.0, -2500.0, -800.0]), *P, 1.0, 0.0, 0.0, mu, mu)
    assert normwise_rel(so, stress) < 1e-10 and normwise_rel(eo, strain) < 1e-10
    assert bad == _lib.PQ3D_ERR_ARG and bad_text == 1
