"""Fault meshes and per-cell friction tables for the benchmark workloads.

The reference reads gmsh v2 meshes (``src/readmsh.py:12-68``) and per-cell
parameter files (``src/QDsim_gpu.py:714-770``).  It ships no generator for
planar structured meshes or rough faults, so this module builds them:

* :func:`planar_fault` -- a vertical strike-slip fault in the plane y = 0,
  structured grid of rectangles, each split into two triangles.
* :func:`rough_fault` -- the same grid displaced to y = h(x, z), where h is a
  seeded Gaussian random field with a power-law spectrum (Hurst exponent H),
  scaled so that rms(h) = ratio * length.
* :func:`friction_table` -- the 10-column table of ``read_parameter``
  (``rake a b dc f0 Tt Tno V shear_rate normal_rate``) for the benchmark
  friction layout: a velocity-weakening rectangle over the central half of the
  fault, velocity-strengthening outside, a linear taper of ``a`` between them
  and a square nucleation patch.

Node coordinates are metres, ``tris`` are 1-based node indices as gmsh writes
them, and the node order makes the element normal (b-a)x(c-a) point to +y
(``src/readmsh.py:75-134`` with node-order flag False).
"""
from __future__ import annotations

import numpy as np

__all__ = ["planar_fault", "rough_fault", "friction_table", "ensemble_tables",
           "element_frames", "write_parameter_file", "write_msh_v2"]


def _grid(length_m: float, width_m: float, nx: int, nz: int):
    xs = np.linspace(-0.5 * length_m, 0.5 * length_m, nx + 1)
    zs = np.linspace(-width_m, 0.0, nz + 1)
    X, Z = np.meshgrid(xs, zs, indexing="ij")          # (nx+1, nz+1)
    return X, Z


def _tris(nx: int, nz: int) -> np.ndarray:
    """Two triangles per cell; node id = ix*(nz+1)+iz (0-based here)."""
    ix, iz = np.meshgrid(np.arange(nx), np.arange(nz), indexing="ij")
    n00 = (ix * (nz + 1) + iz).ravel()
    n10 = ((ix + 1) * (nz + 1) + iz).ravel()
    n01 = (ix * (nz + 1) + iz + 1).ravel()
    n11 = ((ix + 1) * (nz + 1) + iz + 1).ravel()
    # (b-a) x (c-a) . e_y > 0 for a fault in the x-z plane:
    # a=(0,0), b=(0,1)[z], c=(1,0)[x] -> (0,0,1)x(1,0,0) = (0,1,0)
    t1 = np.stack([n00, n01, n10], axis=1)
    t2 = np.stack([n10, n01, n11], axis=1)
    t = np.empty((2 * n00.size, 3), dtype=np.int64)
    t[0::2] = t1
    t[1::2] = t2
    return t + 1


def planar_fault(length_km: float, width_km: float, nx: int, nz: int):
    """Vertical planar fault; returns (nodes[Nn,3] m, tris[N,3] 1-based)."""
    X, Z = _grid(length_km * 1e3, width_km * 1e3, nx, nz)
    nodes = np.stack([X.ravel(), np.zeros(X.size), Z.ravel()], axis=1)
    return np.ascontiguousarray(nodes), _tris(nx, nz)


def rough_height(length_m: float, width_m: float, nx: int, nz: int,
                 hurst: float = 0.8, ratio: float = 1e-3, seed: int = 0) -> np.ndarray:
    """Self-affine Gaussian height field on the (nx+1, nz+1) node grid.

    Spectral synthesis: white Gaussian noise filtered by |k|^-(1+H) in 2-D
    (power spectrum ~ |k|^-(2+2H)), zero mean, then scaled to
    rms = ratio * length_m.
    """
    rng = np.random.default_rng(seed)
    mx, mz = nx + 1, nz + 1
    noise = rng.standard_normal((mx, mz))
    kx = np.fft.fftfreq(mx, d=length_m / nx)
    kz = np.fft.rfftfreq(mz, d=width_m / nz)
    KX, KZ = np.meshgrid(kx, kz, indexing="ij")
    k = np.sqrt(KX ** 2 + KZ ** 2)
    k[0, 0] = np.inf
    filt = k ** (-(1.0 + hurst))
    h = np.fft.irfft2(np.fft.rfft2(noise) * filt, s=(mx, mz))
    h -= h.mean()
    h *= ratio * length_m / np.sqrt(np.mean(h * h))
    return h


def rough_fault(length_km: float, width_km: float, nx: int, nz: int,
                hurst: float = 0.8, ratio: float = 1e-3, seed: int = 0):
    """Rough strike-slip fault y = h(x, z); returns (nodes, tris)."""
    L, W = length_km * 1e3, width_km * 1e3
    X, Z = _grid(L, W, nx, nz)
    H = rough_height(L, W, nx, nz, hurst, ratio, seed)
    nodes = np.stack([X.ravel(), H.ravel(), Z.ravel()], axis=1)
    return np.ascontiguousarray(nodes), _tris(nx, nz)


def element_frames(nodes: np.ndarray, tris: np.ndarray):
    """Receiver frames (e1, e2, n) and centroids, as ``src/readmsh.py:75-134``
    computes them with the node-order flag False.  Returns (frames[N,9], xg[N,3])."""
    a = nodes[tris[:, 0] - 1]
    b = nodes[tris[:, 1] - 1]
    c = nodes[tris[:, 2] - 1]
    xg = ((a + b) + c) / 3.0
    n = np.cross(b - a, c - a)
    n /= np.sqrt(np.sum(n * n, axis=1))[:, None]
    e1 = np.zeros_like(n)
    vert = np.abs(n[:, 2]) < 1
    e1[vert, 0] = n[vert, 1]
    e1[vert, 1] = -n[vert, 0]
    e1[vert] /= np.sqrt(e1[vert, 0] ** 2 + e1[vert, 1] ** 2)[:, None]
    e1[~vert, 0] = 1.0
    e2 = np.cross(n, e1)
    return np.ascontiguousarray(np.concatenate([e1, e2, n], axis=1)), xg


def friction_table(xg: np.ndarray, length_m: float, width_m: float, *,
                   a_vw: float = 0.004, a_vs: float = 0.04, b: float = 0.03,
                   dc: float = 0.14, f0: float = 0.6, sigma_mpa: float = 25.0,
                   vpl: float = 1e-9, v_nuc: float = 0.03, nuc_size_m: float | None = None,
                   taper_m: float | None = None, seed: int = 0) -> np.ndarray:
    """Per-cell table in the ``read_parameter`` layout (src/QDsim_gpu.py:714-770).

    Velocity-weakening rectangle |x| <= L/4, -3W/4 <= z <= -W/4; ``a`` rises
    linearly from ``a_vw`` to ``a_vs`` over ``taper_m`` (default L/20, i.e. 2 km
    on a 40 km fault) outside it.  A square nucleation patch of side
    ``nuc_size_m`` (default L/10) starts at ``v_nuc``; its position inside the
    weakening rectangle is drawn from ``seed``.  Column 5 (Tt) is recomputed by
    the reader from steady state and is written as 0.
    """
    N = xg.shape[0]
    L, W = length_m, width_m
    taper = L / 20.0 if taper_m is None else taper_m
    nuc = L / 10.0 if nuc_size_m is None else nuc_size_m
    x, z = xg[:, 0], xg[:, 2]
    # distance outside the weakening rectangle (0 inside)
    dx = np.maximum(np.abs(x) - 0.25 * L, 0.0)
    dz = np.maximum(np.maximum((-0.75 * W) - z, z - (-0.25 * W)), 0.0)
    dist = np.maximum(dx, dz)
    frac = np.clip(dist / taper, 0.0, 1.0)
    a = a_vw + (a_vs - a_vw) * frac
    rng = np.random.default_rng(seed)
    cx = rng.uniform(-0.25 * L + 0.5 * nuc, 0.25 * L - 0.5 * nuc)
    cz = rng.uniform(-0.75 * W + 0.5 * nuc, -0.25 * W - 0.5 * nuc)
    V = np.full(N, vpl)
    in_nuc = (np.abs(x - cx) <= 0.5 * nuc) & (np.abs(z - cz) <= 0.5 * nuc)
    V[in_nuc] = v_nuc
    tab = np.zeros((N, 10))
    tab[:, 0] = 0.0          # rake (radians)
    tab[:, 1] = a
    tab[:, 2] = b
    tab[:, 3] = dc
    tab[:, 4] = f0
    tab[:, 5] = 0.0          # Tt: recomputed from steady state by the reader
    tab[:, 6] = sigma_mpa
    tab[:, 7] = V
    tab[:, 8] = 0.0          # shear loading rate
    tab[:, 9] = 0.0          # normal loading rate
    return tab


def ensemble_tables(xg: np.ndarray, length_m: float, width_m: float, B: int, seed: int = 0,
                    a_vw: float = 0.004, **kw) -> np.ndarray:
    """B per-run friction tables for the batched ensemble.

    Per run r (drawn from ``seed``): (a-b) ~ U(-0.008, -0.002) inside the
    weakening rectangle (a fixed at ``a_vw``, so b = a - (a-b) there; b keeps
    its default outside), Dc lognormal with median 0.1 m and sigma_ln 0.3,
    sigma_n ~ U(20, 50) MPa, and an independent nucleation-patch location.
    Returns (B, N, 10).
    """
    rng = np.random.default_rng(seed)
    out = []
    for r in range(B):
        amb = rng.uniform(-0.008, -0.002)
        dc = float(np.exp(np.log(0.1) + 0.3 * rng.standard_normal()))
        sig = rng.uniform(20.0, 50.0)
        nseed = int(rng.integers(0, 2 ** 31 - 1))
        t = friction_table(xg, length_m, width_m, a_vw=a_vw, dc=dc, sigma_mpa=sig, seed=nseed, **kw)
        vw = t[:, 1] <= a_vw + 1e-12
        t[vw, 2] = a_vw - amb
        out.append(t)
    return np.stack(out)


def write_parameter_file(path: str, table: np.ndarray) -> None:
    """Write a table in the whitespace-separated layout ``read_parameter`` reads."""
    np.savetxt(path, table, fmt="%.17e")


def write_msh_v2(path: str, nodes: np.ndarray, tris: np.ndarray) -> None:
    """Minimal gmsh v2 ASCII writer (coordinates in km, as ``read_mshV2`` scales by 1e3)."""
    with open(path, "w") as f:
        f.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n%d\n" % len(nodes))
        for i, p in enumerate(nodes / 1e3):
            f.write("%d %.17g %.17g %.17g\n" % (i + 1, p[0], p[1], p[2]))
        f.write("$EndNodes\n$Elements\n%d\n" % len(tris))
        for i, t in enumerate(tris):
            f.write("%d 2 2 0 1 %d %d %d\n" % (i + 1, t[0], t[1], t[2]))
        f.write("$EndElements\n")


def read_mshV2(fname: str):
    """gmsh v2 ASCII reader with the reference's semantics
    (src/readmsh.py:12-68): node coordinates in km -> metres; elements are the
    lines of the $Elements section with at least 8 fields, their last three
    integers the (1-based) vertex tags.  Returns (nodes[Nn,3], tris[N,3])."""
    nodes, tris = [], []
    section = None
    with open(fname) as f:
        for raw in f:
            line = raw.strip()
            if line.startswith("$"):
                section = {"$Nodes": "nodes", "$Elements": "elements"}.get(line)
                first = True
                continue
            if section is None:
                continue
            if first:                      # the count line
                first = False
                continue
            parts = line.split()
            if section == "nodes" and len(parts) >= 4:
                nodes.append([float(parts[1]), float(parts[2]), float(parts[3])])
            elif section == "elements" and len(parts) >= 8:
                tris.append([int(parts[-3]), int(parts[-2]), int(parts[-1])])
    return np.asarray(nodes, dtype=np.float64) * 1e3, np.asarray(tris, dtype=np.int64)


# Cell fields of a snapshot, in the reference's order and names
# (src/QDsim_gpu.py:1927-2073): (VTK name, state key, scale, format).
VTK_FIELDS = (
    ("Normal_[MPa]", "Tno", 1.0, "%f"), ("Pore_pressure[MPa]", "P", 1e-6, "%f"), ("Shear_[MPa]", "Tt", 1.0, "%f"),
    ("Shear_1[MPa]", "Tt1o", 1.0, "%f"), ("Shear_2[MPa]", "Tt2o", 1.0, "%f"),
    ("rake[Degree]", "rake", 180.0 / np.pi, "%f"), ("state", "state", 1.0, "%f"),
    ("Slipv[m/s]", "slipv", 1.0, "%.20f"), ("Slipv1[m/s]", "slipv1", 1.0, "%.20f"),
    ("Slipv2[m/s]", "slipv2", 1.0, "%.20f"), ("a", "a", 1.0, "%f"), ("b", "b", 1.0, "%f"),
    ("a-b", "a-b", 1.0, "%f"), ("dc", "dc", 1.0, "%f"), ("fric", "fric", 1.0, "%f"),
    ("slip", "slip", 1.0, "%.20f"), ("slip1", "slip1", 1.0, "%.20f"), ("slip2", "slip2", 1.0, "%.20f"))


def write_vtk(fname: str, nodes: np.ndarray, tris: np.ndarray, fields: dict) -> None:
    """Legacy ASCII VTK unstructured grid of triangles with the snapshot's
    cell fields (host arrays; ``fields`` keyed by the state names of
    VTK_FIELDS, ``a-b`` derived when absent, ``P`` zero when absent)."""
    nodes = np.asarray(nodes, dtype=np.float64)
    tris = np.asarray(tris, dtype=np.int64)
    N = tris.shape[0]
    f = dict(fields)
    f.setdefault("P", np.zeros(N))
    if "a-b" not in f:
        f["a-b"] = np.asarray(f["a"]) - np.asarray(f["b"])
    with open(fname, "w") as out:
        out.write("# vtk DataFile Version 3.0\ntest\nASCII\nDATASET  UNSTRUCTURED_GRID\n")
        out.write("POINTS %d float\n" % nodes.shape[0])
        np.savetxt(out, nodes, fmt="%f")
        out.write("CELLS %d %d\n" % (N, 4 * N))
        np.savetxt(out, np.column_stack([np.full(N, 3), tris - 1]), fmt="%d")
        out.write("CELL_TYPES %d\n" % N)
        out.write("5 " * N + "\n")
        out.write("CELL_DATA %d " % N)
        for name, key, scale, fmt in VTK_FIELDS:
            out.write("SCALARS %s float\nLOOKUP_TABLE default\n" % name)
            vals = np.asarray(f[key], dtype=np.float64) * scale
            out.write(" ".join(fmt % v for v in vals) + " \n")


def read_vtk_cell_data(fname: str) -> dict:
    """The SCALARS blocks of a file written by :func:`write_vtk` (for checks)."""
    out = {}
    lines = open(fname).read().split("\n")
    for i, line in enumerate(lines):
        if "SCALARS " in line:        # the first one shares its line with CELL_DATA, as the reference writes it
            out[line.split("SCALARS ")[1].split()[0]] = np.array([float(v) for v in lines[i + 2].split()])
    return out
