"""Mesh and snapshot I/O (host): gmsh v2 round trip with the reference
reader's conventions, and the VTK snapshot layout."""
import numpy as np

from pyquake3d_gb300 import mesh


def test_msh_v2_round_trip(tmp_path):
    nodes, tris = mesh.rough_fault(6.0, 3.0, 6, 3, seed=3)
    p = str(tmp_path / "f.msh")
    mesh.write_msh_v2(p, nodes, tris)
    n2, t2 = mesh.read_mshV2(p)
    assert np.array_equal(t2, tris)
    assert np.allclose(n2, nodes, rtol=0, atol=1e-9)


def test_msh_v2_reader_skips_non_triangles(tmp_path):
    """Lines of the $Elements section with fewer than 8 fields (points,
    lines with one tag) are not triangles (src/readmsh.py:45)."""
    p = tmp_path / "g.msh"
    p.write_text("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n3\n1 0 0 0\n2 1 0 0\n3 0 0 -1\n$EndNodes\n"
                 "$Elements\n3\n1 15 2 0 1 1\n2 1 2 0 1 1 2\n3 2 2 0 1 1 2 3\n$EndElements\n")
    n, t = mesh.read_mshV2(str(p))
    assert n.shape == (3, 3) and n[1, 0] == 1000.0
    assert t.tolist() == [[1, 2, 3]]


def test_vtk_snapshot_layout(tmp_path):
    nodes, tris = mesh.planar_fault(4.0, 2.0, 4, 2)
    N = tris.shape[0]
    rng = np.random.default_rng(0)
    fields = {k: rng.standard_normal(N) for _, k, _, _ in mesh.VTK_FIELDS if k not in ("a-b", "P")}
    p = str(tmp_path / "s.vtk")
    mesh.write_vtk(p, nodes, tris, fields)
    txt = open(p).read()
    assert txt.startswith("# vtk DataFile Version 3.0\n")
    assert "POINTS %d float" % nodes.shape[0] in txt and "CELLS %d %d" % (N, 4 * N) in txt
    got = mesh.read_vtk_cell_data(p)
    assert list(got) == [name for name, _, _, _ in mesh.VTK_FIELDS]
    assert np.allclose(got["rake[Degree]"], fields["rake"] * 180 / np.pi, atol=1e-5)
    assert np.allclose(got["a-b"], fields["a"] - fields["b"], atol=1e-5)
    assert np.allclose(got["Slipv[m/s]"], fields["slipv"], atol=1e-15)
    assert np.all(got["Pore_pressure[MPa]"] == 0)
