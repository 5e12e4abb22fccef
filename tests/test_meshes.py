"""Synthetic meshes: sizes, closure and outward orientation (CPU)."""
import numpy as np
import pytest

from nihu_gb300 import meshes


def _check_closed_outward(nodes, elems):
    edges = {}
    for row in elems:
        nc = 3 if row[0] == meshes.TRIA_1 else 4
        idx = row[1:1 + nc]
        for a in range(nc):
            e = (int(idx[a]), int(idx[(a + 1) % nc]))
            edges[e] = edges.get(e, 0) + 1
    # every directed edge appears once and its reverse once: closed and consistently oriented
    for (a, b), c in edges.items():
        assert c == 1 and edges.get((b, a)) == 1
    cen, nrm = meshes.centroids_and_normals(nodes, elems)
    # divergence theorem: sum of (x . n) * area = 3 * volume > 0 for outward normals
    c = meshes.element_corners(nodes, elems)
    vol = 0.0
    for e in range(len(elems)):
        if elems[e, 0] == meshes.TRIA_1:
            a = 0.5 * np.linalg.norm(np.cross(c[e, 1] - c[e, 0], c[e, 2] - c[e, 0]))
        else:
            a = 0.5 * np.linalg.norm(np.cross(c[e, 2] - c[e, 0], c[e, 3] - c[e, 1]))
        vol += cen[e] @ nrm[e] * a / 3
    return vol


@pytest.mark.parametrize("s", [0, 1, 2, 3])
def test_icosphere(s):
    nodes, elems = meshes.icosphere(s)
    assert len(elems) == 20 * 4 ** s
    assert np.allclose(np.linalg.norm(nodes, axis=1), 1.0)
    vol = _check_closed_outward(nodes, elems)
    assert 0.6 * 4 / 3 * np.pi < vol <= 4 / 3 * np.pi


def test_cylinder_small():
    nodes, elems = meshes.cylinder(16, 6, 2)
    assert len(elems) == 16 * 6 + 2 * (16 + 32)
    vol = _check_closed_outward(nodes, elems)
    assert 0.8 * np.pi * 4 < vol < np.pi * 4 + 1e-9
    # planar quads
    c = meshes.element_corners(nodes, elems)
    n = np.cross(c[:, 1] - c[:, 0], c[:, 2] - c[:, 0])
    assert np.allclose(np.einsum("ij,ij->i", n, c[:, 3] - c[:, 0]), 0, atol=1e-12)


def test_cylinder_40k_count():
    nodes, elems = meshes.cylinder_40k()
    assert len(elems) == 40000
    assert np.all(elems[:, 0] == meshes.QUAD_1)


def _write_off(path, nodes, elems):
    """An OFF file as NiHu's reader takes it (nihu/interface/read_off_mesh.hpp):
    header, counts (nodes, faces, edges), coordinates, faces `n i0 .. i(n-1)`."""
    with open(path, "w") as f:
        f.write("OFF\n%d %d 0\n" % (len(nodes), len(elems)))
        for x in nodes:
            f.write("%.17g %.17g %.17g\n" % tuple(x))
        for e in elems:
            idx = [int(v) for v in e[1:] if v >= 0]
            f.write("%d %s\n" % (len(idx), " ".join(map(str, idx))))


def test_read_off_round_trip(tmp_path):
    from nihu_gb300 import meshes
    for name, (nodes, elems) in {"tria": meshes.icosphere(2), "quad": meshes.cylinder(8, 3, 2)}.items():
        p = tmp_path / (name + ".off")
        _write_off(p, nodes, elems)
        n2, e2 = meshes.read_off(p)
        assert np.array_equal(n2, nodes)
        assert np.array_equal(e2, elems)


def test_read_off_errors(tmp_path):
    from nihu_gb300 import meshes
    p = tmp_path / "bad.off"
    p.write_text("PLY\n3 1 0\n0 0 0\n1 0 0\n0 1 0\n3 0 1 2\n")
    with pytest.raises(RuntimeError):
        meshes.read_off(p)
    p.write_text("OFF\n5 1 0\n" + "0 0 0\n" * 5 + "5 0 1 2 3 4\n")
    with pytest.raises(RuntimeError):
        meshes.read_off(p)
