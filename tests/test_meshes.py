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
