"""Physical identities that pin the oracle's double-layer schemes
independently of the reference's code.

Gauss's integral: for a point on a flat face of a closed polyhedron,
int_S dG/dn_y dS_y = -1/2 exactly (G = 1/(4 pi r), outward normals), so the
rows of the collocational Laplace DLP matrix sum to -1/2, and those of the
Galerkin one to -area_i / 2, up to the quadrature error of the reference's
rules only (no discretisation error: the polyhedron is the surface).  The
sums run over every pair class: regular (1-point to 6-point rules),
nearly singular (semi-analytic static parts; polar schemes on quads) and
self terms.

The Laplace hypersingular operator annihilates constants (the double-layer
potential of a constant density is piecewise constant, so its normal
derivative vanishes): the collocational HSP rows sum to zero, which checks
the finite-part self term against the nearly singular and regular schemes.
"""
import numpy as np
import pytest

from nihu_gb300 import meshes
from oracle import oracle

MESHES = {
    "ico2": (lambda: meshes.icosphere(2), 1e-5, 1e-4),
    "ico3": (lambda: meshes.icosphere(3), 3e-5, None),
    "cyl": (lambda: meshes.cylinder(16, 8, 2, radius=1.0, length=3.0), 5e-4, 1e-3),
}


def areas(mesh):
    nodes, elems = mesh
    out = []
    for row in elems:
        nc = 3 if row[0] == 32303 else 4
        c = nodes[row[1:1 + nc]]
        if nc == 3:
            out.append(0.5 * np.linalg.norm(np.cross(c[1] - c[0], c[2] - c[0])))
        else:  # flat quads: half the cross product of the diagonals
            out.append(0.5 * np.linalg.norm(np.cross(c[2] - c[0], c[3] - c[1])))
    return np.array(out)


@pytest.mark.parametrize("name", sorted(MESHES))
def test_collocation_dlp_rows_sum_to_minus_half(name):
    make, tol, _ = MESHES[name]
    m = make()
    D = oracle.assemble(m, m, oracle.LAPLACE, oracle.DLP, 0.0, threads=8)
    assert np.abs(D.real.sum(axis=1) + 0.5).max() < tol


@pytest.mark.parametrize("name", [n for n in sorted(MESHES) if MESHES[n][2]])
def test_galerkin_dlp_rows_sum_to_minus_half_area(name):
    make, _, tol = MESHES[name]
    m = make()
    D = oracle.assemble_galerkin(m, m, oracle.LAPLACE, oracle.DLP, 0.0, threads=8)
    assert np.abs(D.real.sum(axis=1) / areas(m) + 0.5).max() < tol


@pytest.mark.parametrize("name", ["ico2", "ico3"])
def test_laplace_hsp_rows_sum_to_zero(name):
    m = MESHES[name][0]()
    H = oracle.assemble(m, m, oracle.LAPLACE, oracle.HSP, 0.0, threads=8)
    assert np.abs(H.real.sum(axis=1)).max() < 1e-5 * np.abs(np.diag(H)).max()
