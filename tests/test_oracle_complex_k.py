"""The oracle's complex (lossy) wave numbers, pinned by holomorphy.

Every entry is a holomorphic function of the wave number: the quadrature
points and the pair classes do not depend on k, and the kernels are built
from e^{-ikr} and powers of ikr.  So central differences along Re k and
Im k must satisfy df/d(Im k) = i df/d(Re k) (Cauchy-Riemann).  A wrong sign
or a conjugate anywhere in a complex-k formula breaks this: collocation SLP,
DLP, DLPt and HSP over regular, nearly singular and self pairs (triangles;
quads by Duffy, polar and Telles schemes), and Galerkin SLP and DLP on
triangle, quad and mixed meshes.
"""
import numpy as np
import pytest

from nihu_gb300 import meshes
from oracle import oracle

TRIA, QUAD = 32303, 32404
K0 = 2.0 - 0.3j
H = 1e-5


def mixed_cylinder(n_theta=16, n_z=6):
    """A closed quad cylinder with every third side quad split in two
    triangles (coarser caps leave quad pairs whose inverse mapping does not
    converge, which the reference reports as an error too)."""
    nodes, elems = meshes.cylinder(n_theta, n_z, 2, radius=1.0, length=4.0)
    rows = []
    for e, row in enumerate(elems):
        if e < n_theta * n_z and e % 3 == 0:
            a, b, c, d = row[1:5]
            rows.append([TRIA, a, b, c, -1])
            rows.append([TRIA, a, c, d, -1])
        else:
            rows.append(list(row))
    return nodes, np.array(rows, dtype=np.int32)


def cauchy_riemann(f):
    dre = (f(K0 + H) - f(K0 - H)) / (2 * H)
    dim = (f(K0 + 1j * H) - f(K0 - 1j * H)) / (2 * H)
    return np.abs(dim - 1j * dre).max() / np.abs(dre).max()


@pytest.mark.parametrize("op", [oracle.SLP, oracle.DLP, oracle.DLPT, oracle.HSP])
def test_collocation_triangles(op):
    m = meshes.icosphere(1)
    assert cauchy_riemann(lambda k: oracle.assemble(m, m, oracle.HELMHOLTZ, op, k, threads=4)) < 1e-7


@pytest.mark.parametrize("op", [oracle.SLP, oracle.DLP])
def test_collocation_quads_and_mixed(op):
    m = mixed_cylinder()
    assert cauchy_riemann(lambda k: oracle.assemble(m, m, oracle.HELMHOLTZ, op, k, threads=4)) < 1e-7


@pytest.mark.parametrize("name", ["ico1", "mixed"])
@pytest.mark.parametrize("op", [oracle.SLP, oracle.DLP])
def test_galerkin(name, op):
    m = meshes.icosphere(1) if name == "ico1" else mixed_cylinder()
    assert cauchy_riemann(lambda k: oracle.assemble_galerkin(m, m, oracle.HELMHOLTZ, op, k, threads=4)) < 1e-7


def test_the_check_catches_a_conjugate():
    """A conjugated wave number (the classic slip) is not holomorphic."""
    m = meshes.icosphere(1)
    err = cauchy_riemann(lambda k: oracle.assemble(m, m, oracle.HELMHOLTZ, oracle.SLP, np.conj(k), threads=4))
    assert err > 0.1
