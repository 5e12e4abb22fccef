"""The oracle's Galerkin formalism pinned by independent computations (CPU):
polynomial exactness of the singular Galerkin rules, the Laplace SLP and DLP
double integrals of matched triangle pairs against an outer subdivided rule
over the semi-analytic inner integral, the smooth Helmholtz remainder against
a plain product rule, and the pulsating sphere."""
import math

import numpy as np
import pytest

from oracle import oracle
from test_quad_rules import tri

TRIA = 32303
QUAD_ID = 32404


def exact_tri_moment(a, b):
    """integral of x^a y^b over the reference triangle (0,0),(1,0),(0,1)"""
    return math.factorial(a) * math.factorial(b) / math.factorial(a + b + 2)


@pytest.mark.parametrize("match", [2, 1, 0])
def test_singular_rules_integrate_polynomials(match):
    r = oracle.galerkin_rule(match)
    assert len(r) == {2: 1536, 1: 1536, 0: 512}[match]
    for a, b, c, d in [(0, 0, 0, 0), (1, 0, 0, 0), (0, 1, 1, 0), (2, 0, 0, 1), (1, 1, 1, 1), (0, 0, 3, 0)]:
        got = np.sum(r[:, 4] * r[:, 0] ** a * r[:, 1] ** b * r[:, 2] ** c * r[:, 3] ** d)
        want = exact_tri_moment(a, b) * exact_tri_moment(c, d)
        assert abs(got - want) <= 1e-12 * want, (match, a, b, c, d)


def subdivided_points(corners, levels):
    """(points, weights) of the degree-14 rule on 4^levels subtriangles"""
    tris = [np.asarray(corners, float)]
    for _ in range(levels):
        nxt = []
        for t in tris:
            m01, m12, m20 = (t[0] + t[1]) / 2, (t[1] + t[2]) / 2, (t[2] + t[0]) / 2
            nxt += [np.array([t[0], m01, m20]), np.array([m01, t[1], m12]), np.array([m20, m12, t[2]]),
                    np.array([m01, m12, m20])]
        tris = nxt
    q = tri(14)
    pts, ws = [], []
    for t in tris:
        J = np.linalg.norm(np.cross(t[1] - t[0], t[2] - t[0]))
        for xi, eta, w in q:
            pts.append(t[0] + xi * (t[1] - t[0]) + eta * (t[2] - t[0]))
            ws.append(w * J)
    return np.array(pts), np.array(ws)


def pair_matrix(nodes, elems, family, op, k):
    return oracle.assemble_galerkin((np.asarray(nodes, float), np.asarray(elems, np.int32)),
                                    (np.asarray(nodes, float), np.asarray(elems, np.int32)), family, op, k,
                                    same_mesh=True)


# a triangle, its neighbour across the edge 0-1 folded out of plane, and one
# sharing only node 2 (rotated copy), in the node-index conventions of a mesh
NODES = np.array([[0.0, 0.0, 0.0], [1.0, 0.1, 0.0], [0.3, 0.9, 0.0], [0.6, -0.7, 0.45], [-0.5, 1.4, 0.35],
                  [0.2, 1.6, -0.3]])
ELEMS = np.array([[TRIA, 0, 1, 2, -1], [TRIA, 1, 0, 3, -1], [TRIA, 2, 4, 5, -1]])


def inner_laplace(op, trial, x, nx=None):
    """(1/4 pi) int_trial 1/r (SLP) or its DLP kernel, semi-analytic static scheme"""
    return oracle.elem_integral(trial, x, oracle.LAPLACE, op, 0.0, kind=3).real


@pytest.fixture
def fine_angles():
    oracle.lib().oracle_set_static_gauss_points(21)
    yield
    oracle.lib().oracle_set_static_gauss_points(6)


@pytest.mark.parametrize("j,name", [(0, "face"), (1, "edge"), (2, "corner")])
@pytest.mark.parametrize("op", [oracle.SLP, oracle.DLP])
def test_laplace_matched_pairs_against_outer_inner_integration(fine_angles, j, name, op):
    G = pair_matrix(NODES, ELEMS, oracle.LAPLACE, op, 0.0)
    test = NODES[ELEMS[0, 1:4]]
    trial = NODES[ELEMS[j, 1:4]]
    pts, ws = subdivided_points(test, 3)
    ref = sum(w * inner_laplace(op, trial, x) for x, w in zip(pts, ws))
    if op == oracle.DLP and j == 0:
        assert abs(G[0, 0]) <= 1e-14  # flat element: r.n_y = 0
        return
    # the reference's n = 4 Duffy rules against outer/inner integration
    # converged to about 1e-7 (SLP) and 1e-5 (DLP): the tolerances are the
    # rules' own errors (SLP face 1.5e-5, edge 2.7e-5, corner 6e-7; DLP edge
    # 9.8e-4, where the folded neighbour's kernel is steepest, corner 1e-5)
    tol = {(oracle.SLP, "face"): 3e-5, (oracle.SLP, "edge"): 5e-5, (oracle.SLP, "corner"): 2e-6,
           (oracle.DLP, "edge"): 2e-3, (oracle.DLP, "corner"): 5e-5}[(op, name)]
    assert abs(G[0, j].real - ref) <= tol * abs(ref), (name, G[0, j], ref)
    assert G[0, j].imag == 0.0


def test_helmholtz_remainder_is_the_smooth_product_rule():
    """Helmholtz minus Laplace (a bounded kernel) through the singular rule
    against a subdivided product rule on both triangles."""
    k = 2.0
    H = pair_matrix(NODES, ELEMS, oracle.HELMHOLTZ, oracle.SLP, k)
    Lp = pair_matrix(NODES, ELEMS, oracle.LAPLACE, oracle.SLP, 0.0)
    test = NODES[ELEMS[0, 1:4]]
    for j in range(3):
        trial = NODES[ELEMS[j, 1:4]]
        px, wx = subdivided_points(test, 2)
        py, wy = subdivided_points(trial, 2)
        r = np.linalg.norm(px[:, None, :] - py[None, :, :], axis=2)
        f = np.where(r > 0, (np.exp(-1j * k * r) - 1) / np.maximum(r, 1e-300), -1j * k) / (4 * np.pi)
        ref = wx @ f @ wy
        # the n = 4 Duffy rules' own error on this bounded remainder: 1e-5
        # (face, where the product rule itself converges slowly) to 3e-5
        assert abs((H[0, j] - Lp[0, j]) - ref) <= 5e-5 * abs(ref), j


def test_regular_pairs_use_the_interval_degree():
    """Far pairs: the product of two one-point rules (centroid kernel times
    both areas), as the degree-0 Dunavant rule gives."""
    nodes = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [30, 0, 0], [31, 0, 0], [30, 1, 0.2]], float)
    elems = np.array([[TRIA, 0, 1, 2, -1], [TRIA, 3, 4, 5, -1]])
    G = pair_matrix(nodes, elems, oracle.HELMHOLTZ, oracle.SLP, 1.5)
    c0, c1 = nodes[:3].mean(0), nodes[3:].mean(0)
    a0 = 0.5
    a1 = 0.5 * np.linalg.norm(np.cross(nodes[4] - nodes[3], nodes[5] - nodes[3]))
    r = np.linalg.norm(c1 - c0)
    assert abs(G[0, 1] - a0 * a1 * np.exp(-1.5j * r) / (4 * np.pi * r)) <= 1e-14 * abs(G[0, 1])


def test_pulsating_sphere_galerkin():
    """(M - I/2) p = L q with the Galerkin identity (element areas): the
    pulsating-sphere case of the reference's own Galerkin test
    (nihu/test/stallone_unit/helmholtz_3d_pulsating_sphere_test.cpp:40-70)."""
    from nihu_gb300 import meshes
    mesh = meshes.icosphere(2)
    nodes, elems = mesh
    n = len(elems)
    c = nodes[elems[:, 1:4]]
    area = 0.5 * np.linalg.norm(np.cross(c[:, 1] - c[:, 0], c[:, 2] - c[:, 0]), axis=1)
    k = 1.0
    L = oracle.assemble_galerkin(mesh, mesh, oracle.HELMHOLTZ, oracle.SLP, k, threads=4)
    M = oracle.assemble_galerkin(mesh, mesh, oracle.HELMHOLTZ, oracle.DLP, k, threads=4)
    p = np.linalg.solve(M - 0.5 * np.diag(area), L @ np.ones(n))
    pa = -1.0 / (1.0 + 1j * k)
    assert np.abs(p - pa).max() / abs(pa) < 0.01
    # symmetric up to the quadrature: the Galerkin SLP of a closed surface
    assert np.abs(L - L.T).max() <= 1e-5 * np.abs(L).max()


@pytest.mark.parametrize("fam,k", [(oracle.HELMHOLTZ, 1.5), (oracle.LAPLACE, 0.0), (oracle.HELMHOLTZ, 2.0 - 0.3j)])
@pytest.mark.parametrize("op", [oracle.SLP, oracle.DLP])
def test_triangle_quad_matches_are_the_triangle_rules_on_the_split_quad(fam, k, op):
    """Triangle-quad matches (nihu/core/singular_galerkin_quadrature.hpp:624-790):
    the quad's reference square split into the triangles (0, 1, 2) and
    (0, 2, 3) of its rotated corners, the triangle-triangle corner and edge
    rules on them.  On a parallelogram (whose bilinear map is affine on each
    half) an entry equals the sum of the triangle-triangle entries of the
    mesh split along the same diagonal, to rounding: the quad's rotation
    puts corner 0 on the first common node, so an edge match with a quad
    trial element (whose rotation reverses the edge) splits along the other
    diagonal than a quad test element.  A quad test element, a triangle
    sharing its edge (P1, P0) and one sharing its corner P2."""
    T = TRIA
    P = np.array([[0, 0, 0], [1, 0, 0], [1.3, 0.9, 0], [0.3, 0.9, 0], [0.5, -0.8, 0.1], [2.0, 1.2, 0.2],
                  [1.5, 1.8, -0.1]], float)
    mixed = (P, np.array([[32404, 0, 1, 2, 3], [T, 1, 0, 4, -1], [T, 2, 5, 6, -1]], np.int32))
    split02 = (P, np.array([[T, 0, 1, 2, -1], [T, 0, 2, 3, -1], [T, 1, 0, 4, -1], [T, 2, 5, 6, -1]], np.int32))
    split13 = (P, np.array([[T, 0, 1, 3, -1], [T, 1, 2, 3, -1], [T, 1, 0, 4, -1], [T, 2, 5, 6, -1]], np.int32))
    M = oracle.assemble_galerkin(mixed, mixed, fam, op, k, same_mesh=True)
    A = oracle.assemble_galerkin(split02, split02, fam, op, k, same_mesh=True)
    B = oracle.assemble_galerkin(split13, split13, fam, op, k, same_mesh=True)
    pairs = [(M[0, 1], A[0, 2] + A[1, 2]),   # quad test, edge: rotated corner 0 = P0, diagonal P0-P2
             (M[1, 0], B[2, 0] + B[2, 1]),   # quad trial, edge: the reversed edge puts P1 first, diagonal P1-P3
             (M[0, 2], A[0, 3] + A[1, 3]),   # corner P2: diagonal P2-P0
             (M[2, 0], A[3, 0] + A[3, 1])]
    for got, ref in pairs:
        assert abs(got - ref) <= 1e-12 * abs(ref), (got, ref)


QUAD = 32404


@pytest.mark.parametrize("match", [2, 1, 0])
def test_quad_singular_rules_integrate_polynomials(match):
    r = oracle.galerkin_rule(match, quad=True)
    assert len(r) == {2: 2048, 1: 1536, 0: 1280}[match]

    def m(a):  # integral of x^a over [-1, 1]
        return 0.0 if a % 2 else 2.0 / (a + 1)

    for a, b, c, d in [(0, 0, 0, 0), (2, 0, 0, 0), (1, 1, 1, 1), (2, 0, 0, 2), (0, 2, 2, 0), (3, 0, 1, 0)]:
        got = np.sum(r[:, 4] * r[:, 0] ** a * r[:, 1] ** b * r[:, 2] ** c * r[:, 3] ** d)
        assert abs(got - m(a) * m(b) * m(c) * m(d)) <= 1e-12 * 16, (match, a, b, c, d)


def square_points(corners, levels, n=8):
    """(points, weights) of an n x n Gauss rule on 4^levels sub-squares of a flat quad"""
    g, w = np.polynomial.legendre.leggauss(n)
    c = np.asarray(corners, float)
    pts, ws = [], []
    m = 2 ** levels
    for i in range(m):
        for j in range(m):
            for a, wa in zip(g, w):
                for b, wb in zip(g, w):
                    u = -1 + (2 * i + 1 + a) / m
                    v = -1 + (2 * j + 1 + b) / m
                    N = np.array([(1 - u) * (1 - v), (1 + u) * (1 - v), (1 + u) * (1 + v), (1 - u) * (1 + v)]) / 4
                    dNu = np.array([-(1 - v), (1 - v), (1 + v), -(1 + v)]) / 4
                    dNv = np.array([-(1 - u), -(1 + u), (1 + u), (1 - u)]) / 4
                    J = np.linalg.norm(np.cross(dNu @ c, dNv @ c))
                    pts.append(N @ c)
                    ws.append(wa * wb * J / m ** 2)
    return np.array(pts), np.array(ws)


QNODES = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [1, -0.9, 0.35], [0, -0.9, 0.35],
                   [2.0, 1.0, 0.4], [2.0, 2.0, 0.4], [1.0, 2.0, 0.0]], float)
QELEMS = np.array([[QUAD, 0, 1, 2, 3], [QUAD, 5, 4, 1, 0], [QUAD, 2, 6, 7, 8]], np.int32)


@pytest.mark.parametrize("j,name,tol", [(0, "face", 1e-4), (1, "edge", 1e-4), (2, "corner", 1e-5)])
def test_quad_laplace_slp_against_outer_inner_integration(fine_angles, j, name, tol):
    """Flat square with a folded edge neighbour and a corner neighbour: the
    n = 4 Duffy rules against outer Gauss over the semi-analytic inner integral."""
    G = oracle.assemble_galerkin((QNODES, QELEMS), (QNODES, QELEMS), oracle.LAPLACE, oracle.SLP, 0.0, same_mesh=True)
    pts, ws = square_points(QNODES[QELEMS[0, 1:5]], 3)
    trial = QNODES[QELEMS[j, 1:5]]
    ref = sum(w * oracle.elem_integral(trial, x, oracle.LAPLACE, oracle.SLP, 0.0, kind=3).real
              for x, w in zip(pts, ws))
    assert abs(G[0, j].real - ref) <= tol * abs(ref), (name, G[0, j], ref)


def test_pulsating_sphere_galerkin_quads():
    """The quad version of the reference's pulsating-sphere test (its mesh
    sphere_1_5.off is a quad sphere): a cube-sphere of 216 quads."""
    from nihu_gb300 import meshes
    mesh = meshes.cube_sphere(6)
    nodes, elems = mesh
    n = len(elems)
    import nihu_gb300 as g
    area = g.create_mesh(nodes, elems).areas()
    k = 1.0
    L = oracle.assemble_galerkin(mesh, mesh, oracle.HELMHOLTZ, oracle.SLP, k, threads=4)
    M = oracle.assemble_galerkin(mesh, mesh, oracle.HELMHOLTZ, oracle.DLP, k, threads=4)
    p = np.linalg.solve(M - 0.5 * np.diag(area), L @ np.ones(n))
    pa = -1.0 / (1.0 + 1j * k)
    assert np.abs(p - pa).max() / abs(pa) < 0.02
    assert np.abs(L - L.T).max() <= 1e-4 * np.abs(L).max()
