"""The oracle's Burton-Miller operators (DLPt, HSP) pinned by independent
computations: finite differences of the SLP / DLP kernels, the finite-part
integral of 1/r^3 over a flat triangle, and dense quadrature of the nearly
singular static parts (CPU only)."""
import numpy as np
import pytest
from scipy import integrate

from oracle import oracle

TRI = np.array([[0.0, 0.0, 0.0], [1.0, 0.1, 0.0], [0.3, 0.9, 0.0]])
NZ = np.array([0.0, 0.0, 1.0])


def _unit(v):
    v = np.asarray(v, dtype=float)
    return v / np.linalg.norm(v)


@pytest.mark.parametrize("family,k", [(oracle.HELMHOLTZ, 1.7), (oracle.LAPLACE, 0.0)])
def test_kernels_are_normal_derivatives(family, k):
    """DLPt = d/dn_x of SLP, HSP = d/dn_x of DLP (one-point rule, far point)."""
    x = np.array([2.3, -1.1, 0.8])
    nx = _unit([0.3, -0.2, 0.9])
    h = 1e-5

    def val(op, xx, n=None):
        return oracle.elem_integral(TRI, xx, family, op, k, kind=0, degree=0, nx=n)

    dlpt = val(oracle.DLPT, x, nx)
    fd = (val(oracle.SLP, x + h * nx) - val(oracle.SLP, x - h * nx)) / (2 * h)
    assert abs(dlpt - fd) <= 1e-7 * abs(dlpt)
    hsp = val(oracle.HSP, x, nx)
    fd = (val(oracle.DLP, x + h * nx) - val(oracle.DLP, x - h * nx)) / (2 * h)
    assert abs(hsp - fd) <= 1e-6 * abs(hsp)


def _rho(theta, c):
    """distance from c to the boundary of TRI (in its plane) along direction theta"""
    d = np.array([np.cos(theta), np.sin(theta)])
    best = np.inf
    for a, b in zip(TRI, np.roll(TRI, -1, axis=0)):
        e = b[:2] - a[:2]
        m = np.array([[d[0], -e[0]], [d[1], -e[1]]])
        t, s = np.linalg.solve(m, a[:2] - c[:2])
        if t > 0 and -1e-12 <= s <= 1 + 1e-12:
            best = min(best, t)
    return best


def test_hsp_self_static_is_the_finite_part_of_one_over_r_cubed():
    """Laplace HSP over a flat triangle from its centroid: n_x = n_y, r in the
    plane, so the kernel is 1/(4 pi r^3) and its finite part is
    -(1/4 pi) int dtheta / rho(theta)."""
    c = TRI.mean(axis=0)
    fp = -integrate.quad(lambda t: 1.0 / _rho(t, c), 0.0, 2 * np.pi, limit=400, epsabs=0, epsrel=1e-12)[0]
    got = oracle.elem_integral(TRI, c, oracle.LAPLACE, oracle.HSP, 0.0, kind=2, nx=NZ)
    assert abs(got.real * 4 * np.pi - fp) <= 1e-10 * abs(fp)
    assert got.imag == 0.0


@pytest.mark.parametrize("k", [0.5, 2.0])
def test_hsp_self_dynamic_part_against_polar_integration(k):
    """Helmholtz minus Laplace HSP self term = (k^2/2) IG0/(4 pi) plus the
    13-point integral of the bounded remainder; the remainder is checked
    against adaptive polar integration (the degree-7 rule's own error)."""
    c = TRI.mean(axis=0)
    h = oracle.elem_integral(TRI, c, oracle.HELMHOLTZ, oracle.HSP, k, kind=2, nx=NZ)
    lap = oracle.elem_integral(TRI, c, oracle.LAPLACE, oracle.HSP, 0.0, kind=2, nx=NZ)
    slp0 = oracle.elem_integral(TRI, c, oracle.LAPLACE, oracle.SLP, 0.0, kind=2)  # IG0 / (4 pi)

    def dyn(r):
        ikr = 1j * k * r
        if r < 1e-3:
            return -1j * k ** 3 * (1 / 3 - ikr * (1 / 8 - ikr * (1 / 30 - ikr * (1 / 144))))
        return (np.exp(-ikr) * (1 + ikr) - 1 + ikr * ikr / 2) / r ** 3

    def radial(t, part):
        f = lambda r: (dyn(r) * r).real if part == 0 else (dyn(r) * r).imag
        return integrate.quad(f, 0.0, _rho(t, c), epsabs=0, epsrel=1e-10, limit=200)[0]

    exact = complex(integrate.quad(lambda t: radial(t, 0), 0, 2 * np.pi, limit=200, epsrel=1e-10)[0],
                    integrate.quad(lambda t: radial(t, 1), 0, 2 * np.pi, limit=200, epsrel=1e-10)[0]) / (4 * np.pi)
    rest = h - lap - k * k / 2 * slp0
    # the oracle's remainder is the 13-point degree-7 sum, restated here
    from test_quad_rules import tri
    p0, p1, p2 = TRI
    J = np.linalg.norm(np.cross(p1 - p0, p2 - p0))
    mine = sum(w * J * dyn(np.linalg.norm(p0 + xi * (p1 - p0) + eta * (p2 - p0) - c)) for xi, eta, w in tri(7))
    assert abs(rest - mine / (4 * np.pi)) <= 1e-12 * abs(rest)
    # and that sum's own error: the remainder behaves like k^4 |r| at the
    # centroid (one of the rule's points), so the degree-7 rule of the
    # reference misses its real part by up to about 1 % at k = 2
    assert abs(rest - exact) <= 1.5e-2 * abs(exact)
    assert abs(rest.imag - exact.imag) <= 1e-6 * abs(exact)


def _dense(family, op, k, x0, nx, n=120):
    """Tensor Gauss-Legendre on the collapsed square: far from x0 the
    integrand is smooth, so this converges fast."""
    g, w = np.polynomial.legendre.leggauss(n)
    u, wu = (g + 1) / 2, w / 2
    p0, p1, p2 = TRI
    tot = 0.0
    for a, wa in zip(u, wu):
        for b, wb in zip(u, wu):
            xi, eta = a, (1 - a) * b
            jac = (1 - a)
            y = p0 + xi * (p1 - p0) + eta * (p2 - p0)
            tot += wa * wb * jac * _kernel(family, op, k, x0, nx, y)
    area2 = np.linalg.norm(np.cross(p1 - p0, p2 - p0))
    return tot * area2


def _kernel(family, op, k, x, nx, y):
    rv = y - x
    r = np.linalg.norm(rv)
    ik = 1j * k if family == oracle.HELMHOLTZ else 0.0
    g = np.exp(-ik * r) / (4 * np.pi * r)
    if op == oracle.DLPT:
        dg = -g * (1 + ik * r) / r
        return dg * (-rv @ nx) / r
    g3 = np.exp(-ik * r) / (4 * np.pi * r ** 3)
    f1 = -g3 * (1 + ik * r)
    f0 = g3 * (3 + ik * r * (3 + ik * r))
    return f0 * (-rv @ nx / r) * (rv @ NZ / r) - f1 * (nx @ NZ)


# tolerances are the reference schemes' own accuracy at 0.2 above the element:
# DLPt's static part uses 6 angular points per side, HSP's 21 (exact to 1e-6);
# the Helmholtz HSP difference K_k - K_0 still behaves like k^2 / r, which the
# 42-point rule of the dynamic part integrates to about 1e-4
@pytest.mark.parametrize("op,family,k,tol", [(oracle.DLPT, oracle.LAPLACE, 0.0, 3e-3),
                                             (oracle.DLPT, oracle.HELMHOLTZ, 1.3, 3e-3),
                                             (oracle.HSP, oracle.LAPLACE, 0.0, 1e-6),
                                             (oracle.HSP, oracle.HELMHOLTZ, 1.3, 2e-4)])
def test_nearly_singular_scheme_against_dense_quadrature(op, family, k, tol):
    """Points 0.2 above the triangle (the semi-analytic static part, plus the
    42-point dynamic part for Helmholtz)."""
    nx = _unit([0.2, -0.3, 1.0])
    for x0 in ([0.4, 0.3, 0.2], [1.2, 0.6, -0.2], [0.5, -0.3, 0.2]):
        x0 = np.array(x0)
        got = oracle.elem_integral(TRI, x0, family, op, k, kind=3, nx=nx)
        ref = _dense(family, op, k, x0, nx)
        assert abs(got - ref) <= tol * abs(ref), (x0, got, ref)


def test_hsp_degrees_follow_the_one_over_r_cubed_table():
    from nihu_gb300 import meshes
    m = meshes.icosphere(2)
    d = oracle.degree(m, m, oracle.HSP)
    reg = d[d >= 0]
    assert set(np.unique(reg)) <= {0, 2, 4, 6}
    assert (d == -1).sum() == len(m[1])
    dd = oracle.degree(m, m, oracle.DLPT)
    assert (dd == oracle.degree(m, m, oracle.DLP)).all()


def test_pair_list_matches_dense_entries():
    """oracle.assemble_pairs (the FMM near-field loop) equals the dense
    assembly at the listed pairs, self and nearly singular pairs included."""
    from nihu_gb300 import meshes
    m = meshes.icosphere(2)
    kind = oracle.classify(m, m)
    ii, jj = np.nonzero(kind < 0)
    rng = np.random.default_rng(5)
    rows = np.concatenate([ii, rng.integers(0, 320, 200)])
    cols = np.concatenate([jj, rng.integers(0, 320, 200)])
    for op in (oracle.SLP, oracle.DLP, oracle.DLPT, oracle.HSP):
        M = oracle.assemble(m, m, oracle.HELMHOLTZ, op, 1.9)
        v = oracle.assemble_pairs(m, m, oracle.HELMHOLTZ, op, 1.9, rows, cols, threads=2)
        assert np.array_equal(v, M[rows, cols])
    with pytest.raises(RuntimeError):
        oracle.assemble_pairs(m, m, oracle.HELMHOLTZ, oracle.SLP, 1.0, [0], [320])
