"""GPU assembly parity against the FP64 oracle, through the C ABI.

Tolerances (written here, checked on every entry of the matrix):
  * FP64 regular mode: max |A_gpu - A_oracle| / max |A_oracle| <= 1e-11
    (summation order only); every SLP entry within 1e-10 of its own magnitude.
  * FP32 regular mode (the default): every SLP and DLP entry within 1e-5 of
    its own magnitude (PER_ENTRY), against the oracle, on icospheres of 320,
    1280 and 5120 triangles, quad cylinders of 224 and 4608 elements, a mixed
    triangle/quad cylinder and the reference's own sphere meshes.  The one
    exception is a DLP entry of two coplanar flat elements (the diagonal, a
    cylinder column, a cap): r.n = 0 there, the exact entry is zero and the
    oracle's is FP64 rounding; those are bounded absolutely, within 1e-6 of
    the largest entry (FLAT_ZERO).
Singular and nearly singular entries are FP64 in both modes (the nearly
singular dynamic part of triangles is FP32 in the FP32 mode).
"""
import ctypes
import os

import numpy as np
import pytest

import nihu_gb300 as g
from nihu_gb300 import meshes

from parity import FLAT_ZERO, PER_ENTRY, assert_entries, coplanar_pairs, rel_entry, rel_norm  # noqa: F401

pytestmark = pytest.mark.gpu


def mixed_mesh():
    """Closed cylinder with every third side quad split into two triangles."""
    nodes, elems = meshes.cylinder(16, 6, 2, radius=1.0, length=4.0)
    rows = []
    for e, row in enumerate(elems):
        if e < 16 * 6 and e % 3 == 0:
            a, b, c, d = row[1:5]
            rows.append([g.TRIA_1, a, b, c, -1])
            rows.append([g.TRIA_1, a, c, d, -1])
        else:
            rows.append(list(row))
    return nodes, np.array(rows, dtype=np.int32)


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

MESHES = {
    "ico2": lambda: meshes.icosphere(2),
    "ico3": lambda: meshes.icosphere(3),
    "cyl": lambda: meshes.cylinder(16, 8, 2, radius=1.0, length=3.0),
    "mixed": mixed_mesh,
    # the reference's pulsating-sphere meshes (tests/golden, copied unchanged)
    "sphere_1_3": lambda: meshes.read_off(os.path.join(GOLDEN, "sphere_1_3.off")),
    "sphere_1_5": lambda: meshes.read_off(os.path.join(GOLDEN, "sphere_1_5.off")),
}
_cache = {}


def get_mesh(name):
    if name not in _cache:
        _cache[name] = MESHES[name]()
    return _cache[name]


_oracle_cache = {}


def oracle_matrix(oracle, name, family, op, k):
    key = (name, family, op, k)
    if key not in _oracle_cache:
        m = get_mesh(name)
        _oracle_cache[key] = oracle.assemble(m, m, family, op, k, threads=8)
    return _oracle_cache[key]


def gpu_assemble(ctx, mesh, family, ops, k, precision, dtype, test_mesh=None, alpha=1.0, accumulate_into=None):
    L = g.lib()
    trial = g.api.DeviceMesh(ctx, *mesh)
    test = trial if test_mesh is None else g.api.DeviceMesh(ctx, *test_mesh)
    m, n = test.n, trial.n
    cdt = np.complex64 if dtype == g.C64 else np.complex128
    outs = {}
    for op in (g.SLP, g.DLP):
        if ops & op:
            outs[op] = (np.array(accumulate_into[op], dtype=cdt, order="F") if accumulate_into
                        else np.zeros((m, n), dtype=cdt, order="F"))
    alpha = complex(alpha)
    kc = complex(k)
    ctx.check(L.nihu_gb_assemble_c(ctx.handle, test.handle, trial.handle, family, ops, kc.real, kc.imag, alpha.real,
                                   alpha.imag, precision, dtype, outs[g.SLP].ctypes.data if g.SLP in outs else None,
                                   outs[g.DLP].ctypes.data if g.DLP in outs else None, m,
                                   1 if accumulate_into else 0, g.HOST))
    test.close()
    if test_mesh is not None:
        trial.close()
    return outs


# ("ico3", Helmholtz, k = 1) is the plain small configuration itself (1280
# triangles, k = 1, complex128 in the FP64 mode)
CASES = [("ico2", g.HELMHOLTZ_3D, 1.0), ("ico2", g.LAPLACE_3D, 0.0), ("ico3", g.HELMHOLTZ_3D, 5.0),
         ("ico3", g.HELMHOLTZ_3D, 1.0), ("cyl", g.HELMHOLTZ_3D, 2.0), ("cyl", g.LAPLACE_3D, 0.0),
         ("mixed", g.HELMHOLTZ_3D, 1.5), ("sphere_1_3", g.HELMHOLTZ_3D, 1.0), ("sphere_1_3", g.LAPLACE_3D, 0.0),
         ("sphere_1_5", g.HELMHOLTZ_3D, 1.0), ("sphere_1_5", g.HELMHOLTZ_3D, 4.0),
         # complex (lossy) wave numbers: nihu_gb_assemble_c
         ("ico2", g.HELMHOLTZ_3D, 2.0 - 0.3j), ("ico3", g.HELMHOLTZ_3D, 5.0 - 0.5j), ("cyl", g.HELMHOLTZ_3D, 2.0 - 0.3j),
         ("mixed", g.HELMHOLTZ_3D, 1.5 - 0.2j)]


@pytest.mark.parametrize("name,family,k", CASES)
def test_fp64_mode_matches_oracle(gpu_ctx, oracle, name, family, k):
    mesh = get_mesh(name)
    out = gpu_assemble(gpu_ctx, mesh, family, g.SLP | g.DLP, k, g.REGULAR_FP64, g.C128)
    for op in (g.SLP, g.DLP):
        ref = oracle_matrix(oracle, name, family, op, k)
        assert np.all(np.isfinite(out[op]))
        assert rel_norm(out[op], ref) < 1e-11, (op, rel_norm(out[op], ref))
        if op == g.SLP:
            assert rel_entry(out[op], ref) < 1e-10


@pytest.mark.parametrize("name,family,k", CASES)
def test_fp32_mode_matches_oracle(gpu_ctx, oracle, name, family, k):
    """Every SLP and DLP entry of the FP32 mode within PER_ENTRY of the
    oracle's (coplanar DLP pairs within FLAT_ZERO of the largest entry)."""
    mesh = get_mesh(name)
    out = gpu_assemble(gpu_ctx, mesh, family, g.SLP | g.DLP, k, g.REGULAR_FP32, g.C64)
    for op in (g.SLP, g.DLP):
        ref = oracle_matrix(oracle, name, family, op, k)
        assert rel_norm(out[op], ref) < 1e-5, (op, rel_norm(out[op], ref))
        assert_entries(out[op], ref, op, mesh)


@pytest.mark.parametrize("family,k", [(g.HELMHOLTZ_3D, 5.0), (g.HELMHOLTZ_3D, 0.5), (g.LAPLACE_3D, 0.0)])
def test_fp32_mode_every_entry_on_sphere(gpu_ctx, oracle, family, k):
    """Every SLP and DLP entry of the FP32 mode within PER_ENTRY (1e-5) of
    its own magnitude against the oracle, on an icosphere of 5120 triangles
    (DLP diagonal: zero on a flat element, exactly).  This also guards the
    quadrature-level choice of the FP32 kernel, whose warp-uniform paths skip
    the per-lane classification: on this mesh the one-point rule in place of
    degree 2 moves an entry by at least 1.2e-3 and degree 2 in place of
    degree 4 moves an SLP entry by at least 3e-5; a DLP entry moves least at
    its class boundary, about 1e-6, below what an FP32 entry resolves
    (tests/test_parity_sensitivity.py plants such wrong levels in the oracle
    and checks that this comparison fails them)."""
    mesh = meshes.icosphere(4)
    o32 = gpu_assemble(gpu_ctx, mesh, family, g.SLP | g.DLP, k, g.REGULAR_FP32, g.C64)
    for op in (g.SLP, g.DLP):
        ref = oracle.assemble(mesh, mesh, family, op, k, threads=16)
        got = o32[op]
        if op == g.DLP:
            assert np.abs(np.diagonal(got)).max() == 0.0
        assert_entries(got, ref, op, mesh)


@pytest.mark.parametrize("k", [5.0, 0.5])
def test_fp32_mode_every_entry_on_quads(gpu_ctx, oracle, k):
    """The same per-entry check against the oracle on a closed cylinder of
    4608 flat quads (64 x 48 side grid, O-grid caps): the four-corner
    quadrature levels of the FP32 kernel.  Every SLP entry, and every DLP
    entry of a pair that is not coplanar, within PER_ENTRY of its own
    magnitude -- including the nearly coplanar far pairs of neighbouring side
    columns, whose r.n is a few 1e-3 of r (the FP32 kernel forms r from the
    hi/lo split centres and the points' offsets from their element centre).
    A coplanar pair (a side column, a cap) has a DLP entry of rounding size
    only; its FP32 value within FLAT_ZERO of the largest entry."""
    mesh = meshes.cylinder(64, 48, 8, radius=1.0, length=3.0)
    o32 = gpu_assemble(gpu_ctx, mesh, g.HELMHOLTZ_3D, g.SLP | g.DLP, k, g.REGULAR_FP32, g.C64)
    cop = coplanar_pairs(mesh)
    assert cop.sum() > len(cop)
    for op in (g.SLP, g.DLP):
        ref = oracle.assemble(mesh, mesh, g.HELMHOLTZ_3D, op, k, threads=16)
        assert_entries(o32[op], ref, op, mesh)


@pytest.mark.parametrize("ops", [g.SLP, g.DLP])
def test_single_operator_and_complex128_output(gpu_ctx, oracle, ops):
    out = gpu_assemble(gpu_ctx, get_mesh("ico2"), g.HELMHOLTZ_3D, ops, 1.0, g.REGULAR_FP32, g.C128)
    ref = oracle_matrix(oracle, "ico2", g.HELMHOLTZ_3D, ops, 1.0)
    assert list(out) == [ops]
    assert rel_norm(out[ops], ref) < 1e-5


def test_accumulate_and_scale(gpu_ctx, oracle):
    """NiHu's '<<' adds alpha * Op into the existing matrix (nihu/core/weighted_residual.hpp:197-206)."""
    mesh = get_mesh("ico2")
    rng = np.random.default_rng(7)
    n = len(mesh[1])
    base = {op: rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)) for op in (g.SLP, g.DLP)}
    alpha = -0.5 + 0.25j
    out = gpu_assemble(gpu_ctx, mesh, g.HELMHOLTZ_3D, 3, 1.0, g.REGULAR_FP64, g.C128, alpha=alpha,
                       accumulate_into=base)
    for op in (g.SLP, g.DLP):
        ref = base[op] + alpha * oracle_matrix(oracle, "ico2", g.HELMHOLTZ_3D, op, 1.0)
        assert rel_norm(out[op], ref) < 1e-13


def test_field_points_different_mesh(gpu_ctx, oracle):
    """Test mesh != trial mesh: no self terms, nearly singular check still applies
    (nihu/core/integral_transform.hpp:159-161)."""
    trial = get_mesh("ico2")
    nodes, elems = meshes.icosphere(2, radius=1.08)
    test = (nodes, elems)
    out = gpu_assemble(gpu_ctx, trial, g.HELMHOLTZ_3D, 3, 2.0, g.REGULAR_FP64, g.C128, test_mesh=test)
    codes = oracle.classify(test, trial, same_mesh=False)
    assert (codes == -2).sum() > 0 and (codes == -1).sum() == 0
    for op in (g.SLP, g.DLP):
        ref = oracle.assemble(test, trial, g.HELMHOLTZ_3D, op, 2.0, same_mesh=False, threads=8)
        assert rel_norm(out[op], ref) < 1e-12


def test_panel_pipeline_small_budget(oracle):
    """A small HBM budget forces many column panels with overlapped copies."""
    mesh = get_mesh("ico3")
    ctx = g.Context(0, hbm_budget_bytes=48 << 20)
    try:
        out = gpu_assemble(ctx, mesh, g.HELMHOLTZ_3D, 3, 5.0, g.REGULAR_FP32, g.C64)
    finally:
        ctx.close()
    for op in (g.SLP, g.DLP):
        assert rel_norm(out[op], oracle_matrix(oracle, "ico3", g.HELMHOLTZ_3D, op, 5.0)) < 1e-5


def test_device_output(gpu_ctx, oracle):
    L = g.lib()
    mesh = get_mesh("ico2")
    dm = g.api.DeviceMesh(gpu_ctx, *mesh)
    n = dm.n
    bytes_ = n * n * 16
    dptr = ctypes.c_void_p()
    gpu_ctx.check(L.nihu_gb_device_alloc(gpu_ctx.handle, bytes_, ctypes.byref(dptr)))
    try:
        gpu_ctx.check(L.nihu_gb_assemble(gpu_ctx.handle, dm.handle, dm.handle, g.HELMHOLTZ_3D, g.SLP, 1.0, 1.0, 0.0,
                                         g.REGULAR_FP64, g.C128, dptr, None, n, 0, g.DEVICE))
        host = np.zeros((n, n), np.complex128, order="F")
        gpu_ctx.check(L.nihu_gb_memcpy(gpu_ctx.handle, host.ctypes.data, g.HOST, dptr, g.DEVICE, bytes_))
    finally:
        L.nihu_gb_device_free(gpu_ctx.handle, dptr)
        dm.close()
    assert rel_norm(host, oracle_matrix(oracle, "ico2", g.HELMHOLTZ_3D, g.SLP, 1.0)) < 1e-12


@pytest.mark.parametrize("name", ["ico3", "cyl", "mixed"])
def test_pair_statistics_match_oracle(gpu_ctx, oracle, name):
    mesh = get_mesh(name)
    m = g.create_mesh(*mesh)
    stats = g.pair_statistics(m, m, ctx=gpu_ctx)
    codes = oracle.classify(mesh, mesh)
    assert stats[0] == (codes == -1).sum()
    assert stats[1] == (codes == -2).sum()
    assert stats.sum() == codes.size


def graded_mesh():
    """A quad cylinder stretched along its axis (element sizes over a range
    of about 8), two far-apart copies of a small icosphere, and one triangle
    about 60 times the mean element size across the cylinder: columns whose
    search box covers 1 to many grid cells, and one that scans all rows."""
    cn, ce = meshes.cylinder(12, 10, 2, radius=1.0, length=3.0)
    cn = cn.copy()
    z = cn[:, 2] / 3.0
    cn[:, 2] = 3.0 * np.sign(z) * np.abs(z) ** 2.5
    sn, se = meshes.icosphere(2)
    parts_n, parts_e, off = [cn], [ce], len(cn)
    for shift in ((1.0e4, 0.0, 0.0), (-3.0e3, 2.0e3, 5.0)):
        parts_n.append(0.3 * sn + np.array(shift))
        e = se.copy()
        e[:, 1:4] += off
        parts_e.append(e)
        off += len(sn)
    big = np.array([[-6.0, -4.0, 1.2], [6.0, -4.0, 1.2], [0.0, 7.0, 1.2]])
    parts_n.append(big)
    parts_e.append(np.array([[g.TRIA_1, off, off + 1, off + 2, -1]], dtype=np.int32))
    width = max(e.shape[1] for e in parts_e)
    parts_e = [np.hstack([e, -np.ones((len(e), width - e.shape[1]), np.int32)]) for e in parts_e]
    return np.vstack(parts_n), np.vstack(parts_e).astype(np.int32)


def check_near_pairs(ctx, oracle, test_mesh, trial_mesh, same):
    test = g.create_mesh(*test_mesh)
    trial = test if same else g.create_mesh(*trial_mesh)
    col_ptr, rows = g.near_pairs(test, trial, ctx=ctx)
    codes = oracle.classify(test_mesh, trial_mesh, same_mesh=same)
    assert col_ptr[0] == 0 and len(rows) == col_ptr[-1]
    for j in range(codes.shape[1]):
        np.testing.assert_array_equal(rows[col_ptr[j]:col_ptr[j + 1]], np.flatnonzero(codes[:, j] == -2))
    return len(rows)


@pytest.mark.parametrize("name", ["ico3", "cyl", "mixed", "sphere_1_5", "graded"])
def test_near_pairs_match_oracle(gpu_ctx, oracle, name):
    """The grid-built nearly singular list is the brute-force list of the
    reference's test d / D_j < 1.5, rows in increasing order per column."""
    mesh = graded_mesh() if name == "graded" else get_mesh(name)
    assert check_near_pairs(gpu_ctx, oracle, mesh, mesh, True) > 0


def test_near_pairs_two_meshes(gpu_ctx, oracle):
    """Test and trial meshes of different sizes and element scales."""
    ico = meshes.icosphere(3)
    small = (0.97 * meshes.icosphere(2)[0], meshes.icosphere(2)[1])
    assert check_near_pairs(gpu_ctx, oracle, small, ico, False) > 0
    assert check_near_pairs(gpu_ctx, oracle, ico, small, False) > 0
    assert check_near_pairs(gpu_ctx, oracle, graded_mesh(), ico, False) >= 0


def test_nihu_shaped_api(gpu_ctx, oracle):
    """Ls << dirac(sp) * Lop[sp]; Ms << dirac(sp) * Mop[sp]; Ms << dirac(sp) * (-.5*I)[sp]
    (nihu/test/matlab/acoustic_bem.mex.cpp:30-50)."""
    nodes, elems = get_mesh("ico2")
    mesh = g.create_mesh(nodes, elems)
    sp = g.constant_view(mesh)
    n = sp.get_num_dofs()
    k = 1.0
    I = g.identity_integral_operator()
    Lop = g.create_integral_operator(g.helmholtz_3d_SLP_kernel(k))
    Mop = g.create_integral_operator(g.helmholtz_3d_DLP_kernel(k))
    Ls = np.zeros((n, n), np.complex128, order="F")
    Ms = np.zeros((n, n), np.complex128, order="F")
    Ls << g.dirac(sp) * Lop[sp]
    Ms << g.dirac(sp) * Mop[sp]
    Ms << g.dirac(sp) * (-.5 * I)[sp]
    refL = oracle_matrix(oracle, "ico2", g.HELMHOLTZ_3D, g.SLP, k)
    refM = oracle_matrix(oracle, "ico2", g.HELMHOLTZ_3D, g.DLP, k) - 0.5 * np.eye(n)
    assert rel_norm(Ls, refL) < 1e-5
    assert rel_norm(Ms, refM) < 1e-5
    # C-ordered result and a scaled operator
    Lc = np.zeros((n, n), np.complex128)
    Lc << g.dirac(sp) * (2.0 * Lop)[sp]
    assert rel_norm(Lc, 2 * refL) < 1e-5


def test_invalid_arguments_raise(gpu_ctx):
    nodes, elems = get_mesh("ico2")
    bad = elems.copy()
    bad[3, 0] = 12345
    with pytest.raises(ValueError):
        g.api.DeviceMesh(gpu_ctx, nodes, bad)
    bad = elems.copy()
    bad[5, 2] = len(nodes) + 3
    with pytest.raises(IndexError):
        g.api.DeviceMesh(gpu_ctx, nodes, bad)
    dm = g.api.DeviceMesh(gpu_ctx, nodes, elems)
    n = dm.n
    out = np.zeros((n, n), np.complex64, order="F")
    L = g.lib()
    with pytest.raises(ValueError):  # ld < rows
        gpu_ctx.check(L.nihu_gb_assemble(gpu_ctx.handle, dm.handle, dm.handle, 0, 1, 1.0, 1.0, 0.0, 0, 0,
                                         out.ctypes.data, None, n - 1, 0, g.HOST))
    with pytest.raises(ValueError):  # DLP requested without a buffer
        gpu_ctx.check(L.nihu_gb_assemble(gpu_ctx.handle, dm.handle, dm.handle, 0, 3, 1.0, 1.0, 0.0, 0, 0,
                                         out.ctypes.data, None, n, 0, g.HOST))
    dm.close()


@pytest.mark.parametrize("k", [2.0 - 0.3j, 1.0 - 1.0j])
def test_pulsating_sphere_complex_wave_number(gpu_ctx, oracle, k):
    """A lossy medium: the exterior CBIE with a complex wave number through
    nihu_gb_solve_cbie_c; the analytic pressure p = -R/(1 + ikR) holds for
    complex k (nihu/test/stallone_unit/helmholtz_3d_pulsating_sphere_test.cpp:51-56).
    Pressure within 1e-4 of the oracle's dense solve (FP32 mode) and 1e-9
    (FP64 mode, LU), and within the discretisation error of the analytic."""
    mesh = get_mesh("ico3")
    n = len(mesh[1])
    m = g.create_mesh(*mesh)
    L = oracle_matrix(oracle, "ico3", g.HELMHOLTZ_3D, g.SLP, k)
    M = oracle_matrix(oracle, "ico3", g.HELMHOLTZ_3D, g.DLP, k) - 0.5 * np.eye(n)
    pr = np.linalg.solve(M, L @ np.ones(n))
    p32, it, res = g.solve_cbie(m, k, np.ones(n), ctx=gpu_ctx)
    p64, _, _ = g.solve_cbie(m, k, np.ones(n), dtype=g.C128, solver="lu", precision="fp64", ctx=gpu_ctx)
    assert np.abs(p32 - pr).max() / np.abs(pr).max() < 1e-4
    assert np.abs(p64 - pr).max() / np.abs(pr).max() < 1e-9
    pa = -1.0 / (1.0 + 1j * k)
    assert np.abs(p64 - pa).max() / abs(pa) < 0.01


def test_complex_wave_number_through_the_operator_algebra(gpu_ctx, oracle):
    """helmholtz_3d_SLP_kernel(k) with a complex k in the NiHu-shaped front end, collocation and Galerkin."""
    nodes, elems = get_mesh("ico2")
    mesh = g.create_mesh(nodes, elems)
    sp = g.constant_view(mesh)
    n = sp.get_num_dofs()
    k = 2.0 - 0.3j
    Ls = np.zeros((n, n), np.complex128, order="F")
    Ls << g.dirac(sp) * g.create_integral_operator(g.helmholtz_3d_SLP_kernel(k))[sp]
    assert rel_norm(Ls, oracle_matrix(oracle, "ico2", g.HELMHOLTZ_3D, g.SLP, k)) < 1e-5
    # the Galerkin formalism (test space * operator[trial space]) with the same k
    Gs = np.zeros((n, n), np.complex128)
    (sp * g.create_integral_operator(g.helmholtz_3d_SLP_kernel(k))[sp]).eval_into(Gs, precision="fp64", ctx=gpu_ctx)
    ref = oracle.assemble_galerkin((nodes, elems), (nodes, elems), g.HELMHOLTZ_3D, g.SLP, k, same_mesh=True, threads=8)
    assert rel_norm(Gs, ref) < 1e-11
