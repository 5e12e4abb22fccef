"""Burton-Miller operators (DLPt, HSP) and the Burton-Miller solve on the GPU
against the FP64 oracle, through the C ABI.

Tolerances (written here, on every entry of the matrix):
  * FP64 regular mode: max |A_gpu - A_oracle| / max |A_oracle| <= 1e-11
  * FP32 regular mode: the same ratio <= 1e-5
  * surface pressure of the Burton-Miller solve: <= 1e-4 of the FP64 oracle's
    dense solve of the same system
Self entries and the static parts of nearly singular entries are FP64 in both
modes; the dynamic part K_k - K_0 of a nearly singular entry is summed in FP32
in FP32 mode (its size is (kr)^2 of the entry's).
"""
import numpy as np
import pytest

import nihu_gb300 as g
from nihu_gb300 import meshes

pytestmark = pytest.mark.gpu


def rel_norm(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def triangulated(nodes, elems):
    """Every quad split into two triangles along its 0-2 diagonal (the
    degenerate half of a quad with a repeated corner dropped)."""
    rows = []
    for row in elems:
        if row[0] == g.QUAD_1:
            a, b, c, d = row[1:5]
            tris = [(a, b, c), (a, c, d)]
        else:
            tris = [tuple(row[1:4])]
        rows += [[g.TRIA_1, *t, -1] for t in tris if len(set(t)) == 3]
    return nodes, np.array(rows, dtype=np.int32)


MESHES = {
    "ico2": lambda: meshes.icosphere(2),
    "ico3": lambda: meshes.icosphere(3),
    "cyl_tri": lambda: triangulated(*meshes.cylinder(12, 6, 2, radius=1.0, length=3.0)),
}
_cache = {}
_oracle_cache = {}


def get_mesh(name):
    if name not in _cache:
        _cache[name] = MESHES[name]()
    return _cache[name]


def oracle_matrix(oracle, name, family, op, k, test_name=None):
    key = (name, test_name, family, op, k)
    if key not in _oracle_cache:
        m = get_mesh(name)
        t = m if test_name is None else get_mesh(test_name)
        _oracle_cache[key] = oracle.assemble(t, m, family, op, k, same_mesh=test_name is None, threads=8)
    return _oracle_cache[key]


def gpu_bm(ctx, mesh, family, ops, k, precision, dtype, test_mesh=None, alpha=1.0, where=g.HOST):
    L = g.lib()
    trial = g.api.DeviceMesh(ctx, *mesh)
    test = trial if test_mesh is None else g.api.DeviceMesh(ctx, *test_mesh)
    m, n = test.n, trial.n
    cdt = np.complex64 if dtype == g.C64 else np.complex128
    outs = {op: np.zeros((m, n), dtype=cdt, order="F") for op in (g.DLPT, g.HSP) if ops & op}
    alpha = complex(alpha)
    kc = complex(k)
    ctx.check(L.nihu_gb_assemble_bm_c(ctx.handle, test.handle, trial.handle, family, ops, kc.real, kc.imag,
                                      alpha.real, alpha.imag, precision, dtype,
                                      outs[g.DLPT].ctypes.data if g.DLPT in outs else None,
                                      outs[g.HSP].ctypes.data if g.HSP in outs else None, m, 0, where))
    return outs


@pytest.mark.parametrize("name", ["ico2", "ico3"])
@pytest.mark.parametrize("family,k", [(g.HELMHOLTZ_3D, 1.3), (g.HELMHOLTZ_3D, 4.0), (g.LAPLACE_3D, 0.0)])
@pytest.mark.parametrize("precision,tol", [(g.REGULAR_FP64, 1e-11), (g.REGULAR_FP32, 1e-5)])
def test_dlpt_hsp_against_oracle(gpu_ctx, oracle, name, family, k, precision, tol):
    outs = gpu_bm(gpu_ctx, get_mesh(name), family, g.DLPT | g.HSP, k, precision,
                  g.C128 if precision == g.REGULAR_FP64 else g.C64)
    for op, oop in ((g.DLPT, oracle.DLPT), (g.HSP, oracle.HSP)):
        ref = oracle_matrix(oracle, name, family, oop, k)
        err = rel_norm(outs[op].astype(np.complex128), ref)
        assert err <= tol, (op, err)


def test_quad_test_elements_and_separate_meshes(gpu_ctx, oracle):
    """Quad collocation elements (test complexity 1: HSP level 3 is the
    13-point degree-7 rule) against a triangulated trial cylinder of another
    radius, near enough for nearly singular pairs."""
    trial = get_mesh("cyl_tri")
    _cache["cyl_quad"] = meshes.cylinder(8, 7, 2, radius=1.12, length=3.2)
    test = _cache["cyl_quad"]
    k = 2.2
    for precision, tol in ((g.REGULAR_FP64, 1e-11), (g.REGULAR_FP32, 1e-5)):
        outs = gpu_bm(gpu_ctx, trial, g.HELMHOLTZ_3D, g.DLPT | g.HSP, k, precision, g.C128, test_mesh=test)
        for op, oop in ((g.DLPT, oracle.DLPT), (g.HSP, oracle.HSP)):
            ref = oracle_matrix(oracle, "cyl_tri", g.HELMHOLTZ_3D, oop, k, test_name="cyl_quad")
            assert rel_norm(outs[op], ref) <= tol, (precision, op)
    # the pair mix covers every HSP level, nearly singular pairs and quad collocation
    d = oracle.degree(test, trial, oracle.HSP, same_mesh=False)
    assert {3, 5, 7} <= set(np.unique(d[d >= 0])) and (d == -2).any()


def test_scale_accumulate_and_device_output(gpu_ctx, oracle):
    mesh = get_mesh("ico2")
    k = 1.3
    alpha = 0.5 - 2.0j
    outs = gpu_bm(gpu_ctx, mesh, g.HELMHOLTZ_3D, g.HSP, k, g.REGULAR_FP64, g.C128, alpha=alpha)
    ref = alpha * oracle_matrix(oracle, "ico2", g.HELMHOLTZ_3D, oracle.HSP, k)
    assert rel_norm(outs[g.HSP], ref) <= 1e-11
    # the operator algebra of the Python front end: result << test * (alpha * Dop)[trial], twice
    m = g.create_mesh(*mesh)
    sp = g.constant_view(m)
    D = g.create_integral_operator(g.helmholtz_3d_HSP_kernel(k))
    Ht = g.create_integral_operator(g.helmholtz_3d_DLPt_kernel(k))
    res = np.zeros((m.num_elements,) * 2, np.complex128)
    wr = g.dirac(sp) * (alpha * D)[sp]
    wr.eval_into(res, precision="fp64", ctx=gpu_ctx)
    wr.eval_into(res, precision="fp64", ctx=gpu_ctx)
    assert rel_norm(res, 2 * ref) <= 1e-11
    res2 = np.zeros_like(res)
    (g.dirac(sp) * Ht[sp]).eval_into(res2, precision="fp64", ctx=gpu_ctx)
    assert rel_norm(res2, oracle_matrix(oracle, "ico2", g.HELMHOLTZ_3D, oracle.DLPT, k)) <= 1e-11


@pytest.mark.parametrize("precision,dtype,tol", [("fp64", g.C128, 1e-11), ("fp32", g.C64, 1e-5)])
def test_burton_miller_system_matrices(gpu_ctx, oracle, precision, dtype, tol):
    name, k = "ico3", 2.0
    n = len(get_mesh(name)[1])
    c = g.burton_miller_coupling(k)
    A, B = g.assemble_burton_miller(g.create_mesh(*get_mesh(name)), k, dtype=dtype, precision=precision, ctx=gpu_ctx)
    H = g.HELMHOLTZ_3D
    A_ref = (oracle_matrix(oracle, name, H, oracle.DLP, k) - 0.5 * np.eye(n)
             + c * oracle_matrix(oracle, name, H, oracle.HSP, k))
    B_ref = (oracle_matrix(oracle, name, H, oracle.SLP, k) + c * oracle_matrix(oracle, name, H, oracle.DLPT, k)
             + 0.5 * c * np.eye(n))
    assert rel_norm(A.astype(np.complex128), A_ref) <= tol
    assert rel_norm(B.astype(np.complex128), B_ref) <= tol


@pytest.mark.parametrize("name,k", [("ico2", 2.0 - 0.3j), ("ico3", 4.0 - 0.5j), ("ico3", 1.3 + 0.2j)])
def test_complex_wave_number_against_oracle(gpu_ctx, oracle, name, k):
    """DLPt and HSP with a complex (lossy) wave number (nihu_gb_assemble_bm_c):
    FP64 mode within 1e-11 of the oracle (normwise); FP32 mode every entry
    within 1e-5 of its own magnitude (the DLPt diagonal, zero on flat
    elements, within 1e-6 of the largest entry)."""
    mesh = get_mesh(name)
    o64 = gpu_bm(gpu_ctx, mesh, g.HELMHOLTZ_3D, g.DLPT | g.HSP, k, g.REGULAR_FP64, g.C128)
    o32 = gpu_bm(gpu_ctx, mesh, g.HELMHOLTZ_3D, g.DLPT | g.HSP, k, g.REGULAR_FP32, g.C64)
    for op, oop in ((g.DLPT, oracle.DLPT), (g.HSP, oracle.HSP)):
        ref = oracle_matrix(oracle, name, g.HELMHOLTZ_3D, oop, k)
        assert rel_norm(o64[op], ref) <= 1e-11, (op, rel_norm(o64[op], ref))
        got = o32[op].astype(np.complex128)
        ref = ref.copy()
        if op == g.DLPT:
            assert np.abs(np.diagonal(got)).max() < 1e-6 * np.abs(ref).max()
            np.fill_diagonal(ref, 1.0)
            np.fill_diagonal(got, 1.0)
        err = np.abs(got - ref) / np.abs(ref)
        assert err.max() < 1e-5, (op, err.max())


def test_burton_miller_complex_wave_number(gpu_ctx, oracle):
    """The system matrices with k = 2 - 0.3i and the coupling -i/k, and the
    GMRES solve of the pulsating sphere against the oracle's dense solve."""
    name, k = "ico3", 2.0 - 0.3j
    n = len(get_mesh(name)[1])
    c = g.burton_miller_coupling(k)
    H = g.HELMHOLTZ_3D
    A_ref = (oracle_matrix(oracle, name, H, oracle.DLP, k) - 0.5 * np.eye(n)
             + c * oracle_matrix(oracle, name, H, oracle.HSP, k))
    B_ref = (oracle_matrix(oracle, name, H, oracle.SLP, k) + c * oracle_matrix(oracle, name, H, oracle.DLPT, k)
             + 0.5 * c * np.eye(n))
    m = g.create_mesh(*get_mesh(name))
    for precision, dtype, tol in (("fp64", g.C128, 1e-11), ("fp32", g.C64, 1e-5)):
        A, B = g.assemble_burton_miller(m, k, dtype=dtype, precision=precision, ctx=gpu_ctx)
        assert rel_norm(A.astype(np.complex128), A_ref) <= tol
        assert rel_norm(B.astype(np.complex128), B_ref) <= tol
    q = np.ones(n, np.complex128)
    p, it, res = g.solve_burton_miller(m, k, q, dtype=g.C128, precision="fp64", tol=1e-10, ctx=gpu_ctx)
    p_ref = np.linalg.solve(A_ref, B_ref @ q)
    assert np.abs(p - p_ref).max() / np.abs(p_ref).max() < 1e-8


@pytest.mark.parametrize("k", [np.pi, 4.4934])
def test_burton_miller_solve_at_interior_resonances(gpu_ctx, oracle, k):
    """Pulsating unit sphere (q = 1, p = -1/(1 + ik)) at the first two
    fictitious wave numbers of the plain CBIE (zeros of j0 and j1): the
    Burton-Miller solve matches the oracle's dense solve of the same system and
    the analytic pressure."""
    name = "ico3"
    mesh = get_mesh(name)
    n = len(mesh[1])
    q = np.ones(n)
    p, it, rel = g.solve_burton_miller(g.create_mesh(*mesh), k, q, restart=50, max_iters=500, tol=1e-8, ctx=gpu_ctx)
    c = g.burton_miller_coupling(k)
    H = g.HELMHOLTZ_3D
    A = oracle_matrix(oracle, name, H, oracle.DLP, k) - 0.5 * np.eye(n) + c * oracle_matrix(oracle, name, H, oracle.HSP, k)
    B = oracle_matrix(oracle, name, H, oracle.SLP, k) + c * oracle_matrix(oracle, name, H, oracle.DLPT, k) + 0.5 * c * np.eye(n)
    p_ref = np.linalg.solve(A, B @ q)
    assert np.abs(p - p_ref).max() / np.abs(p_ref).max() <= 1e-4
    pa = -1.0 / (1.0 + 1j * k)
    assert np.abs(p - pa).max() / abs(pa) < 0.03
    assert it < 60
    # the same system by LU in FP64
    p_lu, _, _ = g.solve_burton_miller(g.create_mesh(*mesh), k, q, solver="lu", dtype=g.C128, precision="fp64",
                                       ctx=gpu_ctx)
    assert np.abs(p_lu - p_ref).max() / np.abs(p_ref).max() <= 1e-9


def test_invalid_arguments(gpu_ctx):
    L = g.lib()
    quads = g.api.DeviceMesh(gpu_ctx, *meshes.cylinder(8, 3, 1))
    out = np.zeros((quads.n, quads.n), np.complex128, order="F")
    st = L.nihu_gb_assemble_bm(gpu_ctx.handle, quads.handle, quads.handle, g.HELMHOLTZ_3D, g.HSP, 1.0, 1.0, 0.0,
                               g.REGULAR_FP64, g.C128, None, out.ctypes.data, quads.n, 0, g.HOST)
    assert st == 1  # NIHU_GB_ERR_INVALID_ARGUMENT: constant triangles only
    tri = g.api.DeviceMesh(gpu_ctx, *get_mesh("ico2"))
    out = np.zeros((tri.n, tri.n), np.complex128, order="F")
    for ops in (0, g.SLP, g.DLPT | g.SLP, 16):
        st = L.nihu_gb_assemble_bm(gpu_ctx.handle, tri.handle, tri.handle, g.HELMHOLTZ_3D, ops, 1.0, 1.0, 0.0,
                                   g.REGULAR_FP64, g.C128, out.ctypes.data, out.ctypes.data, tri.n, 0, g.HOST)
        assert st == 1, ops


@pytest.mark.parametrize("family,k", [(g.HELMHOLTZ_3D, 5.0), (g.LAPLACE_3D, 0.0)])
def test_fp32_mode_every_entry_on_sphere(gpu_ctx, oracle, family, k):
    """Every DLPt and HSP entry of the FP32 mode against the oracle on an
    icosphere of 5120 triangles, within 1e-5 of its own magnitude (the DLPt
    diagonal, zero on flat elements, within 1e-6 of the largest entry): a
    pair integrated with too few points by the regular kernel's warp-uniform
    paths fails here."""
    mesh = meshes.icosphere(4)
    o32 = gpu_bm(gpu_ctx, mesh, family, g.DLPT | g.HSP, k, g.REGULAR_FP32, g.C64)
    for op in (g.DLPT, g.HSP):
        ref = oracle.assemble(mesh, mesh, family, op, k, threads=16)
        got = o32[op].astype(np.complex128)
        if op == g.DLPT:
            assert np.abs(np.diagonal(got)).max() < 1e-6 * np.abs(ref).max()
            ref = ref.copy()
            np.fill_diagonal(ref, 1.0)
            np.fill_diagonal(got, 1.0)
        err = np.abs(got - ref) / np.abs(ref)
        assert err.max() < 1e-5, (op, err.max())
