"""Pair-list assembly (nihu_gb_assemble_pairs, the FMM near-field P2P
evaluation) against the FP64 oracle's dense matrices, through the C ABI.

Tolerances, on every listed entry, relative to the largest |entry| of the
oracle's dense matrix: FP64 regular quadrature 1e-11, FP32 1e-5.
"""
import ctypes

import numpy as np
import pytest

import nihu_gb300 as g
from nihu_gb300 import meshes
from test_gpu_assembly import mixed_mesh

pytestmark = pytest.mark.gpu

_oracle_cache = {}


def oracle_dense(oracle, name, mesh, op, k, family=None, test_mesh=None):
    family = oracle.HELMHOLTZ if family is None else family
    key = (name, op, k, family)
    if key not in _oracle_cache:
        t = mesh if test_mesh is None else test_mesh
        _oracle_cache[key] = oracle.assemble(t, mesh, family, op, k, same_mesh=test_mesh is None, threads=8)
    return _oracle_cache[key]


def pair_list(mesh, test_mesh=None, n_random=4000, seed=0):
    """Every self pair, every nearly singular pair (d/D < 1.5) and random others."""
    from oracle import oracle
    t = mesh if test_mesh is None else test_mesh
    kind = oracle.classify(t, mesh, same_mesh=test_mesh is None)  # -1 self, -2 nearly singular, else regular
    ii, jj = np.nonzero(kind < 0)
    rng = np.random.default_rng(seed)
    m, n = kind.shape
    ri, rj = rng.integers(0, m, n_random), rng.integers(0, n, n_random)
    rows = np.concatenate([ii, ri]).astype(np.int32)
    cols = np.concatenate([jj, rj]).astype(np.int32)
    perm = rng.permutation(len(rows))
    return rows[perm], cols[perm]


@pytest.mark.parametrize("name", ["ico3", "mixed"])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-11), ("fp32", 1e-5)])
def test_slp_dlp_pairs_against_oracle(gpu_ctx, oracle, name, precision, tol):
    mesh = meshes.icosphere(3) if name == "ico3" else mixed_mesh()
    k = 2.5
    rows, cols = pair_list(mesh)
    m = g.create_mesh(*mesh)
    a, b = g.assemble_pairs(m, m, rows, cols, g.SLP | g.DLP, k, precision=precision, ctx=gpu_ctx)
    S = oracle_dense(oracle, name, mesh, oracle.SLP, k)
    D = oracle_dense(oracle, name, mesh, oracle.DLP, k)
    assert np.abs(b - S[rows, cols]).max() / np.abs(S).max() <= tol
    assert np.abs(a - D[rows, cols]).max() / np.abs(D).max() <= tol


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-11), ("fp32", 1e-5)])
def test_burton_miller_near_field_with_identity(gpu_ctx, oracle, precision, tol):
    """The Burton-Miller FMM solver's two near fields: DLP + alpha HSP - I/2
    and SLP + alpha DLPt + alpha/2 I."""
    mesh = meshes.icosphere(3)
    k = 3.0
    alpha = -1j / k
    rows, cols = pair_list(mesh, seed=1)
    m = g.create_mesh(*mesh)
    a, b = g.assemble_pairs(m, m, rows, cols, g.SLP | g.DLP | g.DLPT | g.HSP, k,
                            coef=[1.0, 1.0, alpha, alpha], ident=[-0.5, alpha / 2], precision=precision, ctx=gpu_ctx)
    n = len(mesh[1])
    A = (oracle_dense(oracle, "ico3", mesh, oracle.DLP, k) + alpha * oracle_dense(oracle, "ico3", mesh, oracle.HSP, k)
         - 0.5 * np.eye(n))
    B = (oracle_dense(oracle, "ico3", mesh, oracle.SLP, k) + alpha * oracle_dense(oracle, "ico3", mesh, oracle.DLPT, k)
         + alpha / 2 * np.eye(n))
    assert np.abs(a - A[rows, cols]).max() / np.abs(A).max() <= tol
    assert np.abs(b - B[rows, cols]).max() / np.abs(B).max() <= tol
    # the same operators one at a time agree with the fused call
    _, t = g.assemble_pairs(m, m, rows, cols, g.DLPT, k, precision="fp64", ctx=gpu_ctx)
    Ht = oracle_dense(oracle, "ico3", mesh, oracle.DLPT, k)
    assert np.abs(t - Ht[rows, cols]).max() / np.abs(Ht).max() <= 1e-11


def test_near_field_matrix_of_a_box_partition(gpu_ctx, oracle):
    """P2P list as an FMM builds it: all pairs of elements in the same or a
    neighbouring leaf box; the sparse near field equals the dense matrix on
    that pattern, and near + far matvec equals the dense matvec."""
    sp = pytest.importorskip("scipy.sparse")
    mesh = meshes.icosphere(3)
    nodes, elems = mesh
    c = meshes.centroids_and_normals(nodes, elems)[0]
    box = np.floor((c + 1.0001) / 0.5).astype(int)  # 4 x 4 x 4 leaf boxes
    rows, cols = [], []
    keys = {}
    for e, bx in enumerate(map(tuple, box)):
        keys.setdefault(bx, []).append(e)
    for bx, members in keys.items():
        for nb, others in keys.items():
            if max(abs(np.array(bx) - np.array(nb))) <= 1:
                for i in members:
                    rows += [i] * len(others)
                    cols += others
    rows, cols = np.array(rows, np.int32), np.array(cols, np.int32)
    n = len(elems)
    k = 2.0
    m = g.create_mesh(*mesh)
    _, s = g.assemble_pairs(m, m, rows, cols, g.SLP, k, precision="fp64", ctx=gpu_ctx)
    near = sp.csr_matrix((s, (rows, cols)), shape=(n, n))
    S = oracle_dense(oracle, "ico3", mesh, oracle.SLP, k)
    mask = near.toarray() != 0
    assert mask.sum() == len(rows)  # no duplicate pairs, no zero entries
    assert np.abs(near.toarray()[mask] - S[mask]).max() / np.abs(S).max() <= 1e-11
    x = np.random.default_rng(3).standard_normal(n)
    far = np.where(mask, 0.0, S)
    assert np.allclose(near @ x + far @ x, S @ x, rtol=0, atol=1e-12 * np.abs(S @ x).max())


def test_field_points(gpu_ctx, oracle):
    """Pairs between a field mesh (a larger sphere) and the surface: no self
    terms, nearly singular pairs where the spheres are close."""
    surf = meshes.icosphere(2)
    fn, fe = meshes.icosphere(2)
    field = (fn * 1.08, fe)
    rows, cols = pair_list(surf, test_mesh=field, seed=2)
    ms, mf = g.create_mesh(*surf), g.create_mesh(*field)
    k = 1.7
    a, b = g.assemble_pairs(mf, ms, rows, cols, g.SLP | g.DLP, k, precision="fp64", ctx=gpu_ctx)
    S = oracle_dense(oracle, "field", surf, oracle.SLP, k, test_mesh=field)
    D = oracle_dense(oracle, "field", surf, oracle.DLP, k, test_mesh=field)
    assert np.abs(b - S[rows, cols]).max() / np.abs(S).max() <= 1e-11
    assert np.abs(a - D[rows, cols]).max() / np.abs(D).max() <= 1e-11


def test_device_arrays_and_errors(gpu_ctx):
    L = g.lib()
    mesh = meshes.icosphere(2)
    m = g.create_mesh(*mesh)
    dm = m.device(gpu_ctx)
    rows, cols = pair_list(mesh, n_random=500, seed=4)
    n = len(rows)
    a_host, b_host = g.assemble_pairs(m, m, rows, cols, g.SLP | g.DLP, 1.0, ctx=gpu_ctx)
    ptr = {nm: ctypes.c_void_p() for nm in ("r", "c", "a", "b")}
    for nm, size in (("r", 4 * n), ("c", 4 * n), ("a", 16 * n), ("b", 16 * n)):
        gpu_ctx.check(L.nihu_gb_device_alloc(gpu_ctx.handle, size, ctypes.byref(ptr[nm])))
    gpu_ctx.check(L.nihu_gb_memcpy(gpu_ctx.handle, ptr["r"], g.DEVICE, rows.ctypes.data, g.HOST, 4 * n))
    gpu_ctx.check(L.nihu_gb_memcpy(gpu_ctx.handle, ptr["c"], g.DEVICE, cols.ctypes.data, g.HOST, 4 * n))
    gpu_ctx.check(L.nihu_gb_assemble_pairs(gpu_ctx.handle, dm.handle, dm.handle, g.HELMHOLTZ_3D, g.SLP | g.DLP, 1.0,
                                           None, None, g.REGULAR_FP32, g.C128, n, ptr["r"], ptr["c"], ptr["a"],
                                           ptr["b"], g.DEVICE))
    a_dev, b_dev = np.zeros(n, np.complex128), np.zeros(n, np.complex128)
    gpu_ctx.check(L.nihu_gb_memcpy(gpu_ctx.handle, a_dev.ctypes.data, g.HOST, ptr["a"], g.DEVICE, 16 * n))
    gpu_ctx.check(L.nihu_gb_memcpy(gpu_ctx.handle, b_dev.ctypes.data, g.HOST, ptr["b"], g.DEVICE, 16 * n))
    assert np.array_equal(a_dev, a_host) and np.array_equal(b_dev, b_host)
    # an index out of range in device memory is reported, not read
    bad = rows.copy()
    bad[n // 2] = 10 ** 6
    gpu_ctx.check(L.nihu_gb_memcpy(gpu_ctx.handle, ptr["r"], g.DEVICE, bad.ctypes.data, g.HOST, 4 * n))
    st = L.nihu_gb_assemble_pairs(gpu_ctx.handle, dm.handle, dm.handle, g.HELMHOLTZ_3D, g.SLP, 1.0, None, None,
                                  g.REGULAR_FP32, g.C128, n, ptr["r"], ptr["c"], None, ptr["b"], g.DEVICE)
    assert st == 1
    for p_ in ptr.values():
        L.nihu_gb_device_free(gpu_ctx.handle, p_)
    # host arrays: checked before any launch
    with pytest.raises(g.InvalidArgumentError):
        g.assemble_pairs(m, m, bad, cols, g.SLP, 1.0, ctx=gpu_ctx)
    # Burton-Miller operators need triangle trial elements
    q = g.create_mesh(*meshes.cylinder(8, 3, 1))
    with pytest.raises(g.InvalidArgumentError):
        g.assemble_pairs(q, q, [0], [0], g.HSP, 1.0, ctx=gpu_ctx)
    # an empty list is a no-op
    a, b = g.assemble_pairs(m, m, [], [], g.SLP | g.DLP, 1.0, ctx=gpu_ctx)
    assert len(a) == 0 and len(b) == 0


@pytest.mark.parametrize("name", ["ico3", "mixed"])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-11), ("fp32", 1e-5)])
def test_complex_wave_number_pairs(gpu_ctx, oracle, name, precision, tol):
    """A complex (lossy) wave number (nihu_gb_assemble_pairs_c): SLP and DLP
    on triangles and quads (Duffy self terms, inverse-mapped nearly singular
    quads), and on the icosphere the Burton-Miller near field with DLPt and
    HSP, against the oracle's entries of the same pairs."""
    mesh = meshes.icosphere(3) if name == "ico3" else mixed_mesh()
    k = 2.5 - 0.4j
    rows, cols = pair_list(mesh, seed=3)
    m = g.create_mesh(*mesh)
    ops = g.SLP | g.DLP | g.DLPT | g.HSP if name == "ico3" else g.SLP | g.DLP
    alpha = -1j / k
    coef = [1.0, 1.0, alpha, alpha]
    a, b = g.assemble_pairs(m, m, rows, cols, ops, k, coef=coef, precision=precision, ctx=gpu_ctx)
    A = oracle_dense(oracle, name, mesh, oracle.DLP, k)
    B = oracle_dense(oracle, name, mesh, oracle.SLP, k)
    if name == "ico3":
        A = A + alpha * oracle_dense(oracle, name, mesh, oracle.HSP, k)
        B = B + alpha * oracle_dense(oracle, name, mesh, oracle.DLPT, k)
    assert np.abs(a - A[rows, cols]).max() / np.abs(A).max() <= tol
    assert np.abs(b - B[rows, cols]).max() / np.abs(B).max() <= tol
