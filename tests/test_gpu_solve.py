"""GPU matvec, GMRES, LU and the CBIE solve (C ABI), checked against numpy
(FP64) and the analytic pulsating sphere."""
import numpy as np
import pytest

import nihu_gb300 as g
from nihu_gb300 import meshes

pytestmark = pytest.mark.gpu


def rand_c(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


@pytest.mark.parametrize("m,n", [(1, 1), (7, 3), (513, 257), (2000, 1500), (4096, 4096)])
@pytest.mark.parametrize("dt", [np.complex64, np.complex128])
def test_matvec(gpu_ctx, m, n, dt):
    rng = np.random.default_rng(m * 31 + n)
    A = np.asfortranarray(rand_c(rng, m, n).astype(dt))
    x = rand_c(rng, n)
    y = g.matvec(A, x, ctx=gpu_ctx)
    ref = A.astype(np.complex128) @ x
    tol = 1e-5 if dt == np.complex64 else 1e-13
    assert np.abs(y - ref).max() / np.abs(ref).max() < tol


@pytest.mark.parametrize("dt", [np.complex64, np.complex128])
def test_gmres(gpu_ctx, dt):
    rng = np.random.default_rng(3)
    n = 700
    A = np.eye(n) + 0.3 * rand_c(rng, n, n) / np.sqrt(n)
    b = rand_c(rng, n)
    x, it, res = g.gmres(A.astype(dt), b, restart=20, tol=1e-10 if dt == np.complex128 else 1e-6, ctx=gpu_ctx)
    ref = np.linalg.solve(A.astype(dt).astype(np.complex128), b)
    assert it > 1
    assert np.linalg.norm(x - ref) / np.linalg.norm(ref) < (1e-8 if dt == np.complex128 else 1e-5)


def test_gmres_not_converged_raises(gpu_ctx):
    rng = np.random.default_rng(5)
    n = 300
    A = rand_c(rng, n, n)
    with pytest.raises(g.NotConvergedError):
        g.gmres(A, rand_c(rng, n), restart=5, max_iters=10, tol=1e-12, ctx=gpu_ctx)


@pytest.mark.parametrize("n", [1, 5, 64, 333])
def test_lu_solve(gpu_ctx, n):
    rng = np.random.default_rng(n)
    A = rand_c(rng, n, n) + n * np.eye(n) * 0.1
    b = rand_c(rng, n)
    x = g.lu_solve(A, b, ctx=gpu_ctx)
    ref = np.linalg.solve(A, b)
    assert np.linalg.norm(x - ref) / np.linalg.norm(ref) < 1e-11


def test_lu_singular_raises(gpu_ctx):
    A = np.zeros((4, 4), complex)
    with pytest.raises(g.NihuError):
        g.lu_solve(A, np.ones(4), ctx=gpu_ctx)


@pytest.mark.parametrize("solver,dtype", [("gmres", g.C64), ("lu", g.C128)])
def test_pulsating_sphere(gpu_ctx, oracle, solver, dtype):
    """q = 1 on the unit sphere: p = -R/(1+ikR) (nihu/test/stallone_unit/helmholtz_3d_pulsating_sphere_test.cpp:51-56).
    Surface pressure within 1e-4 of the FP64 oracle solution; the analytic error is the
    discretisation error of 1280 flat triangles (about 1%)."""
    mesh_arr = meshes.icosphere(3)
    mesh = g.create_mesh(*mesh_arr)
    k = 1.0
    n = mesh.num_elements
    q = np.ones(n, complex)
    p, it, res = g.solve_cbie(mesh, k, q, dtype=dtype, solver=solver, tol=1e-8, ctx=gpu_ctx)
    L = oracle.assemble(mesh_arr, mesh_arr, oracle.HELMHOLTZ, oracle.SLP, k, threads=8)
    M = oracle.assemble(mesh_arr, mesh_arr, oracle.HELMHOLTZ, oracle.DLP, k, threads=8)
    p_ref = np.linalg.solve(M - 0.5 * np.eye(n), L @ q)
    assert np.abs(p - p_ref).max() / np.abs(p_ref).max() < 1e-4
    pa = -1.0 / (1 + 1j * k)
    assert np.abs(p - pa).max() / abs(pa) < 0.02


def test_lu_ill_conditioned_falls_back_to_fp64(gpu_ctx):
    """cond(A) = 1e9: the FP32 factors cannot be refined (cond x eps32 > 1), so
    the solve takes the FP64 factorisation; the result is as accurate as an FP64
    LU can be (cond x eps64)."""
    rng = np.random.default_rng(11)
    n = 200
    Q1, _ = np.linalg.qr(rand_c(rng, n, n))
    Q2, _ = np.linalg.qr(rand_c(rng, n, n))
    A = (Q1 * np.logspace(0, -9, n)) @ Q2.conj().T
    b = rand_c(rng, n)
    x = g.lu_solve(A, b, ctx=gpu_ctx)
    # backward stable: the residual is a few eps |A| |x|; the error is cond x that
    assert np.linalg.norm(A @ x - b) / (np.linalg.norm(A, 2) * np.linalg.norm(x)) < 1e-13
    ref = np.linalg.solve(A, b)
    assert np.linalg.norm(x - ref) / np.linalg.norm(ref) < 1e-5


@pytest.mark.parametrize("n", [2048, 3000])
def test_lu_panel_widths_below_sixteen(gpu_ctx, n):
    """Orders whose first panels hold fewer than 16 columns in shared memory."""
    rng = np.random.default_rng(n)
    A = rand_c(rng, n, n) + n * np.eye(n) * 0.05
    b = rand_c(rng, n)
    x = g.lu_solve(A, b, ctx=gpu_ctx)
    ref = np.linalg.solve(A, b)
    assert np.linalg.norm(x - ref) / np.linalg.norm(ref) < 1e-11
