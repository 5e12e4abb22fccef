"""Multi-right-hand-side GEMM (FP32 / TF32 / split BF16x9) and the
mixed-precision refinement solver, against numpy and the FP64 oracle."""
import numpy as np
import pytest

import nihu_gb300 as g
from nihu_gb300 import meshes

pytestmark = pytest.mark.gpu


def rand_c(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


@pytest.mark.parametrize("mode,tol", [(g.GEMM_FP32, 1e-5), (g.GEMM_BF16X9, 1e-5), (g.GEMM_TF32, 3e-3),
                                      (g.GEMM_BF16X3, 1e-4), (g.GEMM_BF16X6, 1e-5)])
@pytest.mark.parametrize("m,n,nrhs", [(1000, 700, 64), (333, 517, 5), (1024, 4096, 64), (640, 1000, 100),
                                      (130, 70, 1)])
def test_gemm_modes(gpu_ctx, mode, tol, m, n, nrhs):
    rng = np.random.default_rng(m + n + nrhs)
    A = rand_c(rng, m, n).astype(np.complex64)
    X = rand_c(rng, n, nrhs)
    Y = g.gemm(A, X, mode=mode, ctx=gpu_ctx)
    ref = A.astype(np.complex128) @ X
    assert np.abs(Y - ref).max() / np.abs(ref).max() < tol


@pytest.mark.parametrize("inner_mode", [g.GEMM_TF32, g.GEMM_BF16X9])
def test_solve_multi_random(gpu_ctx, inner_mode):
    rng = np.random.default_rng(1)
    n, nrhs = 900, 12
    A = (np.eye(n) + 0.4 * rand_c(rng, n, n) / np.sqrt(n)).astype(np.complex64)
    B = rand_c(rng, n, nrhs)
    # 1e-6: the residual of a complex64 matrix is accumulated in FP32 per product
    X, outer, inner, res = g.solve_multi(A, B, inner_mode=inner_mode, tol=1e-6, ctx=gpu_ctx)
    ref = np.linalg.solve(A.astype(np.complex128), B)
    assert res.max() <= 1e-6
    assert np.linalg.norm(X - ref, axis=0).max() / np.linalg.norm(ref, axis=0).min() < 1e-5
    assert outer >= 1 and inner >= 1


def test_solve_multi_cylinder_plane_waves(gpu_ctx, oracle):
    """Rigid closed cylinder, 16 plane waves: (M - I/2) p = L q per direction;
    surface pressure within 1e-4 of the FP64 oracle solution."""
    mesh = meshes.cylinder(16, 8, 2, radius=1.0, length=3.0)
    n = len(mesh[1])
    k = 2.0
    dirs = meshes.sphere_directions(16, seed=5)
    Q = meshes.plane_wave_neumann(*mesh, k, dirs)
    L = oracle.assemble(mesh, mesh, oracle.HELMHOLTZ, oracle.SLP, k, threads=8)
    M = oracle.assemble(mesh, mesh, oracle.HELMHOLTZ, oracle.DLP, k, threads=8) - 0.5 * np.eye(n)
    P_ref = np.linalg.solve(M, L @ Q)
    m = g.create_mesh(*mesh)
    sp = g.constant_view(m)
    Lg = np.zeros((n, n), np.complex64, order="F")
    Mg = np.zeros((n, n), np.complex64, order="F")
    Lg << g.dirac(sp) * g.create_integral_operator(g.helmholtz_3d_SLP_kernel(k))[sp]
    Mg << g.dirac(sp) * g.create_integral_operator(g.helmholtz_3d_DLP_kernel(k))[sp]
    Mg << g.dirac(sp) * (-.5 * g.identity_integral_operator())[sp]
    Bg = g.gemm(Lg, Q, mode=g.GEMM_BF16X9, ctx=gpu_ctx)
    X, outer, inner, res = g.solve_multi(Mg, Bg, inner_mode=g.GEMM_TF32, tol=1e-6, ctx=gpu_ctx)
    assert res.max() <= 1e-6
    err = np.abs(X - P_ref).max(axis=0) / np.abs(P_ref).max(axis=0)
    assert err.max() < 1e-4, err


def test_per_rhs_error_against_oracle_solution_10k_quads(gpu_ctx, oracle):
    """The multi-RHS precision path on a 10080-quad closed cylinder (R = 1,
    L = 4: 80 x 100 side grid and O-grid caps of 8 rings), k = 4, 64 plane
    waves with seeded directions: complex64 matrices with FP32 regular
    quadrature, B = SLP Q by the FP32-accurate product, and the
    mixed-precision refinement solve (TF32 inner products, FP64 residual).
    Each right-hand side's surface pressure against the oracle's dense FP64
    solve of the FP64 system within 1e-4 in the 2-norm (the surface pressure
    target); the median is reported in the assertion message."""
    mesh = meshes.cylinder(80, 100, 8, radius=1.0, length=4.0)
    n = len(mesh[1])
    assert n == 10080
    k, nrhs = 4.0, 64
    Q = meshes.plane_wave_neumann(*mesh, k, meshes.sphere_directions(nrhs, seed=2026))
    Lo = oracle.assemble(mesh, mesh, oracle.HELMHOLTZ, oracle.SLP, k, threads=16)
    Mo = oracle.assemble(mesh, mesh, oracle.HELMHOLTZ, oracle.DLP, k, threads=16)
    Mo[np.diag_indices(n)] -= 0.5
    P_ref = np.linalg.solve(Mo, Lo @ Q)
    del Lo, Mo
    m = g.create_mesh(*mesh)
    sp = g.constant_view(m)
    Lg = np.zeros((n, n), np.complex64, order="F")
    Mg = np.zeros((n, n), np.complex64, order="F")
    Lg << g.dirac(sp) * g.create_integral_operator(g.helmholtz_3d_SLP_kernel(k))[sp]
    Mg << g.dirac(sp) * g.create_integral_operator(g.helmholtz_3d_DLP_kernel(k))[sp]
    Mg << g.dirac(sp) * (-.5 * g.identity_integral_operator())[sp]
    Bg = g.gemm(Lg, Q, mode=g.GEMM_FP32, ctx=gpu_ctx)
    X, outer, inner, res = g.solve_multi(Mg, Bg, inner_mode=g.GEMM_TF32, tol=1e-6, ctx=gpu_ctx)
    assert res.max() <= 1e-6
    err = np.linalg.norm(X - P_ref, axis=0) / np.linalg.norm(P_ref, axis=0)
    assert err.max() < 1e-4, (err.max(), np.median(err))


def test_cylinder_40k_entries_match_oracle(gpu_ctx, oracle):
    """The full-size 40000-quad cylinder (k = 4): both matrices assembled on the
    device, their first 64 columns (every row) against the FP64 oracle."""
    import ctypes
    nodes, elems = meshes.cylinder_40k()
    n = len(elems)
    k, nc = 4.0, 64
    L = g.lib()
    dm = g.api.DeviceMesh(gpu_ctx, nodes, elems)
    ps, pd = ctypes.c_void_p(), ctypes.c_void_p()
    gpu_ctx.check(L.nihu_gb_device_alloc(gpu_ctx.handle, 8 * n * n, ctypes.byref(ps)))
    gpu_ctx.check(L.nihu_gb_device_alloc(gpu_ctx.handle, 8 * n * n, ctypes.byref(pd)))
    try:
        gpu_ctx.check(L.nihu_gb_assemble(gpu_ctx.handle, dm.handle, dm.handle, g.HELMHOLTZ_3D, 3, k, 1.0, 0.0,
                                         g.REGULAR_FP32, g.C64, ps, pd, n, 0, g.DEVICE))
        for ptr, op in ((ps, oracle.SLP), (pd, oracle.DLP)):
            got = np.zeros((n, nc), np.complex64, order="F")
            gpu_ctx.check(L.nihu_gb_memcpy(gpu_ctx.handle, got.ctypes.data, g.HOST, ptr, g.DEVICE, got.nbytes))
            ref = oracle.assemble((nodes, elems), (nodes, elems), oracle.HELMHOLTZ, op, k, cols=(0, nc),
                                  same_mesh=True, threads=16)
            assert np.abs(got - ref).max() / np.abs(ref).max() < 1e-5
    finally:
        L.nihu_gb_device_free(gpu_ctx.handle, ps)
        L.nihu_gb_device_free(gpu_ctx.handle, pd)
    dm.close()
