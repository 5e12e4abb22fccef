"""Frequency sweep (batched assembly + lockstep GMRES) against the plain
single-instance path and the FP64 oracle."""
import numpy as np
import pytest

import nihu_gb300 as g
from nihu_gb300 import meshes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("subdiv", [2, 4])
def test_assemble_sweep_matches_single_assembly(gpu_ctx, subdiv):
    """Frequency-batch matrices against the single-wave-number kernel (FP32
    mode): normwise 1e-6, and every entry but the zero DLP diagonal within
    1e-5 of its own magnitude (measured: below 8e-7), so that a pair the batch kernel integrates at
    another quadrature level than the single kernel (one point in place of
    degree 2 moves an entry by more than 1e-3 on these spheres) fails."""
    import ctypes
    L = g.lib()
    mesh = meshes.icosphere(subdiv)
    dm = g.api.DeviceMesh(gpu_ctx, *mesh)
    n = dm.n
    ks = np.array([0.5, 1.7, 4.2, 9.0])
    nk = len(ks)
    S = np.zeros((n, n * nk), np.complex64, order="F")
    D = np.zeros((n, n * nk), np.complex64, order="F")
    dS, dD = ctypes.c_void_p(), ctypes.c_void_p()
    gpu_ctx.check(L.nihu_gb_device_alloc(gpu_ctx.handle, S.nbytes, ctypes.byref(dS)))
    gpu_ctx.check(L.nihu_gb_device_alloc(gpu_ctx.handle, D.nbytes, ctypes.byref(dD)))
    try:
        gpu_ctx.check(L.nihu_gb_assemble_sweep(gpu_ctx.handle, dm.handle, dm.handle, g.HELMHOLTZ_3D, 3,
                                               ks.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), nk, 0, 0, dS, dD,
                                               n, n * n))
        gpu_ctx.check(L.nihu_gb_memcpy(gpu_ctx.handle, S.ctypes.data, g.HOST, dS, g.DEVICE, S.nbytes))
        gpu_ctx.check(L.nihu_gb_memcpy(gpu_ctx.handle, D.ctypes.data, g.HOST, dD, g.DEVICE, D.nbytes))
    finally:
        L.nihu_gb_device_free(gpu_ctx.handle, dS)
        L.nihu_gb_device_free(gpu_ctx.handle, dD)
    for f, k in enumerate(ks):
        s1 = np.zeros((n, n), np.complex64, order="F")
        d1 = np.zeros((n, n), np.complex64, order="F")
        gpu_ctx.check(L.nihu_gb_assemble(gpu_ctx.handle, dm.handle, dm.handle, g.HELMHOLTZ_3D, 3, float(k), 1.0, 0.0,
                                         0, 0, s1.ctypes.data, d1.ctypes.data, n, 0, g.HOST))
        for a, b in ((S[:, f * n:(f + 1) * n], s1), (D[:, f * n:(f + 1) * n], d1)):
            assert np.abs(a - b).max() / np.abs(b).max() < 1e-6
            a, b = a.copy(), b.copy()
            np.fill_diagonal(a, 1.0)
            np.fill_diagonal(b, 1.0)
            err = np.abs(a - b) / np.abs(b)
            assert err.max() < 1e-5, (k, err.max())
    dm.close()


def test_solve_sweep_pulsating_sphere(gpu_ctx, oracle):
    mesh_arr = meshes.icosphere(3)
    mesh = g.create_mesh(*mesh_arr)
    n = mesh.num_elements
    rng = np.random.default_rng(4)
    ks = np.sort(rng.uniform(0.1, 2.5, 9))
    P, cycles, iters, res = g.solve_sweep(mesh, ks, np.ones(n), tol=1e-7, ctx=gpu_ctx)
    assert res.max() <= 1e-7
    for f, k in enumerate(ks):
        p1, it1, res1 = g.solve_cbie(mesh, float(k), np.ones(n), tol=1e-7, ctx=gpu_ctx)
        assert np.abs(P[:, f] - p1).max() / np.abs(p1).max() < 1e-5
        pa = -1.0 / (1 + 1j * k)
        assert np.abs(P[:, f] - pa).max() / abs(pa) < 0.03
    # one wave number against the FP64 oracle
    k = float(ks[4])
    L = oracle.assemble(mesh_arr, mesh_arr, oracle.HELMHOLTZ, oracle.SLP, k, threads=8)
    M = oracle.assemble(mesh_arr, mesh_arr, oracle.HELMHOLTZ, oracle.DLP, k, threads=8) - 0.5 * np.eye(n)
    p_ref = np.linalg.solve(M, L @ np.ones(n))
    assert np.abs(P[:, 4] - p_ref).max() / np.abs(p_ref).max() < 1e-4


@pytest.mark.parametrize("subdiv", [1, 2])
def test_assemble_sweep_fp64_series_matches_direct(gpu_ctx, subdiv):
    """Frequency batches evaluate the nearly singular dynamic part through its
    power series in k; in FP64 mode the entries match the per-wave-number
    direct quadrature to rounding (coarse meshes reach k r ~ 18, beyond the
    series length, where the batch falls back to the direct sum)."""
    import ctypes
    L = g.lib()
    dm = g.api.DeviceMesh(gpu_ctx, *meshes.icosphere(subdiv))
    n = dm.n
    ks = np.array([0.3, 2.0, 5.5, 9.7])
    nk = len(ks)
    S = np.zeros((n, n * nk), np.complex128, order="F")
    D = np.zeros((n, n * nk), np.complex128, order="F")
    dS, dD = ctypes.c_void_p(), ctypes.c_void_p()
    gpu_ctx.check(L.nihu_gb_device_alloc(gpu_ctx.handle, S.nbytes, ctypes.byref(dS)))
    gpu_ctx.check(L.nihu_gb_device_alloc(gpu_ctx.handle, D.nbytes, ctypes.byref(dD)))
    try:
        gpu_ctx.check(L.nihu_gb_assemble_sweep(gpu_ctx.handle, dm.handle, dm.handle, g.HELMHOLTZ_3D, 3,
                                               ks.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), nk, 1, 1, dS, dD,
                                               n, n * n))
        gpu_ctx.check(L.nihu_gb_memcpy(gpu_ctx.handle, S.ctypes.data, g.HOST, dS, g.DEVICE, S.nbytes))
        gpu_ctx.check(L.nihu_gb_memcpy(gpu_ctx.handle, D.ctypes.data, g.HOST, dD, g.DEVICE, D.nbytes))
    finally:
        L.nihu_gb_device_free(gpu_ctx.handle, dS)
        L.nihu_gb_device_free(gpu_ctx.handle, dD)
    for f, k in enumerate(ks):
        s1 = np.zeros((n, n), np.complex128, order="F")
        d1 = np.zeros((n, n), np.complex128, order="F")
        gpu_ctx.check(L.nihu_gb_assemble(gpu_ctx.handle, dm.handle, dm.handle, g.HELMHOLTZ_3D, 3, float(k), 1.0, 0.0,
                                         1, 1, s1.ctypes.data, d1.ctypes.data, n, 0, g.HOST))
        for a, b in ((S[:, f * n:(f + 1) * n], s1), (D[:, f * n:(f + 1) * n], d1)):
            assert np.abs(a - b).max() / np.abs(b).max() < 1e-12
    dm.close()


def test_sweep_plan_graph_matches_eager_sweep(gpu_ctx):
    """The captured sweep gives the eager batched sweep's results, and replays
    with new wave numbers and data."""
    ms = [g.create_mesh(*meshes.icosphere(s)) for s in (1, 2, 3)]
    rng = np.random.default_rng(31)
    nk = 10
    mesh_of = np.arange(nk) % 3
    plan = g.SweepPlan(ms, mesh_of, k_max=6.0, tol=1e-7, ctx=gpu_ctx)
    # the autotuner kept one of its candidates (the launch model's choice or 4, 8, 16 CTAs per cluster)
    tuning = plan.tuning()
    assert tuning["cluster"] in (1, 2, 4, 8, 16) and tuning["freq_per_block"] in (8, 16, 20)
    assert tuning["replay_ms"] > 0.0
    for rep in range(2):
        ks = rng.uniform(0.2, 6.0, nk)
        q = [rng.standard_normal(ms[i].num_elements) + 1j * rng.standard_normal(ms[i].num_elements) for i in mesh_of]
        P, it, rel, conv = plan.run(ks, q, check=False)
        P2, it2, rel2, conv2 = g.solve_sweep_batched(ms, ks, mesh_of, q=q, tol=1e-7, ctx=gpu_ctx, check=False)
        assert list(it) == list(it2)
        for a, b in zip(P, P2):
            assert np.abs(a - b).max() <= 1e-6 * np.abs(b).max()
    with pytest.raises(g.InvalidArgumentError):
        plan.run(np.full(nk, 7.0))
    plan.close()


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_sweep_right_hand_sides_without_slp_matrices(gpu_ctx, precision):
    """The batched sweep forms b = SLP q inside the assembly (no SLP matrix):
    with random complex Neumann data on a 320 / 1280 mix, every solution
    matches the plain path (SLP matrix + matvec) to 1e-5, the bound the
    batch and single kernels' nearly singular entries already agree to."""
    ms = [g.create_mesh(*meshes.icosphere(s)) for s in (2, 3)]
    rng = np.random.default_rng(77)
    nk = 7
    mesh_of = np.array([0, 1, 1, 0, 1, 0, 1])
    ks = rng.uniform(0.3, 5.0, nk)
    q = [rng.standard_normal(ms[i].num_elements) + 1j * rng.standard_normal(ms[i].num_elements) for i in mesh_of]
    P, it, rel, conv = g.solve_sweep_batched(ms, ks, mesh_of, q=q, tol=1e-7, precision=precision, ctx=gpu_ctx,
                                             check=False)
    assert all(conv)
    for f in range(nk):
        p1, it1, res1 = g.solve_cbie(ms[mesh_of[f]], float(ks[f]), q[f], tol=1e-7, precision=precision, ctx=gpu_ctx)
        assert np.abs(P[f] - p1).max() <= 1e-5 * np.abs(p1).max(), f


def test_sweep_plan_in_place_staging(gpu_ctx):
    """nihu_gb_sweep_plan_host_buffers: Neumann data written straight into the
    plan's pinned staging give the same pressures as host arrays passed in."""
    import ctypes
    L = g.lib()
    ms = [g.create_mesh(*meshes.icosphere(s)) for s in (1, 2)]
    mesh_of = np.array([0, 1, 1, 0, 1], np.int32)
    plan = g.SweepPlan(ms, mesh_of, k_max=4.0, tol=1e-7, ctx=gpu_ctx)
    rng = np.random.default_rng(8)
    ks = rng.uniform(0.3, 4.0, len(mesh_of))
    q = [rng.standard_normal(ms[i].num_elements) + 1j * rng.standard_normal(ms[i].num_elements) for i in mesh_of]
    P_ref, it_ref, _, _ = plan.run(ks, q, check=False)
    qp, pp = ctypes.c_void_p(), ctypes.c_void_p()
    gpu_ctx.check(L.nihu_gb_sweep_plan_host_buffers(plan.handle, ctypes.byref(qp), ctypes.byref(pp)))
    total = sum(ms[i].num_elements for i in mesh_of)
    qbuf = np.frombuffer((ctypes.c_double * (2 * total)).from_address(qp.value), np.complex128)
    pbuf = np.frombuffer((ctypes.c_double * (2 * total)).from_address(pp.value), np.complex128)
    qbuf[:] = 0
    qbuf[:] = np.concatenate(q)
    it = np.zeros(len(mesh_of), np.int32)
    st = L.nihu_gb_sweep_plan_run(plan.handle, np.ascontiguousarray(ks).ctypes.data, qp, pp, it.ctypes.data, None, None)
    assert st in (0, 6)  # OK, or not converged (the plan's result is still written)
    assert list(it) == list(it_ref)
    assert np.array_equal(np.concatenate(P_ref), pbuf)
    # the Python front end's own copies are not views of the staging
    P2, _, _, _ = plan.run(ks * 0.5, q, check=False)
    assert not np.array_equal(np.concatenate(P_ref), np.concatenate(P2))
    # copy=False: views of the staging, the same values
    P3, _, _, _ = plan.run(ks, q, check=False, copy=False)
    assert np.shares_memory(P3[0], pbuf) and np.array_equal(np.concatenate(P3), np.concatenate(P_ref))
    plan.close()
