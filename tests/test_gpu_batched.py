"""Persistent batched GMRES (nihu_gb_solve_batched / nihu_gb_solve_sweep_batched)
against the single-system GPU GMRES, numpy and the FP64 oracle."""
import numpy as np
import pytest

import nihu_gb300 as g
from nihu_gb300 import meshes

pytestmark = pytest.mark.gpu


def _system(rng, n, shift=3.0):
    A = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(2 * n)
    A = (A + shift * np.eye(n)).astype(np.complex64)
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    return np.asfortranarray(A), b


def test_uneven_sizes_match_single_system_gmres(gpu_ctx):
    rng = np.random.default_rng(11)
    sizes = [1, 2, 3, 17, 64, 129, 257, 1000, 1281]
    systems = [_system(rng, n, shift=1.5 + 0.2 * i) for i, n in enumerate(sizes)]
    xs, it, rel, conv = g.solve_batched([A for A, _ in systems], [b for _, b in systems], restart=30,
                                        max_iters=500, tol=1e-7, ctx=gpu_ctx)
    assert conv.all() and (rel < 1e-7).all()
    for f, (A, b) in enumerate(systems):
        x_ref = np.linalg.solve(A.astype(np.complex128), b)
        assert np.abs(xs[f] - x_ref).max() / np.abs(x_ref).max() < 1e-5, sizes[f]
        x1, it1, rel1 = g.gmres(A, b, restart=30, max_iters=500, tol=1e-7, ctx=gpu_ctx)
        assert np.abs(xs[f] - x1).max() / np.abs(x1).max() < 1e-5, sizes[f]
        assert abs(int(it[f]) - it1) <= 1, (sizes[f], it[f], it1)


def test_restart_cycles_and_iteration_cap(gpu_ctx):
    rng = np.random.default_rng(12)
    # eigenvalues in a unit disc around 1.6: restarted GMRES(8) needs several
    # cycles (24 iterations in exact arithmetic to 1e-5; the tolerance stays
    # well above the FP32 matvec's rounding level, where counts would depend
    # on summation order)
    n = 300
    A, b = _system(rng, n, shift=1.6)
    x1, it1, rel1 = g.gmres(A, b, restart=8, max_iters=400, tol=1e-5, ctx=gpu_ctx)
    xs, it, rel, conv = g.solve_batched([A], [b], restart=8, max_iters=400, tol=1e-5, ctx=gpu_ctx)
    assert abs(int(it[0]) - 24) <= 1 and abs(it1 - 24) <= 1
    A64 = A.astype(np.complex128)
    for x in (xs[0], x1):
        assert np.linalg.norm(b - A64 @ x) / np.linalg.norm(b) < 1.5e-5
    assert np.abs(xs[0] - x1).max() / np.abs(x1).max() < 1e-4
    # the cap ends the solve and is reported
    with pytest.raises(g.NotConvergedError):
        g.solve_batched([A], [b], restart=8, max_iters=5, tol=1e-12, ctx=gpu_ctx)
    xs, it, rel, conv = g.solve_batched([A, A], [b, b], restart=8, max_iters=5, tol=1e-12, ctx=gpu_ctx, check=False)
    assert list(it) == [5, 5] and not conv.any() and (rel > 1e-12).all()


def test_zero_rhs_and_empty_batch(gpu_ctx):
    rng = np.random.default_rng(13)
    A, b = _system(rng, 40)
    xs, it, rel, conv = g.solve_batched([A, A], [np.zeros(40), b], ctx=gpu_ctx)
    assert np.all(xs[0] == 0) and it[0] == 0 and conv[0]
    assert conv[1] and it[1] > 0
    xs, it, rel, conv = g.solve_batched([], [], ctx=gpu_ctx)
    assert xs == [] and len(it) == 0


def test_alone_and_in_a_batch_are_identical(gpu_ctx):
    """A system's result does not depend on what else is in the launch."""
    rng = np.random.default_rng(14)
    sizes = [513, 64, 1000, 200, 1000, 7]
    systems = [_system(rng, n) for n in sizes]
    xs, it, _, _ = g.solve_batched([A for A, _ in systems], [b for _, b in systems], tol=1e-8, ctx=gpu_ctx)
    for f in (0, 2, 5):
        x1, it1, _, _ = g.solve_batched([systems[f][0]], [systems[f][1]], tol=1e-8, ctx=gpu_ctx)
        assert it1[0] == it[f]
        assert np.array_equal(x1[0], xs[f])


def test_invalid_arguments(gpu_ctx):
    rng = np.random.default_rng(15)
    A, b = _system(rng, 10)
    with pytest.raises(g.InvalidArgumentError):
        g.solve_batched([A], [b], restart=0, ctx=gpu_ctx)
    with pytest.raises(g.InvalidArgumentError):
        g.solve_batched([A], [b], max_iters=0, ctx=gpu_ctx)


def test_sweep_over_meshes_matches_plain_path(gpu_ctx, oracle):
    ms = [g.create_mesh(*meshes.icosphere(s)) for s in (1, 2, 3)]
    rng = np.random.default_rng(16)
    ks = rng.uniform(0.1, 2.8, 12)
    mesh_of = np.arange(12) % 3
    P, it, rel, conv = g.solve_sweep_batched(ms, ks, mesh_of, restart=50, max_iters=1000, tol=1e-7, ctx=gpu_ctx)
    assert conv.all()
    for f, k in enumerate(ks):
        m = ms[mesh_of[f]]
        n = m.num_elements
        assert P[f].shape == (n,)
        p1, it1, _ = g.solve_cbie(m, float(k), np.ones(n), restart=50, max_iters=1000, tol=1e-7, ctx=gpu_ctx)
        assert np.abs(P[f] - p1).max() / np.abs(p1).max() < 1e-5
        assert abs(int(it[f]) - it1) <= 1
        if n >= 320:
            pa = -1.0 / (1 + 1j * k)
            assert np.abs(P[f] - pa).max() / abs(pa) < 0.05
    # one instance of the finest mesh against the FP64 oracle
    f = 2
    mesh_arr = meshes.icosphere(3)
    n = len(mesh_arr[1])
    k = float(ks[f])
    L = oracle.assemble(mesh_arr, mesh_arr, oracle.HELMHOLTZ, oracle.SLP, k, threads=8)
    M = oracle.assemble(mesh_arr, mesh_arr, oracle.HELMHOLTZ, oracle.DLP, k, threads=8) - 0.5 * np.eye(n)
    p_ref = np.linalg.solve(M, L @ np.ones(n))
    assert np.abs(P[f] - p_ref).max() / np.abs(p_ref).max() < 1e-4


def test_sweep_per_instance_neumann_data(gpu_ctx):
    ms = [g.create_mesh(*meshes.icosphere(s)) for s in (1, 2)]
    ks = np.array([0.7, 1.3, 2.1])
    mesh_of = np.array([1, 0, 1])
    rng = np.random.default_rng(17)
    q = [rng.standard_normal(ms[i].num_elements) + 1j * rng.standard_normal(ms[i].num_elements) for i in mesh_of]
    P, it, rel, conv = g.solve_sweep_batched(ms, ks, mesh_of, q=q, tol=1e-7, ctx=gpu_ctx)
    for f in range(3):
        p1, _, _ = g.solve_cbie(ms[mesh_of[f]], float(ks[f]), q[f], tol=1e-7, ctx=gpu_ctx)
        assert np.abs(P[f] - p1).max() / np.abs(p1).max() < 1e-5
