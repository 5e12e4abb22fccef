"""Serving loop (nihu_gb_server_*): continuous batching of CBIE solves with
device-resident Krylov state, against the plain single-instance path and the
FP64 oracle; a result is the same alone and in any mix."""
import numpy as np
import pytest

import nihu_gb300 as g
from nihu_gb300 import meshes

pytestmark = pytest.mark.gpu


def _requests(rng, mesh_arrays, count, kmax=3.0):
    out = []
    for _ in range(count):
        i = int(rng.integers(len(mesh_arrays)))
        k = float(rng.uniform(0.5, kmax))
        d = rng.standard_normal(3)
        out.append((i, k, meshes.plane_wave_neumann(*mesh_arrays[i], k, [d])[:, 0]))
    return out


def _drain(server, limit=10000):
    res = {}
    for _ in range(limit):
        q, a, _d = server.step()
        while True:
            t = server.take()
            if t is None:
                break
            res[t[0]] = t
        if q == 0 and a == 0:
            return res
    raise AssertionError("server did not drain")


def test_server_matches_plain_path_and_oracle(gpu_ctx, oracle):
    arrays = [meshes.icosphere(s) for s in (1, 2, 3)]
    ms = [g.create_mesh(*a) for a in arrays]
    rng = np.random.default_rng(21)
    reqs = _requests(rng, arrays, 12)
    sv = g.Server(ms, tol=1e-7, quantum=6, ctx=gpu_ctx)
    ids = [sv.submit(i, k, q) for i, k, q in reqs]
    res = _drain(sv)
    assert sorted(res) == ids
    for rid, (i, k, q) in zip(ids, reqs):
        _, p, it, rel, conv = res[rid]
        assert conv and rel < 1e-7
        p1, it1, _ = g.solve_cbie(ms[i], k, q, tol=1e-7, ctx=gpu_ctx)
        assert np.abs(p - p1).max() / np.abs(p1).max() < 1e-5
        assert abs(it - it1) <= 1
    # one request on the finest mesh against the FP64 oracle
    rid = next(r for r, (i, _, _) in zip(ids, reqs) if i == 2)
    i, k, q = reqs[ids.index(rid)]
    n = ms[2].num_elements
    L = oracle.assemble(arrays[2], arrays[2], oracle.HELMHOLTZ, oracle.SLP, k, threads=8)
    M = oracle.assemble(arrays[2], arrays[2], oracle.HELMHOLTZ, oracle.DLP, k, threads=8) - 0.5 * np.eye(n)
    p_ref = np.linalg.solve(M, L @ q)
    assert np.abs(res[rid][1] - p_ref).max() / np.abs(p_ref).max() < 1e-4
    sv.close()


def test_alone_and_in_the_mix_are_identical(gpu_ctx):
    arrays = [meshes.icosphere(s) for s in (1, 2, 3)]
    ms = [g.create_mesh(*a) for a in arrays]
    rng = np.random.default_rng(22)
    target = (1, 2.3, meshes.plane_wave_neumann(*arrays[1], 2.3, [[0.3, -0.5, 0.8]])[:, 0])
    # alone
    sv = g.Server(ms, restart=12, tol=1e-8, quantum=3, ctx=gpu_ctx)
    sv.submit(*target)
    alone = list(_drain(sv).values())[0]
    sv.close()
    # in a mix: others before it, with it, and arriving while it is in flight
    sv = g.Server(ms, restart=12, tol=1e-8, quantum=3, ctx=gpu_ctx)
    for i, k, q in _requests(rng, arrays, 5):
        sv.submit(i, k, q)
    sv.step()
    for i, k, q in _requests(rng, arrays, 3):
        sv.submit(i, k, q)
    tid = sv.submit(*target)
    for i, k, q in _requests(rng, arrays, 4):
        sv.submit(i, k, q)
    sv.step()
    for i, k, q in _requests(rng, arrays, 6):
        sv.submit(i, k, q)
    mixed = _drain(sv)[tid]
    sv.close()
    assert mixed[2] == alone[2]
    assert np.array_equal(mixed[1], alone[1])


def test_quantum_and_restart_resume_exactly(gpu_ctx):
    """Pausing inside a cycle and at a cycle end (quantum 1) gives the same
    result as one uninterrupted launch."""
    arrays = [meshes.icosphere(2)]
    ms = [g.create_mesh(*a) for a in arrays]
    q = meshes.plane_wave_neumann(*arrays[0], 4.0, [[1.0, 0.2, -0.1]])[:, 0]
    out = []
    for quantum in (0, 1, 4):
        sv = g.Server(ms, restart=5, tol=1e-9, quantum=quantum, ctx=gpu_ctx)
        sv.submit(0, 4.0, q)
        out.append(list(_drain(sv).values())[0])
        sv.close()
    assert out[0][2] > 10  # several restart cycles
    for o in out[1:]:
        assert o[2] == out[0][2] and np.array_equal(o[1], out[0][1])


def test_budget_admission_and_oversize_requests(gpu_ctx):
    arrays = [meshes.icosphere(s) for s in (2, 3)]
    ms = [g.create_mesh(*a) for a in arrays]
    n1 = ms[1].num_elements
    # room for one request of the 1280-element mesh at a time (its 8 n^2 DLP matrix + state)
    budget = 8 * n1 * n1 + 60 * 16 * n1 + (1 << 20)
    sv = g.Server(ms, hbm_budget_bytes=budget, tol=1e-6, quantum=0, ctx=gpu_ctx)
    sv.reserve()  # the whole budget mapped into the pool first: admission is unchanged
    rng = np.random.default_rng(23)
    ids = [sv.submit(1, float(k), meshes.plane_wave_neumann(*arrays[1], float(k), [rng.standard_normal(3)])[:, 0])
           for k in (1.0, 1.5, 2.0)]
    queued, active, done = sv.step()
    assert active + done == 1 and queued == 2
    res = _drain(sv)
    assert sorted(res) == ids and all(r[4] for r in res.values())
    with pytest.raises(g.NihuError):
        small = g.Server(ms, hbm_budget_bytes=1 << 20, ctx=gpu_ctx)
        small.submit(1, 1.0, np.ones(n1))
