"""Per-phase timing of the collocational assembly (and a target for ncu).

    python -m nihu_gb300.profile_assembly --subdiv 5 --k 5 --budget-mb 1536

assembles the Helmholtz SLP and DLP matrices of an icosphere (with ``--bm``
the two Burton-Miller system matrices instead).

    python -m nihu_gb300.profile_assembly --sweep 16 --subdiv 4
    python -m nihu_gb300.profile_assembly --sweep-config4

run a frequency sweep instead (nihu_gb_solve_sweep_batched: the frequency-batch
assembly kernels and one persistent GMRES launch): `--sweep N` solves N wave
numbers uniform in [0.1, 10] on one icosphere, `--sweep-config4` the
256 wave numbers on icospheres of 320 / 1280 / 5120 triangles.  Both run the
sweep twice (the first call builds the near-pair lists).  With
``--budget-mb`` the context's HBM budget forces host output in column panels,
so every kernel launch covers one panel of the full-size problem while the
device holds only about the budget -- small enough for an ``ncu`` capture of
a single launch (``-k regex:k_regular -c 1``).  Without it both matrices are
assembled into device memory in one launch each.  Prints the per-phase device
times of the last repetition.
"""
from __future__ import annotations

import argparse
import ctypes
import json

import numpy as np

from . import _capi as C
from . import api, meshes


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--subdiv", type=int, default=5, help="icosphere subdivisions (20 * 4^s triangles)")
    ap.add_argument("--cylinder", type=int, default=0, metavar="N_THETA",
                    help="closed quad cylinder with this many elements around instead (n_z = 1.25 n_theta)")
    ap.add_argument("--k", type=float, default=5.0, help="wave number")
    ap.add_argument("--laplace", action="store_true")
    ap.add_argument("--budget-mb", type=int, default=0, help="HBM budget: host output in column panels")
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--fp64", action="store_true", help="FP64 regular quadrature")
    ap.add_argument("--bm", action="store_true", help="the Burton-Miller system (nihu_gb_assemble_burton_miller, "
                                                     "coupling -i/k) instead of SLP and DLP")
    ap.add_argument("--sweep", type=int, default=0, metavar="N", help="frequency sweep of N wave numbers")
    ap.add_argument("--sweep-config4", action="store_true", help="the 256-instance sweep on three icospheres")
    a = ap.parse_args(argv)
    if a.sweep or a.sweep_config4:
        return sweep(a)

    if a.cylinder:
        nt = a.cylinder
        nodes, elems = meshes.cylinder(nt, int(1.25 * nt), max(2, nt // 10))
    else:
        nodes, elems = meshes.icosphere(a.subdiv)
    ctx = api.Context(0, hbm_budget_bytes=a.budget_mb << 20)
    L = C.lib()
    dm = api.DeviceMesh(ctx, nodes, elems)
    n = dm.n
    fam = C.LAPLACE_3D if a.laplace else C.HELMHOLTZ_3D
    prec = C.REGULAR_FP64 if a.fp64 else C.REGULAR_FP32
    if a.budget_mb:
        hs = np.zeros((n, n), np.complex64, order="F")
        hd = np.zeros((n, n), np.complex64, order="F")
        ps, pd, where = hs.ctypes.data, hd.ctypes.data, C.HOST
    else:
        ps, pd = ctypes.c_void_p(), ctypes.c_void_p()
        ctx.check(L.nihu_gb_device_alloc(ctx.handle, 8 * n * n, ctypes.byref(ps)))
        ctx.check(L.nihu_gb_device_alloc(ctx.handle, 8 * n * n, ctypes.byref(pd)))
        where = C.DEVICE
    ctx.set_profiling(True)
    for r in range(a.reps):
        ctx.profile_reset()
        if a.bm:
            c = api.burton_miller_coupling(a.k) if fam == C.HELMHOLTZ_3D else 1.0 + 0.0j
            ctx.check(L.nihu_gb_assemble_burton_miller(ctx.handle, dm.handle, fam, a.k, c.real, c.imag, prec, C.C64,
                                                       pd, ps, n, where))
        else:
            ctx.check(L.nihu_gb_assemble(ctx.handle, dm.handle, dm.handle, fam, C.SLP | C.DLP, a.k, 1.0, 0.0, prec,
                                         C.C64, ps, pd, n, 0, where))
    prof = ctx.profile()
    print(json.dumps({"n_elements": n, "where": "host panels" if a.budget_mb else "device",
                      "phases_ms": {k: round(v[0], 4) for k, v in prof.items()},
                      "launches": {k: v[1] for k, v in prof.items()}}))
    ctx.close()


def sweep(a):
    rng = np.random.default_rng(2026)
    if a.sweep_config4:
        mesh_list = [api.create_mesh(*meshes.icosphere(s_)) for s_ in (2, 3, 4)]
        ks = rng.uniform(0.1, 10.0, 256)
        mesh_of = np.arange(256) % 3
    else:
        mesh_list = [api.create_mesh(*meshes.icosphere(a.subdiv))]
        ks = rng.uniform(0.1, 10.0, a.sweep)
        mesh_of = np.zeros(a.sweep, np.int32)
    ctx = api.Context(0)
    ctx.set_profiling(True)
    for _ in range(2):
        ctx.profile_reset()
        P, it, rel, conv = api.solve_sweep_batched(mesh_list, ks, mesh_of, restart=50, max_iters=1000, tol=1e-6,
                                                   ctx=ctx, check=False)
    prof = ctx.profile()
    print(json.dumps({"instances": len(ks), "meshes": [m.num_elements for m in mesh_list],
                      "iterations_total": int(np.sum(it)), "converged": int(np.sum(conv)),
                      "phases_ms": {k: round(v[0], 4) for k, v in prof.items()},
                      "launches": {k: v[1] for k, v in prof.items()}}))
    ctx.close()


if __name__ == "__main__":
    main()
