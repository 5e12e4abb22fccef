#!/usr/bin/env python3
"""Headline benchmark of the dense collocation BEM hot path on one GB300.

Workload (the large single instance): unit icosphere subdivided 5 times
(20480 flat constant triangles), Helmholtz 3D, k = 5; one step assembles both
the SLP and the DLP matrix (2 x 20480^2 complex64 entries, regular quadrature
in FP32, singular and nearly singular entries in FP64) into device memory.
Metric: BEM entries per second (SLP and DLP entries counted separately).

Also reported, in the same JSON line:
  e2e          the same metric through the C ABI with host buffers: mesh arrays
               uploaded and both matrices copied to pinned host memory per step
  roofline     achieved HBM bandwidth of the dominant kernel (assemble_regular)
  solve        GMRES(50) to 1e-6 on (DLP - I/2) p = SLP q (pulsating sphere),
               FP32 matvec / FP64 Arnoldi, with matvec bandwidth
  cpu_baseline the FP64 CPU oracle on the host cores on a sample of rows

--impl reference times the CPU restatement of NiHu's assembly (the oracle) on
all host cores instead, on a bounded row sample per step.
Multi-GPU: replicas only (every rank assembles the same instance on its GPU).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SUBDIV = 5
K_WAVE = 5.0
METRIC = "BEM entries/s"
UNIT = "entries/s"


def parse(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--cpu-seconds", type=float, default=15.0, help="CPU baseline sample budget")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-solve", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--config", default="large",
                   choices=["large", "small", "multirhs", "sweep", "serve", "bm", "p2p", "galerkin", "profile"],
                   help="large: the headline line (20480-triangle icosphere), with short runs of the small, "
                        "multirhs, sweep and serve configurations in its 'configs' object; multirhs: the "
                        "40000-quad cylinder with 64 plane waves; sweep: 256 wave numbers on three icospheres; "
                        "serve: the served stream; bm: the Burton-Miller system on the 20480-triangle icosphere; "
                        "p2p: the Burton-Miller near field of a box partition of the same mesh; "
                        "galerkin: Galerkin SLP and DLP on the same mesh (each a separate line); "
                        "profile: per-phase device times of one assembly or sweep (an ncu target, see --subdiv)")
    p.add_argument("--no-configs", action="store_true", help="large: leave out the short runs of the other configs")
    p.add_argument("--no-fp64-check", action="store_true",
                   help="multirhs: leave out the per-right-hand-side error against the FP64 solution")
    p.add_argument("--requests", type=int, default=1000, help="serve: requests in the stream")
    p.add_argument("--quantum", type=int, default=8, help="serve: GMRES steps per system per round")
    p.add_argument("--plain-sample", type=int, default=4, help="serve: requests per mesh timed on the plain path")
    prof = p.add_argument_group("profile", "--config profile: the assembly of one mesh, or a sweep")
    prof.add_argument("--subdiv", type=int, default=5, help="icosphere subdivisions (20 * 4^s triangles)")
    prof.add_argument("--cylinder", type=int, default=0, metavar="N_THETA",
                      help="closed quad cylinder with this many elements around instead (n_z = 1.25 n_theta, "
                           "15 n_theta / 160 cap rings: 160 gives the 40000-quad cylinder's proportions)")
    prof.add_argument("--k", type=float, default=5.0, help="wave number")
    prof.add_argument("--laplace", action="store_true")
    prof.add_argument("--budget-mb", type=int, default=0,
                      help="HBM budget: host output in column panels, so that one launch covers one panel")
    prof.add_argument("--reps", type=int, default=2)
    prof.add_argument("--fp64", action="store_true", help="FP64 regular quadrature")
    prof.add_argument("--bm", action="store_true", help="the Burton-Miller system instead of SLP and DLP")
    prof.add_argument("--sweep", type=int, default=0, metavar="N", help="frequency sweep of N wave numbers")
    prof.add_argument("--sweep-config4", action="store_true", help="the 256-instance sweep on three icospheres")
    prof.add_argument("--gemm", type=int, nargs=3, default=None, metavar=("M", "N", "NRHS"),
                      help="the multi-RHS product Y = A X of a random complex64 M x N matrix in device memory")
    prof.add_argument("--gemm-mode", type=int, default=3, help="GEMM arithmetic (nihu_gb300.h NIHU_GB_GEMM_*)")
    return p.parse_args(argv)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def workload_config(n):
    return {
        "workload": "icosphere s=5 (%d flat constant triangles), Helmholtz 3D SLP+DLP collocation, k=5" % n,
        "n_elements": n,
        "entries_per_step": 2 * n * n,
        "storage": "complex64",
        "regular_quadrature": "fp32, distance-adaptive 1/3/6-point Dunavant",
        "singular_nearly_singular": "fp64 self terms; nearly singular static parts (semi-analytic) with fp64 plane frame, foot vectors and winding angle and fp32 angular point sums; fp32 nearly singular dynamic parts (42-point K_k - K_0)",
        "l2": "256 MB written between timed steps (L2 flushed); outputs 6.7 GB >> 129 MB L2",
        "parallelism": "replicas only (1 GPU per instance)",
    }


# ------------------------------------------------------------ CPU baseline

def cpu_sample(mesh, seconds, threads):
    """Time the FP64 oracle on a sample of full rows (SLP and DLP) on `threads`
    host threads; returns (entries/s, rows, elapsed)."""
    from oracle import oracle
    n = len(mesh[1])
    t0 = time.perf_counter()
    oracle.assemble(mesh, mesh, oracle.HELMHOLTZ, oracle.SLP, K_WAVE, rows=(0, 1))
    oracle.assemble(mesh, mesh, oracle.HELMHOLTZ, oracle.DLP, K_WAVE, rows=(0, 1))
    per_row = time.perf_counter() - t0
    rows = int(max(threads, min(8192, seconds * threads / max(per_row, 1e-6))))
    rows = max(threads, (rows // threads) * threads)
    t0 = time.perf_counter()
    # contiguous blocks spread over the sphere: row ranges of equal size
    blocks = np.linspace(0, n, threads + 1).astype(int)
    per = rows // threads
    errs = []

    def work(b):
        try:
            a = int(blocks[b])
            for op in (oracle.SLP, oracle.DLP):
                oracle.assemble(mesh, mesh, oracle.HELMHOLTZ, op, K_WAVE, rows=(a, min(n, a + per)))
        except Exception as e:  # pragma: no cover
            errs.append(e)

    ts = [threading.Thread(target=work, args=(b,)) for b in range(threads)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    el = time.perf_counter() - t0
    if errs:
        raise errs[0]
    return 2.0 * per * threads * n / el, per * threads, el


def run_reference(args):
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo", init_method="env://")
        dist.barrier()
        if rank != 0:
            dist.destroy_process_group()
            return
    from oracle import oracle
    from nihu_gb300 import meshes
    oracle.build()
    mesh = meshes.icosphere(SUBDIV)
    n = len(mesh[1])
    threads = os.cpu_count() or 1
    per_step = max(2.0, min(12.0, 150.0 / max(1, args.steps + args.warmup)))
    for _ in range(args.warmup):
        cpu_sample(mesh, 0.5, threads)
    vals, rows_tot, el_tot = [], 0, 0.0
    for _ in range(args.steps):
        v, rows, el = cpu_sample(mesh, per_step, threads)
        vals.append(v)
        rows_tot += rows
        el_tot += el
    value = float(np.mean(vals))
    # a step is one bounded row sample of the workload (timed), not the whole
    # 2 n^2 entries, which would take minutes per step on the host
    ms_per_step = 1e3 * el_tot / max(1, args.steps)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp64", "data": "synthetic (icosphere mesh generated in-process)", "impl": "reference",
        "config": workload_config(n),
        "step": "one sample of %d full rows (both matrices); ms_per_step is its measured time; the whole "
                "20480 x 20480 pair at this rate would take %.0f ms" % (rows_tot // max(1, args.steps),
                                                                        1e3 * 2.0 * n * n / value),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "%d full rows x %d columns x (SLP, DLP) per step, FP64 restatement of NiHu's "
                                   "collocational assembly (the reference needs Eigen/Boost, absent)" % (rows_tot // max(1, args.steps), n)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


# ------------------------------------------------------------ clocks

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------ our arm

def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def recorded_traffic():
    """Per-launch DRAM bytes of the regular kernel from the committed ncu summary, if any."""
    try:
        with open(os.path.join(ROOT, "profiles", "roofline_traffic.json")) as f:
            d = json.load(f)
        return d
    except (OSError, ValueError):
        return None


def replicas_summary(ms_per_step, units_per_step, dist=None, device="cpu"):
    """Replicas: the slowest rank's step time (all-reduce MAX) and the whole
    job's throughput, every rank processing units_per_step per step."""
    ws = 1
    if dist is not None:
        import torch
        ws = dist.get_world_size()
        t = torch.tensor([ms_per_step], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_per_step = float(t.item())
    return ms_per_step, units_per_step * ws / (ms_per_step / 1e3)


def run_ours(args):
    import torch

    import nihu_gb300 as g
    from nihu_gb300 import meshes
    from nihu_gb300 import _capi as C

    ws, rank, local = dist_env()
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo", init_method="env://")
    torch.cuda.set_device(local)
    L = g.lib()
    mesh = meshes.icosphere(SUBDIV)
    nodes, elems = mesh
    n = len(elems)
    ctx = g.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))
    dm = g.api.DeviceMesh(ctx, nodes, elems)
    mat_bytes = n * n * 8
    ps, pd = ctypes.c_void_p(), ctypes.c_void_p()
    ctx.check(L.nihu_gb_device_alloc(ctx.handle, mat_bytes, ctypes.byref(ps)))
    ctx.check(L.nihu_gb_device_alloc(ctx.handle, mat_bytes, ctypes.byref(pd)))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def step():
        ctx.check(L.nihu_gb_assemble(ctx.handle, dm.handle, dm.handle, C.HELMHOLTZ_3D, C.SLP | C.DLP, K_WAVE, 1.0, 0.0,
                                     C.REGULAR_FP32, C.C64, ps, pd, n, 0, C.DEVICE))

    for _ in range(args.warmup):
        step()
    counts = (ctypes.c_int64 * 11)()
    ctx.check(L.nihu_gb_pair_statistics(ctx.handle, dm.handle, dm.handle, counts))
    counts = np.array(list(counts))
    n_regular = int(counts[2:].sum())

    ctx.set_profiling(True)
    ctx.profile_reset()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = ctx.launch_count
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    torch.cuda.synchronize()
    t_wall0 = time.perf_counter()
    for s in range(args.steps):
        flush.fill_(s & 0xFF)  # evict the previous step's lines from L2 (not timed)
        torch.cuda.synchronize()
        ev[s][0].record(stream)
        step()
        ev[s][1].record(stream)
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall0
    launches = ctx.launch_count - launches0
    clk = clocks.stop()
    prof = ctx.profile()
    ctx.set_profiling(False)
    step_ms = [a.elapsed_time(b) for a, b in ev]
    entries = 2.0 * n * n
    ms_per_step, value = replicas_summary(float(np.mean(step_ms)), entries, dist, "cuda")

    reg_ms, reg_n = prof.get("assemble_regular", (0.0, 0))
    sing_ms, sing_n = prof.get("assemble_singular", (0.0, 0))
    reg_avg = reg_ms / max(reg_n, 1)
    alg_bytes = 16.0 * n_regular  # one complex64 SLP + one complex64 DLP entry written per regular pair
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / (reg_avg / 1e3) / 1e9
    tr = recorded_traffic()
    traffic = None
    if tr and tr.get("kernel") == "k_regular2" and tr.get("n_elements") == n:
        traffic = tr.get("dram_bytes_per_launch")
    roofline = {"kernel": "k_regular2 (assemble_regular.cu)", "bound": "hbm", "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                "peak_source": "%s (MEASURED_PEAKS.json hbm_gbs)" % peak_kind if peak_kind == "measured" else "fallback 6.8 TB/s",
                "algorithmic_bytes_per_launch": alg_bytes, "avg_launch_ms": reg_avg,
                "regular_pairs": n_regular, "near_pairs": int(counts[1]), "self_pairs": int(counts[0]),
                "level_histogram_slp_dlp": counts[2:].reshape(3, 3).tolist()}
    phases = {k: {"ms_per_step": v[0] / args.steps, "launches": v[1]} for k, v in prof.items()}

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32 regular quadrature, nearly singular dynamic parts and static angular sums, fp64 self terms and nearly singular geometry; complex64 storage",
        "data": "synthetic (icosphere mesh generated in-process)",
        "config": workload_config(n), "gpu_launches": int(launches), "clocks": clk, "roofline": roofline,
        "phases": phases, "wall_s_timed_region": t_wall,
    }

    # ---- e2e through the C ABI with host buffers
    if not args.no_e2e:
        hs, hd = ctypes.c_void_p(), ctypes.c_void_p()
        ctx.check(L.nihu_gb_host_alloc(ctx.handle, mat_bytes, ctypes.byref(hs)))
        ctx.check(L.nihu_gb_host_alloc(ctx.handle, mat_bytes, ctypes.byref(hd)))
        e2e_steps = max(1, min(args.steps, 5))

        def e2e_step():
            m = ctypes.c_void_p()
            ctx.check(L.nihu_gb_mesh_create(ctx.handle, nodes.ctypes.data, len(nodes), elems.ctypes.data, n,
                                            elems.shape[1], ctypes.byref(m)))
            ctx.check(L.nihu_gb_assemble(ctx.handle, m, m, C.HELMHOLTZ_3D, C.SLP | C.DLP, K_WAVE, 1.0, 0.0,
                                         C.REGULAR_FP32, C.C64, hs, hd, n, 0, C.HOST))
            L.nihu_gb_mesh_destroy(m)

        e2e_step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            e2e_step()
        torch.cuda.synchronize()
        e2e_ms = (time.perf_counter() - t0) * 1e3 / e2e_steps
        # spot check of the host copy against the device matrices (first column)
        col = np.ctypeslib.as_array(ctypes.cast(hs, ctypes.POINTER(ctypes.c_float)), shape=(2 * n,)).copy()
        dcol = np.zeros(2 * n, np.float32)
        ctx.check(L.nihu_gb_memcpy(ctx.handle, dcol.ctypes.data, C.HOST, ps, C.DEVICE, 8 * n))
        out["e2e"] = {"value": entries * ws / (e2e_ms / 1e3), "unit": UNIT,
                      "h2d_bytes_per_step": int(nodes.nbytes + elems.nbytes), "d2h_bytes_per_step": int(2 * mat_bytes),
                      "ms_per_step": e2e_ms, "steps": e2e_steps,
                      "path": "nihu_gb_mesh_create + nihu_gb_assemble(where=HOST, pinned) + nihu_gb_mesh_destroy",
                      "host_matches_device_first_column": bool(np.array_equal(col, dcol))}
        L.nihu_gb_host_free(hs)
        L.nihu_gb_host_free(hd)

    # ---- GMRES solve on the assembled matrices
    if not args.no_solve:
        ctx.check(L.nihu_gb_add_identity(ctx.handle, dm.handle, -0.5, 0.0, C.C64, pd, n, C.DEVICE))
        q = np.ones(n, np.complex128)
        dq, drhs, dp = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        for p_ in (dq, drhs, dp):
            ctx.check(L.nihu_gb_device_alloc(ctx.handle, 16 * n, ctypes.byref(p_)))
        ctx.check(L.nihu_gb_memcpy(ctx.handle, dq, C.DEVICE, q.ctypes.data, C.HOST, 16 * n))
        ctx.profile_reset()
        ctx.set_profiling(True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.check(L.nihu_gb_matvec(ctx.handle, C.C64, ps, n, n, n, dq, drhs, 1.0, 0.0, 0.0, 0.0, C.DEVICE))
        ctx.check(L.nihu_gb_memcpy(ctx.handle, dp, C.DEVICE, np.zeros(n, np.complex128).ctypes.data, C.HOST, 16 * n))
        it, res = ctypes.c_int(0), ctypes.c_double(0.0)
        st = L.nihu_gb_gmres(ctx.handle, C.C64, pd, n, n, drhs, dp, 50, 1000, 1e-6, ctypes.byref(it),
                             ctypes.byref(res), C.DEVICE)
        torch.cuda.synchronize()
        solve_ms = (time.perf_counter() - t0) * 1e3
        prof = ctx.profile()
        ctx.set_profiling(False)
        p = np.zeros(n, np.complex128)
        ctx.check(L.nihu_gb_memcpy(ctx.handle, p.ctypes.data, C.HOST, dp, C.DEVICE, 16 * n))
        pa = -1.0 / (1 + 1j * K_WAVE)
        gm_ms, gm_n = prof.get("gemv_c64", (0.0, 0))
        gm_avg = gm_ms / max(gm_n, 1)
        out["solve"] = {
            "solver": "GMRES(50), FP32 matvec (complex64 matrix), FP64 CGS2 Arnoldi, tol 1e-6",
            "status": int(st), "iterations": it.value, "rel_residual": res.value, "ms": solve_ms,
            "matvecs": gm_n, "matvec_avg_ms": gm_avg,
            "matvec_gbs": 8.0 * n * n / (gm_avg / 1e3) / 1e9 if gm_avg else None,
            "matvec_frac_of_hbm": (8.0 * n * n / (gm_avg / 1e3) / 1e9) / peak if gm_avg else None,
            "pressure_error_vs_analytic": float(np.abs(p - pa).max() / abs(pa)),
        }
        for p_ in (dq, drhs, dp):
            L.nihu_gb_device_free(ctx.handle, p_)

    L.nihu_gb_device_free(ctx.handle, ps)
    L.nihu_gb_device_free(ctx.handle, pd)
    dm.close()
    ctx.close()

    # ---- CPU baseline (rank 0, N = 1 only)
    if not args.no_cpu and rank == 0 and ws == 1:
        threads = os.cpu_count() or 1
        v, rows, el = cpu_sample(mesh, args.cpu_seconds, threads)
        out["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                               "sample": "%d full rows x %d columns x (SLP, DLP), FP64 oracle (restatement of NiHu's "
                                         "collocational assembly), %.1f s" % (rows, n, el)}
    if not args.no_configs and rank == 0 and ws == 1:
        out["configs"] = other_configs(args)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(out), flush=True)


def run_small(args):
    """Plain small case: icosphere of 1280 triangles, k = 1, complex128 SLP and
    DLP assembled in FP64 (nihu_gb_assemble), pulsating-sphere data q = 1, the
    right-hand side on the GPU and a dense FP64 LU solve (nihu_gb_lu_solve);
    surface pressure against the analytic -R/(1+ikR).  Timed device-resident
    (CUDA events) and end to end through nihu_gb_solve_cbie with host data; the
    CPU baseline is the FP64 oracle's assembly plus numpy's LU on the host
    cores, whose pressure also checks the GPU's."""
    import torch

    import nihu_gb300 as g
    from nihu_gb300 import _capi as C

    k = 1.0
    nodes, elems = g.meshes.icosphere(3)
    n = len(elems)
    mesh = g.create_mesh(nodes, elems)
    ctx = g.Context(0)
    L = g.lib()
    dm = mesh.device(ctx)
    ps, pd, pb, px = (ctypes.c_void_p() for _ in range(4))
    for p_, size in ((ps, 16 * n * n), (pd, 16 * n * n), (pb, 16 * n), (px, 16 * n)):
        ctx.check(L.nihu_gb_device_alloc(ctx.handle, size, ctypes.byref(p_)))
    q = np.ones(n, np.complex128)
    pq = ctypes.c_void_p()
    ctx.check(L.nihu_gb_device_alloc(ctx.handle, 16 * n, ctypes.byref(pq)))
    ctx.check(L.nihu_gb_memcpy(ctx.handle, pq, C.DEVICE, q.ctypes.data, C.HOST, 16 * n))
    stream = torch.cuda.ExternalStream(ctx.stream)

    def step():
        ctx.check(L.nihu_gb_assemble(ctx.handle, dm.handle, dm.handle, C.HELMHOLTZ_3D, C.SLP | C.DLP, k, 1.0, 0.0,
                                     C.REGULAR_FP64, C.C128, ps, pd, n, 0, C.DEVICE))
        ctx.check(L.nihu_gb_add_identity(ctx.handle, dm.handle, -0.5, 0.0, C.C128, pd, n, C.DEVICE))
        ctx.check(L.nihu_gb_matvec(ctx.handle, C.C128, ps, n, n, n, pq, pb, 1.0, 0.0, 0.0, 0.0, C.DEVICE))
        ctx.check(L.nihu_gb_lu_solve(ctx.handle, pd, n, n, pb, px, C.DEVICE))

    for _ in range(max(3, args.warmup)):
        step()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    torch.cuda.synchronize()
    for s_ in range(args.steps):
        ev[s_][0].record(stream)
        step()
        ev[s_][1].record(stream)
    torch.cuda.synchronize()
    ms = float(np.mean([a.elapsed_time(b) for a, b in ev]))
    p = np.zeros(n, np.complex128)
    ctx.check(L.nihu_gb_memcpy(ctx.handle, p.ctypes.data, C.HOST, px, C.DEVICE, 16 * n))
    ctx.set_profiling(True)
    ctx.profile_reset()
    step()
    phases = {kk: round(v[0], 3) for kk, v in ctx.profile().items()}
    ctx.set_profiling(False)
    # end to end: host data in, host pressure out, through the composite call
    e2e = []
    for _ in range(max(1, args.steps)):
        t0 = time.perf_counter()
        p_e2e, _, _ = g.solve_cbie(mesh, k, q, dtype=g.C128, solver="lu", precision="fp64", ctx=ctx)
        e2e.append(time.perf_counter() - t0)
    pa = -1.0 / (1.0 + 1j * k)
    out = {"metric": "plain small solve (config 1)", "impl": "ours", "value": ms, "unit": "ms",
           "higher_is_better": False, "n_elements": n, "k": k,
           "dtype": "complex128: FP64 assembly; FP32 LU with FP64 iterative refinement (FP64 LU fallback)",
           "data": "synthetic (icosphere generated in-process), pulsating sphere q = 1",
           "steps": args.steps, "ms_per_step": ms,
           "e2e": {"value": 1e3 * float(np.median(e2e)), "unit": "ms", "h2d_bytes_per_step": 16 * n + 20 * len(nodes),
                   "d2h_bytes_per_step": 16 * n, "path": "nihu_gb_solve_cbie(dtype=C128, solver=LU, FP64)"},
           "phases_ms": phases,
           "pressure_error_vs_analytic": float(np.abs(p - pa).max() / abs(pa)),
           "device_vs_e2e_max_rel_difference": float(np.abs(p - p_e2e).max() / np.abs(p).max())}
    if not args.no_cpu:
        from oracle import oracle
        oracle.build()
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        Ls = oracle.assemble((nodes, elems), (nodes, elems), oracle.HELMHOLTZ, oracle.SLP, k, same_mesh=True,
                             threads=threads)
        Ms = oracle.assemble((nodes, elems), (nodes, elems), oracle.HELMHOLTZ, oracle.DLP, k, same_mesh=True,
                             threads=threads) - 0.5 * np.eye(n)
        p_cpu = np.linalg.solve(Ms, Ls @ q)
        t_cpu = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": 1e3 * t_cpu, "unit": "ms", "cores": threads, "kind": "port",
                               "sample": "the whole solve: FP64 oracle assembly of both matrices on all host cores "
                                         "+ numpy LU"}
        out["pressure_gpu_vs_cpu_oracle"] = float(np.abs(p - p_cpu).max() / np.abs(p_cpu).max())
    for p_ in (ps, pd, pb, px, pq):
        L.nihu_gb_device_free(ctx.handle, p_)
    ctx.close()
    return out


def run_multirhs(args):
    """Multi-RHS precision path: closed cylinder R=1, L=4, 40000 flat quads,
    k=4, 64 plane waves with seeded uniform directions.  Times the assembly of
    SLP and DLP (complex64), the right-hand sides B = SLP Q (the FP32-accurate
    split-BF16 product, BF16x6 on tcgen05) and the mixed-precision refinement
    solve of (DLP - I/2) X = B (BF16x3 tcgen05 products inside GMRES, BF16x6
    residuals combined in FP64), and one product of every GEMM mode."""
    import torch

    import nihu_gb300 as g
    from nihu_gb300 import _capi as C
    from nihu_gb300 import meshes

    L = g.lib()
    k = 4.0
    nrhs = 64
    nodes, elems = meshes.cylinder_40k()
    n = len(elems)
    ctx = g.Context(0)
    dm = g.api.DeviceMesh(ctx, nodes, elems)
    ps, pd, pq, pb, px = (ctypes.c_void_p() for _ in range(5))
    for p_, size in ((ps, 8 * n * n), (pd, 8 * n * n), (pq, 16 * n * nrhs), (pb, 16 * n * nrhs), (px, 16 * n * nrhs)):
        ctx.check(L.nihu_gb_device_alloc(ctx.handle, size, ctypes.byref(p_)))
    Q = meshes.plane_wave_neumann(nodes, elems, k, meshes.sphere_directions(nrhs, seed=2026))
    ctx.check(L.nihu_gb_memcpy(ctx.handle, pq, C.DEVICE, Q.ctypes.data, C.HOST, Q.nbytes))
    counts = (ctypes.c_int64 * 11)()
    ctx.check(L.nihu_gb_pair_statistics(ctx.handle, dm.handle, dm.handle, counts))

    def assemble():
        ctx.check(L.nihu_gb_assemble(ctx.handle, dm.handle, dm.handle, C.HELMHOLTZ_3D, C.SLP | C.DLP, k, 1.0, 0.0,
                                     C.REGULAR_FP32, C.C64, ps, pd, n, 0, C.DEVICE))

    assemble()  # warm-up (builds the nearly singular pair list)
    ctx.set_profiling(True)
    ctx.profile_reset()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    steps = max(1, min(args.steps, 3))
    for _ in range(steps):
        assemble()
    torch.cuda.synchronize()
    asm_ms = (time.perf_counter() - t0) * 1e3 / steps
    prof_asm = ctx.profile()
    ctx.profile_reset()
    ctx.check(L.nihu_gb_add_identity(ctx.handle, dm.handle, -0.5, 0.0, C.C64, pd, n, C.DEVICE))
    # warm-up of every GEMM mode (the library's first call of a mode loads its kernels)
    for mode in (C.GEMM_FP32, C.GEMM_TF32, C.GEMM_BF16X9, C.GEMM_BF16X3, C.GEMM_BF16X6):
        ctx.check(L.nihu_gb_gemm(ctx.handle, mode, ps, n, n, n, pq, n, nrhs, px, n, 1.0, 0.0, 0.0, 0.0, C.DEVICE))
    torch.cuda.synchronize()
    ctx.profile_reset()
    t0 = time.perf_counter()
    ctx.check(L.nihu_gb_gemm(ctx.handle, C.GEMM_BF16X6, ps, n, n, n, pq, n, nrhs, pb, n, 1.0, 0.0, 0.0, 0.0, C.DEVICE))
    torch.cuda.synchronize()
    rhs_ms = (time.perf_counter() - t0) * 1e3
    # one product of each GEMM mode on the 40000 x 40000 matrix (64 right-hand sides)
    mode_ms = {}
    for mname, mode in (("fp32_cuda_cores_cublas", C.GEMM_FP32), ("tf32_tensor_cublas", C.GEMM_TF32),
                        ("bf16x9_tensor_cublas", C.GEMM_BF16X9), ("bf16x3_tcgen05", C.GEMM_BF16X3),
                        ("bf16x6_tcgen05", C.GEMM_BF16X6)):
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        ctx.check(L.nihu_gb_gemm(ctx.handle, mode, ps, n, n, n, pq, n, nrhs, px, n, 1.0, 0.0, 0.0, 0.0, C.DEVICE))
        torch.cuda.synchronize()
        ms_ = (time.perf_counter() - t1) * 1e3
        mode_ms[mname] = {"ms": ms_, "hbm_gbs": 8.0 * n * n / (ms_ / 1e3) / 1e9,
                          "complex_tflops": 8.0 * n * n * nrhs / (ms_ / 1e3) / 1e12}
    oi, ii = ctypes.c_int(0), ctypes.c_int(0)
    res = np.zeros(nrhs)
    torch.cuda.synchronize()
    ctx.profile_reset()  # the solve's phases alone
    t0 = time.perf_counter()
    st = L.nihu_gb_solve_multi(ctx.handle, pd, n, n, pb, px, nrhs, C.GEMM_BF16X3, C.GEMM_BF16X6, 30, 20, 1e-6, 1e-3,
                               ctypes.byref(oi), ctypes.byref(ii), res.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                               C.DEVICE)
    torch.cuda.synchronize()
    solve_ms = (time.perf_counter() - t0) * 1e3
    prof_solve = ctx.profile()
    ctx.set_profiling(False)
    err = fp64_error_per_rhs(ctx, L, C, dm, n, nrhs, k, pd, pq, px) if not args.no_fp64_check else None
    peak, _ = measured_peaks()
    gem = {}
    for name, (ms_, cnt) in prof_solve.items():
        if name.startswith("gemm"):
            avg = ms_ / max(cnt, 1)
            gem[name] = {"launches": cnt, "avg_ms": avg, "hbm_gbs": 8.0 * n * n / (avg / 1e3) / 1e9,
                         "hbm_frac": 8.0 * n * n / (avg / 1e3) / 1e9 / peak,
                         "tflops_complex": 8.0 * n * n * nrhs / (avg / 1e3) / 1e12}
            parts_products = {"gemm_bf16x3": 3, "gemm_bf16x6": 6}.get(name)
            if parts_products:
                # BF16 tensor work: products x 2 (2n rows of the float view) (2 nrhs) n
                gem[name]["tensor_tflops_bf16"] = parts_products * 2.0 * (2 * n) * (2 * nrhs) * n / (avg / 1e3) / 1e12
    out = {
        "metric": "multi-RHS solve (config 3)", "impl": "ours", "n_elements": n, "nrhs": nrhs, "k": k,
        "assembly_ms": asm_ms, "assembly_entries_per_s": 2.0 * n * n / (asm_ms / 1e3),
        "assembly_phases_ms": {kk: v[0] / steps for kk, v in prof_asm.items()},
        "near_pairs": int(counts[1]), "rhs_gemm_ms": rhs_ms, "solve_ms": solve_ms, "solve_status": int(st),
        "outer_iterations": oi.value, "inner_iterations": ii.value, "max_rel_residual": float(res.max()),
        "gemm": gem, "gemm_modes_one_product": mode_ms, "solves_per_s": nrhs / ((rhs_ms + solve_ms) / 1e3),
        "value": nrhs / ((rhs_ms + solve_ms) / 1e3), "unit": "solves/s", "err_per_rhs": err,
        "note": "max_rel_residual is |B - A X|/|B| of the complex64 system the solver sees; err_per_rhs is "
                "each right-hand side's solution against the FP64 solution of the FP64-quadrature system "
                "(the oracle's arithmetic; the GPU FP64 mode matches the oracle to 1e-11), reached by FP64 "
                "iterative refinement; tests/test_gpu_multi.py checks the solution against the oracle's own "
                "dense FP64 solve on a 10080-quad cylinder",
    }
    for p_ in (ps, pd, pq, pb, px):
        L.nihu_gb_device_free(ctx.handle, p_)
    dm.close()
    ctx.close()
    return out


def fp64_error_per_rhs(ctx, L, C, dm, n, nrhs, k, pd32, pq, px, steps=3):
    """Error of each right-hand side's solution X (device, complex128 n x nrhs)
    against the FP64 solution X64 of the FP64-quadrature system
    (DLP64 - I/2) X64 = SLP64 Q.  The FP64 matrices are assembled in the
    FP64 mode; X64 is reached from X by iterative refinement whose residuals
    B64 - A64 X64 are FP64 matrix-vector products and whose corrections are
    solved on the complex64 matrix pd32.  Returns max and median of
    |X - X64|_2 / |X64|_2 over the right-hand sides, and the FP64 relative
    residual of X itself."""
    col = 16 * n
    p64s, p64d, pb64, pr, pdx = (ctypes.c_void_p() for _ in range(5))
    for p_, size in ((p64s, 16 * n * n), (p64d, 16 * n * n), (pb64, col * nrhs), (pr, col * nrhs),
                     (pdx, col * nrhs)):
        ctx.check(L.nihu_gb_device_alloc(ctx.handle, size, ctypes.byref(p_)))
    try:
        ctx.check(L.nihu_gb_assemble(ctx.handle, dm.handle, dm.handle, C.HELMHOLTZ_3D, C.SLP | C.DLP, k, 1.0, 0.0,
                                     C.REGULAR_FP64, C.C128, p64s, p64d, n, 0, C.DEVICE))
        ctx.check(L.nihu_gb_add_identity(ctx.handle, dm.handle, -0.5, 0.0, C.C128, p64d, n, C.DEVICE))

        def cols(p_, j):
            return ctypes.c_void_p(p_.value + col * j)

        for j in range(nrhs):  # B64 = SLP64 Q
            ctx.check(L.nihu_gb_matvec(ctx.handle, C.C128, p64s, n, n, n, cols(pq, j), cols(pb64, j), 1.0, 0.0, 0.0,
                                       0.0, C.DEVICE))
        X = np.zeros((n, nrhs), np.complex128, order="F")
        ctx.check(L.nihu_gb_memcpy(ctx.handle, X.ctypes.data, C.HOST, px, C.DEVICE, X.nbytes))
        B64 = np.zeros_like(X)
        ctx.check(L.nihu_gb_memcpy(ctx.handle, B64.ctypes.data, C.HOST, pb64, C.DEVICE, B64.nbytes))
        X64 = X.copy(order="F")  # ndarray.copy defaults to C order
        res0 = None
        for s_ in range(steps):
            ctx.check(L.nihu_gb_memcpy(ctx.handle, pdx, C.DEVICE, X64.ctypes.data, C.HOST, X64.nbytes))
            ctx.check(L.nihu_gb_memcpy(ctx.handle, pr, C.DEVICE, pb64, C.DEVICE, col * nrhs))
            for j in range(nrhs):  # R = B64 - A64 X64
                ctx.check(L.nihu_gb_matvec(ctx.handle, C.C128, p64d, n, n, n, cols(pdx, j), cols(pr, j), -1.0, 0.0,
                                           1.0, 0.0, C.DEVICE))
            R = np.zeros_like(X)
            ctx.check(L.nihu_gb_memcpy(ctx.handle, R.ctypes.data, C.HOST, pr, C.DEVICE, R.nbytes))
            if res0 is None:
                res0 = np.linalg.norm(R, axis=0) / np.linalg.norm(B64, axis=0)
            oi, ii = ctypes.c_int(0), ctypes.c_int(0)
            rr = np.zeros(nrhs)
            ctx.check(L.nihu_gb_solve_multi(ctx.handle, pd32, n, n, pr, pdx, nrhs, C.GEMM_BF16X3, C.GEMM_BF16X6, 30, 20,
                                            1e-6, 1e-3, ctypes.byref(oi), ctypes.byref(ii),
                                            rr.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), C.DEVICE))
            D = np.zeros_like(X)
            ctx.check(L.nihu_gb_memcpy(ctx.handle, D.ctypes.data, C.HOST, pdx, C.DEVICE, D.nbytes))
            X64 += D
        e = np.linalg.norm(X - X64, axis=0) / np.linalg.norm(X64, axis=0)
        last = float((np.linalg.norm(D, axis=0) / np.linalg.norm(X64, axis=0)).max())
        return {"max": float(e.max()), "median": float(np.median(e)),
                "fp64_rel_residual_max": float(res0.max()), "refinement_steps": steps,
                "last_correction_rel": last,
                "reference": "FP64-quadrature matrices (GPU FP64 mode), FP64 residuals"}
    finally:
        for p_ in (p64s, p64d, pb64, pr, pdx):
            L.nihu_gb_device_free(ctx.handle, p_)


def run_sweep(args):
    """Batched frequency sweep: icospheres of 320, 1280 and 5120 triangles,
    256 wave numbers uniform in [0.1, 10] (seeded) dealt round-robin to the
    meshes; pulsating-sphere Neumann data; every instance assembled (complex64,
    FP64 singular terms) and solved by GMRES(50) to 1e-6 (at most 1000
    iterations).  The batched path (nihu_gb_solve_sweep_batched: one call,
    per-mesh frequency-batched assembly, one persistent GMRES launch over all
    256 systems) is timed against the plain single-instance path
    (nihu_gb_solve_cbie, one call per instance) on every instance.  The
    timed batched path is the sweep plan (nihu_gb_sweep_plan_*: the same work
    captured once as a CUDA graph and replayed); the eager single call is
    reported beside it."""
    import torch

    import nihu_gb300 as g

    rng = np.random.default_rng(2026)
    ks_all = rng.uniform(0.1, 10.0, 256)
    subdivs = (2, 3, 4)
    mesh_list = [g.create_mesh(*g.meshes.icosphere(s_)) for s_ in subdivs]
    mesh_of = np.arange(256) % 3
    sizes = [m.num_elements for m in mesh_list]
    ctx = g.Context(0)
    for m in mesh_list:
        m.device(ctx)
    restart, max_iters, tol = 50, 1000, 1e-6
    out = {"metric": "BEM solves/s (batched frequency sweep, config 4)", "impl": "ours", "unit": "solves/s",
           "instances": 256, "meshes": sizes, "restart": restart, "max_iters": max_iters, "tol": tol,
           "note": "the plain CBIE (DLP - I/2) p = SLP q is singular at the sphere's interior Dirichlet "
                   "eigenvalues (k = pi, 4.49, 5.76, ...); wave numbers close to them may stop at the "
                   "iteration cap on either path"}
    # eager path: one nihu_gb_solve_sweep_batched call (phases timed with CUDA events)
    ctx.set_profiling(True)
    for _ in range(max(1, args.warmup)):  # warm-up: near lists, scratch, code paths
        g.solve_sweep_batched(mesh_list, ks_all, mesh_of, restart=restart, max_iters=max_iters, tol=tol, ctx=ctx,
                              check=False)
    eager = []
    for _ in range(max(1, args.steps)):
        ctx.profile_reset()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g.solve_sweep_batched(mesh_list, ks_all, mesh_of, restart=restart, max_iters=max_iters, tol=tol, ctx=ctx,
                              check=False)
        torch.cuda.synchronize()
        eager.append(time.perf_counter() - t0)
    prof = ctx.profile()
    out["phases_ms"] = {k: round(v[0], 3) for k, v in prof.items()}
    out["launches"] = {k: v[1] for k, v in prof.items()}
    out["eager_seconds"] = float(np.median(eager))
    ctx.set_profiling(False)
    # the timed path: the sweep captured once as a CUDA graph, replayed per run
    # (host Neumann data in, host pressures out, every run)
    t0 = time.perf_counter()
    plan = g.SweepPlan(mesh_list, mesh_of, k_max=10.0, restart=restart, max_iters=max_iters, tol=tol, ctx=ctx)
    out["plan_create_seconds"] = time.perf_counter() - t0  # includes the autotuner's candidate replays
    out["plan_tuning"] = plan.tuning()
    q1 = [np.ones(sizes[i]) for i in mesh_of]
    for _ in range(max(1, args.warmup)):
        plan.run(ks_all, q1, check=False, copy=False)
    times = []
    for _ in range(max(1, args.steps)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        # host Neumann data written into the pinned staging, pressures read from it in place
        P, it, rel, conv = plan.run(ks_all, q1, check=False, copy=False)
        times.append(time.perf_counter() - t0)
    P = [p_.copy() for p_ in P]  # the last run's pressures, kept past close()
    plan.close()
    batched_s = float(np.median(times))
    out["batched_seconds"] = batched_s
    out["batched_seconds_all"] = times
    out["value"] = 256 / batched_s
    # plain single-instance path on every instance
    ctx.set_profiling(False)
    per_mesh = {}
    plain_s, agree, it_diff = 0.0, 0.0, []
    pa_err = []
    for f in range(256):
        m = mesh_list[mesh_of[f]]
        n = m.num_elements
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        p1, it1, res1 = g.solve_cbie(m, float(ks_all[f]), np.ones(n), restart=restart, max_iters=max_iters, tol=tol,
                                     ctx=ctx, check=False)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        plain_s += dt
        agree = max(agree, float(np.abs(P[f] - p1).max() / np.abs(p1).max()))
        it_diff.append(int(it[f]) - it1)
        pa = -1.0 / (1 + 1j * ks_all[f])
        pa_err.append(float(np.abs(P[f] - pa).max() / abs(pa)))
        d = per_mesh.setdefault(str(n), {"instances": 0, "plain_seconds": 0.0, "iterations": [], "converged": 0,
                                         "not_converged_k": [], "pressure_error_vs_analytic": []})
        d["instances"] += 1
        d["plain_seconds"] += dt
        d["iterations"].append(int(it[f]))
        if conv[f]:
            d["converged"] += 1
            d["pressure_error_vs_analytic"].append(pa_err[-1])
        else:
            d["not_converged_k"].append(round(float(ks_all[f]), 4))
    for d in per_mesh.values():
        its = np.array(d.pop("iterations"))
        errs = d.pop("pressure_error_vs_analytic")
        d["iterations_median"] = float(np.median(its))
        d["iterations_max"] = int(its.max())
        d["iterations_total"] = int(its.sum())
        d["pressure_error_vs_analytic_median"] = float(np.median(errs)) if errs else None
    out["per_mesh"] = per_mesh
    out["plain_seconds"] = plain_s
    out["plain_solves_per_s"] = 256 / plain_s
    out["speedup_vs_plain_gpu"] = out["value"] / out["plain_solves_per_s"]
    out["batched_vs_plain_max_rel_difference"] = agree
    out["iteration_difference_batched_minus_plain"] = {"max_abs": int(np.abs(it_diff).max()),
                                                       "equal": int(np.sum(np.array(it_diff) == 0))}
    # matrix bytes the solves stream: iterations + restarts, one n^2 complex64 matrix read each
    mat_bytes = sum(8.0 * sizes[mesh_of[f]] ** 2 * (int(it[f]) + int(it[f]) // restart) for f in range(256))
    gm = [v for k, v in prof.items() if k.startswith("persistent_gmres")]
    if gm:
        ms_ = gm[0][0]
        out["persistent_gmres"] = {"ms": ms_, "matrix_bytes": mat_bytes,
                                   "achieved_GBs": mat_bytes / (ms_ * 1e-3) / 1e9}
    ctx.close()
    return out


def run_serve(args):
    """Served stream: Poisson arrivals (seeded, mean 2000 requests/s) of
    exterior Helmholtz solves (rigid-body plane-wave scattering, CBIE with
    q = -dp_inc/dn) on icospheres of 320 / 1280 / 5120 / 20480 triangles with
    probabilities 0.4 / 0.3 / 0.2 / 0.1, k uniform in [0.5, 8], directions
    uniform on the sphere; a 150 GB HBM budget.  The serving loop
    (nihu_gb_server_*) runs on the wall clock: requests are submitted when
    their arrival time has passed, and a request's latency runs from its
    arrival to the round that returns it.  The plain single-instance path
    (nihu_gb_solve_cbie per request) is timed on a stratified sample."""
    import torch

    import nihu_gb300 as g

    rng = np.random.default_rng(5005)
    n_req = args.requests
    rate = 2000.0
    subdivs = (2, 3, 4, 5)
    probs = (0.4, 0.3, 0.2, 0.1)
    arrays = [g.meshes.icosphere(s_) for s_ in subdivs]
    mesh_list = [g.create_mesh(*a) for a in arrays]
    sizes = [m.num_elements for m in mesh_list]
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n_req))
    which = rng.choice(len(subdivs), size=n_req, p=probs)
    ks = rng.uniform(0.5, 8.0, n_req)
    dirs = rng.standard_normal((n_req, 3))
    qs = [g.meshes.plane_wave_neumann(*arrays[which[r]], ks[r], dirs[r:r + 1])[:, 0] for r in range(n_req)]
    ctx = g.Context(0)
    restart, max_iters, tol, quantum = 50, 1000, 1e-6, args.quantum
    server_kw = dict(hbm_budget_bytes=150 << 30, max_active=4096, restart=restart, max_iters=max_iters, tol=tol,
                     quantum=quantum, ctx=ctx)
    # warm-up: one request per mesh (near lists, code paths, memory pool)
    sv = g.Server(mesh_list, **server_kw)
    sv.reserve()  # the HBM budget mapped into the server's pool before serving starts
    for i in range(len(subdivs)):
        sv.submit(i, 1.0, np.ones(sizes[i]))
    while sv.step()[:2] != (0, 0):
        pass
    while sv.take() is not None:
        pass
    torch.cuda.synchronize()
    ctx.set_profiling(True)
    ctx.profile_reset()
    done_t = np.full(n_req, np.nan)
    results = {}
    id_of = {}
    steps = 0
    host = {"submit": 0.0, "step": 0.0, "take": 0.0, "idle": 0.0}
    t0 = time.perf_counter()
    nxt = 0
    n_done = 0
    while n_done < n_req:
        now = time.perf_counter() - t0
        while nxt < n_req and arrivals[nxt] <= now:
            id_of[sv.submit(int(which[nxt]), float(ks[nxt]), qs[nxt])] = nxt
            nxt += 1
        t_a = time.perf_counter()
        host["submit"] += t_a - t0 - now
        queued, active, _ = sv.step()
        steps += 1
        t_step = time.perf_counter() - t0
        host["step"] += t_step - (t_a - t0)
        while True:
            t = sv.take()
            if t is None:
                break
            r = id_of.pop(t[0])
            done_t[r] = t_step
            results[r] = t
            n_done += 1
        host["take"] += time.perf_counter() - t0 - t_step
        if queued == 0 and active == 0 and nxt < n_req:
            wait = arrivals[nxt] - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
                host["idle"] += wait
    t_end = float(np.nanmax(done_t))
    prof = ctx.profile()
    ctx.set_profiling(False)
    sv.close()
    lat = done_t - arrivals
    its = np.array([results[r][2] for r in range(n_req)])
    conv = np.array([results[r][4] for r in range(n_req)])
    out = {"metric": "BEM solves/s (served stream, config 5)", "impl": "ours", "unit": "solves/s",
           "requests": n_req, "arrival_rate_per_s": rate, "meshes": sizes, "mesh_probabilities": probs,
           "hbm_budget_GB": 150, "restart": restart, "tol": tol, "quantum": quantum, "rounds": steps,
           "value": n_req / (t_end - arrivals[0]),
           "wall_s": t_end - arrivals[0],
           "latency_ms": {"p50": float(np.percentile(lat, 50) * 1e3), "p99": float(np.percentile(lat, 99) * 1e3),
                          "mean": float(lat.mean() * 1e3), "max": float(lat.max() * 1e3)},
           "converged": int(conv.sum()),
           "per_mesh": {}}
    # where the wall time goes: device phases (CUDA events on the server's
    # stream), host time inside the calls, and the HBM floor of the stream --
    # every DLP matrix written once and read once per GMRES iteration
    # (complex64, 8 n^2 bytes), at the measured copy bandwidth
    peak, _ = measured_peaks()
    floor_bytes = sum(8.0 * sizes[which[r]] ** 2 * (1 + its[r]) for r in range(n_req))
    out["phases_ms"] = {k_: round(v_[0], 3) for k_, v_ in prof.items()}
    out["host_s"] = {k_: round(v_, 4) for k_, v_ in host.items()}
    out["hbm_floor"] = {"bytes": floor_bytes, "seconds": floor_bytes / (peak * 1e9),
                        "solves_per_s": n_req / (floor_bytes / (peak * 1e9))}
    for i, n in enumerate(sizes):
        sel = which == i
        if sel.any():
            out["per_mesh"][str(n)] = {"requests": int(sel.sum()),
                                       "latency_ms_p50": float(np.percentile(lat[sel], 50) * 1e3),
                                       "latency_ms_p99": float(np.percentile(lat[sel], 99) * 1e3),
                                       "iterations_median": float(np.median(its[sel]))}
    # plain single-instance path on a stratified sample (a few requests per mesh)
    plain = {}
    agree = 0.0
    plain_s = 0.0
    for i, n in enumerate(sizes):
        idx = np.flatnonzero(which == i)[:args.plain_sample]
        if len(idx) == 0:
            continue
        t_sum = 0.0
        for r in idx:
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            p1, it1, _ = g.solve_cbie(mesh_list[i], float(ks[r]), qs[r], restart=restart, max_iters=max_iters,
                                      tol=tol, ctx=ctx, check=False)
            torch.cuda.synchronize()
            t_sum += time.perf_counter() - t1
            agree = max(agree, float(np.abs(results[r][1] - p1).max() / np.abs(p1).max()))
        plain[str(n)] = t_sum / len(idx)
        plain_s += t_sum / len(idx) * int((which == i).sum())
    out["plain_seconds_per_request"] = plain
    out["plain_solves_per_s"] = n_req / plain_s
    out["speedup_vs_plain_gpu"] = out["value"] / out["plain_solves_per_s"]
    out["served_vs_plain_max_rel_difference"] = agree
    ctx.close()
    return out


def run_bm(args):
    """Burton-Miller system on the headline mesh (icosphere s=5, 20480
    triangles, Helmholtz, k = 5, coupling -i/k): one step assembles
    A = DLP - I/2 + c HSP and B = SLP + c DLPt + c/2 I (complex64, all four
    kernels per quadrature point, FP64 nearly singular and self terms) into
    device memory.  Metric: system entries per second (A and B counted
    separately).  Also the GMRES solve A p = B q (pulsating sphere), the end to
    end call with host buffers, and the FP64 oracle on a row sample of the
    four operators as the CPU baseline."""
    import torch

    import nihu_gb300 as g
    from nihu_gb300 import meshes
    from nihu_gb300 import _capi as C

    mesh = meshes.icosphere(SUBDIV)
    nodes, elems = mesh
    n = len(elems)
    k = K_WAVE
    c = g.burton_miller_coupling(k)
    ctx = g.Context(0)
    L = g.lib()
    stream = torch.cuda.ExternalStream(ctx.stream)
    dm = g.api.DeviceMesh(ctx, nodes, elems)
    mat_bytes = n * n * 8
    pa_, pb_ = ctypes.c_void_p(), ctypes.c_void_p()
    ctx.check(L.nihu_gb_device_alloc(ctx.handle, mat_bytes, ctypes.byref(pa_)))
    ctx.check(L.nihu_gb_device_alloc(ctx.handle, mat_bytes, ctypes.byref(pb_)))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def step():
        ctx.check(L.nihu_gb_assemble_burton_miller(ctx.handle, dm.handle, C.HELMHOLTZ_3D, k, c.real, c.imag,
                                                   C.REGULAR_FP32, C.C64, pa_, pb_, n, C.DEVICE))

    for _ in range(max(3, args.warmup)):
        step()
    counts = (ctypes.c_int64 * 11)()
    ctx.check(L.nihu_gb_pair_statistics(ctx.handle, dm.handle, dm.handle, counts))
    counts = np.array(list(counts))
    n_regular = int(counts[2:].sum())
    ctx.set_profiling(True)
    ctx.profile_reset()
    clocks = ClockSampler(0)
    clocks.start()
    launches0 = ctx.launch_count
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    torch.cuda.synchronize()
    for s_ in range(args.steps):
        flush.fill_(s_ & 0xFF)  # evict the previous step's lines from L2 (not timed)
        torch.cuda.synchronize()
        ev[s_][0].record(stream)
        step()
        ev[s_][1].record(stream)
    torch.cuda.synchronize()
    launches = ctx.launch_count - launches0
    clk = clocks.stop()
    prof = ctx.profile()
    ctx.set_profiling(False)
    ms = float(np.mean([a.elapsed_time(b) for a, b in ev]))
    entries = 2.0 * n * n
    reg_ms, reg_n = prof.get("assemble_regular_bm", (0.0, 0))
    reg_avg = reg_ms / max(reg_n, 1)
    alg_bytes = 16.0 * n_regular  # one complex64 entry of A and one of B written per regular pair
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / (reg_avg / 1e3) / 1e9
    out = {
        "metric": "Burton-Miller system entries/s", "impl": "ours", "value": entries / (ms / 1e3),
        "unit": "entries/s", "n_gpus": 1, "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32 regular quadrature, nearly singular dynamic parts and static angular sums, fp64 self terms and nearly singular geometry; complex64 storage",
        "data": "synthetic (icosphere mesh generated in-process)",
        "config": {"workload": "icosphere s=5 (%d flat constant triangles), Helmholtz 3D Burton-Miller system "
                               "A = DLP - I/2 + c HSP, B = SLP + c DLPt + c/2 I, c = -i/k, k=5" % n,
                   "n_elements": n, "entries_per_step": int(entries), "operator_entries_per_step": int(4 * n * n),
                   "l2": "256 MB written between timed steps (L2 flushed); outputs 6.7 GB >> 129 MB L2"},
        "gpu_launches": int(launches), "clocks": clk,
        "roofline": {"kernel": "k_regular_bm (assemble_bm.cu)", "bound": "hbm", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "traffic": None,
                     "peak_source": "%s (MEASURED_PEAKS.json hbm_gbs)" % peak_kind,
                     "algorithmic_bytes_per_launch": alg_bytes, "avg_launch_ms": reg_avg,
                     "regular_pairs": n_regular, "near_pairs": int(counts[1]), "self_pairs": int(counts[0])},
        "phases": {kk: {"ms_per_step": v[0] / args.steps, "launches": v[1]} for kk, v in prof.items()},
    }
    # GMRES solve of A p = B q on the assembled matrices
    q = np.ones(n, np.complex128)
    dq, drhs, dp = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    for p_ in (dq, drhs, dp):
        ctx.check(L.nihu_gb_device_alloc(ctx.handle, 16 * n, ctypes.byref(p_)))
    ctx.check(L.nihu_gb_memcpy(ctx.handle, dq, C.DEVICE, q.ctypes.data, C.HOST, 16 * n))
    ctx.check(L.nihu_gb_memcpy(ctx.handle, dp, C.DEVICE, np.zeros(n, np.complex128).ctypes.data, C.HOST, 16 * n))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ctx.check(L.nihu_gb_matvec(ctx.handle, C.C64, pb_, n, n, n, dq, drhs, 1.0, 0.0, 0.0, 0.0, C.DEVICE))
    it, res = ctypes.c_int(0), ctypes.c_double(0.0)
    st = L.nihu_gb_gmres(ctx.handle, C.C64, pa_, n, n, drhs, dp, 50, 1000, 1e-6, ctypes.byref(it), ctypes.byref(res),
                         C.DEVICE)
    torch.cuda.synchronize()
    solve_ms = (time.perf_counter() - t0) * 1e3
    p = np.zeros(n, np.complex128)
    ctx.check(L.nihu_gb_memcpy(ctx.handle, p.ctypes.data, C.HOST, dp, C.DEVICE, 16 * n))
    pa = -1.0 / (1 + 1j * k)
    out["solve"] = {"solver": "GMRES(50), FP32 matvec, FP64 Arnoldi, tol 1e-6", "status": int(st),
                    "iterations": it.value, "rel_residual": res.value, "ms": solve_ms,
                    "pressure_error_vs_analytic": float(np.abs(p - pa).max() / abs(pa))}
    for p_ in (dq, drhs, dp):
        L.nihu_gb_device_free(ctx.handle, p_)
    # end to end: mesh arrays in, both matrices out to pinned host memory
    if not args.no_e2e:
        ha, hb = ctypes.c_void_p(), ctypes.c_void_p()
        ctx.check(L.nihu_gb_host_alloc(ctx.handle, mat_bytes, ctypes.byref(ha)))
        ctx.check(L.nihu_gb_host_alloc(ctx.handle, mat_bytes, ctypes.byref(hb)))
        e2e_steps = max(1, min(args.steps, 3))

        def e2e_step():
            m = ctypes.c_void_p()
            ctx.check(L.nihu_gb_mesh_create(ctx.handle, nodes.ctypes.data, len(nodes), elems.ctypes.data, n,
                                            elems.shape[1], ctypes.byref(m)))
            ctx.check(L.nihu_gb_assemble_burton_miller(ctx.handle, m, C.HELMHOLTZ_3D, k, c.real, c.imag,
                                                       C.REGULAR_FP32, C.C64, ha, hb, n, C.HOST))
            L.nihu_gb_mesh_destroy(m)

        e2e_step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            e2e_step()
        torch.cuda.synchronize()
        e2e_ms = (time.perf_counter() - t0) * 1e3 / e2e_steps
        out["e2e"] = {"value": entries / (e2e_ms / 1e3), "unit": "entries/s",
                      "h2d_bytes_per_step": int(nodes.nbytes + elems.nbytes), "d2h_bytes_per_step": int(2 * mat_bytes),
                      "ms_per_step": e2e_ms, "steps": e2e_steps,
                      "path": "nihu_gb_mesh_create + nihu_gb_assemble_burton_miller(where=HOST, pinned)"}
        L.nihu_gb_host_free(ha)
        L.nihu_gb_host_free(hb)
    L.nihu_gb_device_free(ctx.handle, pa_)
    L.nihu_gb_device_free(ctx.handle, pb_)
    dm.close()
    ctx.close()
    if not args.no_cpu:
        # the FP64 oracle on a row sample of the four operators, all host cores
        from oracle import oracle
        oracle.build()
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        for op in (oracle.SLP, oracle.DLP, oracle.DLPT, oracle.HSP):
            oracle.assemble(mesh, mesh, oracle.HELMHOLTZ, op, k, rows=(0, 1))
        per_row = time.perf_counter() - t0
        rows = int(max(threads, min(8192, args.cpu_seconds * threads / max(per_row, 1e-6))))
        rows = max(threads, (rows // threads) * threads)
        blocks = np.linspace(0, n, threads + 1).astype(int)
        per = rows // threads

        def work(b):
            a = int(blocks[b])
            for op in (oracle.SLP, oracle.DLP, oracle.DLPT, oracle.HSP):
                oracle.assemble(mesh, mesh, oracle.HELMHOLTZ, op, k, rows=(a, min(n, a + per)))

        t0 = time.perf_counter()
        ts = [threading.Thread(target=work, args=(b,)) for b in range(threads)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
        el = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": 2.0 * rows * n / el, "unit": "entries/s", "cores": threads, "kind": "port",
                               "sample": "%d full rows x %d columns x (SLP, DLP, DLPt, HSP), FP64 oracle, %.1f s "
                                         "(system entries: two operators per entry of A and of B)" % (rows, n, el)}
    return out


def box_near_field(centres, h):
    """P2P list of a uniform box partition with leaf size h: every pair of
    elements in the same or a neighbouring leaf box (as an FMM's leaf-level
    near field); rows sorted by box."""
    key = np.floor((centres + 1.0001) / h).astype(np.int64)
    nb = int(key.max()) + 2
    code = (key[:, 0] * nb + key[:, 1]) * nb + key[:, 2]
    order = np.argsort(code, kind="stable")
    codes, starts, counts = np.unique(code[order], return_index=True, return_counts=True)
    where = {int(c): (int(s0), int(cn)) for c, s0, cn in zip(codes, starts, counts)}
    rows, cols = [], []
    offs = [(dx * nb + dy) * nb + dz for dx in (-1, 0, 1) for dy in (-1, 0, 1) for dz in (-1, 0, 1)]
    for c, (s0, cn) in where.items():
        mine = order[s0:s0 + cn]
        for o in offs:
            hit = where.get(c + o)
            if hit is None:
                continue
            other = order[hit[0]:hit[0] + hit[1]]
            rows.append(np.repeat(mine, len(other)))
            cols.append(np.tile(other, len(mine)))
    return np.concatenate(rows).astype(np.int32), np.concatenate(cols).astype(np.int32)


def run_p2p(args):
    """Near field of a box partition (the P2P part of NiHu's Burton-Miller FMM
    solver, nihu/fmm/helmholtz_burton_miller_solver.hpp:170-190) on the
    20480-triangle icosphere, k = 5: leaf boxes of 0.125, every pair of
    elements in the same or a neighbouring box, each evaluated with the full
    singular check into the two near-field operators
    a = DLP + alpha HSP - I/2 and b = SLP + alpha DLPt + alpha/2 I
    (complex64, FP32 regular quadrature).  Metric: near-field entries per
    second (a and b counted separately), pairs and outputs resident in HBM;
    e2e with the pair list uploaded and both value arrays read back per step."""
    import torch

    import nihu_gb300 as g
    from nihu_gb300 import meshes
    from nihu_gb300 import _capi as C

    mesh = meshes.icosphere(SUBDIV)
    nodes, elems = mesh
    n = len(elems)
    k = K_WAVE
    alpha = g.burton_miller_coupling(k)
    cen = meshes.centroids_and_normals(nodes, elems)[0]
    rows, cols = box_near_field(cen, 0.125)
    npairs = len(rows)
    coef = np.array([1.0, 0.0, 1.0, 0.0, alpha.real, alpha.imag, alpha.real, alpha.imag])
    ident = np.array([-0.5, 0.0, alpha.real / 2, alpha.imag / 2])
    ops = C.SLP | C.DLP | C.DLPT | C.HSP
    ctx = g.Context(0)
    L = g.lib()
    stream = torch.cuda.ExternalStream(ctx.stream)
    dm = g.api.DeviceMesh(ctx, nodes, elems)
    ptr = {nm: ctypes.c_void_p() for nm in ("r", "c", "a", "b")}
    for nm, size in (("r", 4 * npairs), ("c", 4 * npairs), ("a", 8 * npairs), ("b", 8 * npairs)):
        ctx.check(L.nihu_gb_device_alloc(ctx.handle, size, ctypes.byref(ptr[nm])))
    ctx.check(L.nihu_gb_memcpy(ctx.handle, ptr["r"], C.DEVICE, rows.ctypes.data, C.HOST, 4 * npairs))
    ctx.check(L.nihu_gb_memcpy(ctx.handle, ptr["c"], C.DEVICE, cols.ctypes.data, C.HOST, 4 * npairs))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def step():
        ctx.check(L.nihu_gb_assemble_pairs(ctx.handle, dm.handle, dm.handle, C.HELMHOLTZ_3D, ops, k,
                                           coef.ctypes.data, ident.ctypes.data, C.REGULAR_FP32, C.C64, npairs,
                                           ptr["r"], ptr["c"], ptr["a"], ptr["b"], C.DEVICE))

    for _ in range(max(3, args.warmup)):
        step()
    ctx.set_profiling(True)
    ctx.profile_reset()
    clocks = ClockSampler(0)
    clocks.start()
    launches0 = ctx.launch_count
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    torch.cuda.synchronize()
    for s_ in range(args.steps):
        flush.fill_(s_ & 0xFF)
        torch.cuda.synchronize()
        ev[s_][0].record(stream)
        step()
        ev[s_][1].record(stream)
    torch.cuda.synchronize()
    launches = ctx.launch_count - launches0
    clk = clocks.stop()
    prof = ctx.profile()
    ctx.set_profiling(False)
    ms = float(np.mean([a_.elapsed_time(b_) for a_, b_ in ev]))
    entries = 2.0 * npairs
    ph_ms, ph_n = prof.get("assemble_pairs", (0.0, 0))
    avg = ph_ms / max(ph_n, 1)
    alg_bytes = 24.0 * npairs  # int32 row + column read, two complex64 values written
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / (avg / 1e3) / 1e9
    n_self = int(np.sum(rows == cols))
    out = {
        "metric": "near-field (P2P) entries/s", "impl": "ours", "value": entries / (ms / 1e3), "unit": "entries/s",
        "n_gpus": 1, "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32 regular quadrature and nearly singular dynamic parts, fp64 self terms and nearly singular "
                 "static parts; complex64 values",
        "data": "synthetic (icosphere mesh generated in-process, uniform leaf boxes)",
        "config": {"workload": "Burton-Miller near field (P2P) of icosphere s=5 (%d triangles), k=5, leaf boxes "
                               "0.125, same and neighbouring boxes: %d pairs" % (n, npairs),
                   "n_elements": n, "pairs": npairs, "self_pairs": n_self, "entries_per_step": int(entries),
                   "l2": "256 MB written between timed steps (L2 flushed)"},
        "gpu_launches": int(launches), "clocks": clk,
        "roofline": {"kernel": "k_pairs_regular + k_pairs_singular (assemble_pairs.cu)", "bound": "hbm",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": None,
                     "peak_source": "%s (MEASURED_PEAKS.json hbm_gbs)" % peak_kind,
                     "algorithmic_bytes_per_launch": alg_bytes, "avg_launch_ms": avg,
                     "note": "compute-bound: near-field pairs take 3-12 regular points per operator or the FP64 "
                             "nearly singular schemes"},
        "phases": {kk: {"ms_per_step": v[0] / args.steps, "launches": v[1]} for kk, v in prof.items()},
    }
    a_dev = np.zeros(npairs, np.complex64)
    ctx.check(L.nihu_gb_memcpy(ctx.handle, a_dev.ctypes.data, C.HOST, ptr["a"], C.DEVICE, 8 * npairs))
    for p_ in ptr.values():
        L.nihu_gb_device_free(ctx.handle, p_)
    if not args.no_e2e:
        ha, hb = np.zeros(npairs, np.complex64), np.zeros(npairs, np.complex64)

        def e2e_step():
            ctx.check(L.nihu_gb_assemble_pairs(ctx.handle, dm.handle, dm.handle, C.HELMHOLTZ_3D, ops, k,
                                               coef.ctypes.data, ident.ctypes.data, C.REGULAR_FP32, C.C64, npairs,
                                               rows.ctypes.data, cols.ctypes.data, ha.ctypes.data, hb.ctypes.data,
                                               C.HOST))

        e2e_step()
        t0 = time.perf_counter()
        e2e_steps = max(1, min(args.steps, 5))
        for _ in range(e2e_steps):
            e2e_step()
        e2e_ms = (time.perf_counter() - t0) * 1e3 / e2e_steps
        out["e2e"] = {"value": entries / (e2e_ms / 1e3), "unit": "entries/s",
                      "h2d_bytes_per_step": int(8 * npairs), "d2h_bytes_per_step": int(16 * npairs),
                      "ms_per_step": e2e_ms, "steps": e2e_steps,
                      "path": "nihu_gb_assemble_pairs(where=HOST): pair list in, both value arrays out",
                      "host_matches_device": bool(np.array_equal(ha, a_dev))}
    dm.close()
    ctx.close()
    if not args.no_cpu:
        from oracle import oracle
        oracle.build()
        threads = os.cpu_count() or 1
        rng = np.random.default_rng(7)
        probe = rng.choice(npairs, size=min(npairs, 1 << 14), replace=False)
        t0 = time.perf_counter()
        for op in (oracle.SLP, oracle.DLP, oracle.DLPT, oracle.HSP):
            oracle.assemble_pairs(mesh, mesh, oracle.HELMHOLTZ, op, k, rows[probe], cols[probe], same_mesh=True,
                                  threads=threads)
        per_pair = (time.perf_counter() - t0) / len(probe)
        size = int(min(npairs, max(len(probe), args.cpu_seconds / max(per_pair, 1e-12))))
        sample = rng.choice(npairs, size=size, replace=False)
        t0 = time.perf_counter()
        for op in (oracle.SLP, oracle.DLP, oracle.DLPT, oracle.HSP):
            oracle.assemble_pairs(mesh, mesh, oracle.HELMHOLTZ, op, k, rows[sample], cols[sample], same_mesh=True,
                                  threads=threads)
        el = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": 2.0 * len(sample) / el, "unit": "entries/s", "cores": threads,
                               "kind": "port",
                               "sample": "%d random pairs of the list x (SLP, DLP, DLPt, HSP), FP64 oracle, %.1f s "
                                         "(near-field entries: two operators per entry of a and of b)"
                                         % (len(sample), el)}
    return out


def run_galerkin(args):
    """Galerkin SLP and DLP on the headline mesh (icosphere s=5, 20480
    triangles, Helmholtz, k = 5, complex64, FP32 regular quadrature: the
    product rules, the singular Galerkin rules of the face, edge and corner
    pairs and the unmatched close pairs) into device memory.  Metric: entries per second
    (SLP and DLP counted separately)."""
    import torch

    import nihu_gb300 as g
    from nihu_gb300 import meshes
    from nihu_gb300 import _capi as C

    mesh = meshes.icosphere(SUBDIV)
    nodes, elems = mesh
    n = len(elems)
    k = K_WAVE
    ctx = g.Context(0)
    L = g.lib()
    stream = torch.cuda.ExternalStream(ctx.stream)
    dm = g.api.DeviceMesh(ctx, nodes, elems)
    mat_bytes = n * n * 8
    ps, pd = ctypes.c_void_p(), ctypes.c_void_p()
    ctx.check(L.nihu_gb_device_alloc(ctx.handle, mat_bytes, ctypes.byref(ps)))
    ctx.check(L.nihu_gb_device_alloc(ctx.handle, mat_bytes, ctypes.byref(pd)))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def step():
        ctx.check(L.nihu_gb_assemble_galerkin(ctx.handle, dm.handle, dm.handle, C.HELMHOLTZ_3D, C.SLP | C.DLP, k, 1.0,
                                              0.0, C.REGULAR_FP32, C.C64, ps, pd, n, 0, C.DEVICE))

    for _ in range(max(3, args.warmup)):
        step()
    counts = (ctypes.c_int64 * 11)()
    ctx.check(L.nihu_gb_pair_statistics(ctx.handle, dm.handle, dm.handle, counts))
    counts = np.array(list(counts))
    n_regular = int(counts[2:].sum())
    ctx.set_profiling(True)
    ctx.profile_reset()
    clocks = ClockSampler(0)
    clocks.start()
    launches0 = ctx.launch_count
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    torch.cuda.synchronize()
    for s_ in range(args.steps):
        flush.fill_(s_ & 0xFF)
        torch.cuda.synchronize()
        ev[s_][0].record(stream)
        step()
        ev[s_][1].record(stream)
    torch.cuda.synchronize()
    launches = ctx.launch_count - launches0
    clk = clocks.stop()
    prof = ctx.profile()
    ctx.set_profiling(False)
    ms = float(np.mean([a_.elapsed_time(b_) for a_, b_ in ev]))
    entries = 2.0 * n * n
    reg_ms, reg_n = prof.get("galerkin_regular", (0.0, 0))
    reg_avg = reg_ms / max(reg_n, 1)
    alg_bytes = 16.0 * n_regular
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / (reg_avg / 1e3) / 1e9
    out = {
        "metric": "Galerkin BEM entries/s", "impl": "ours", "value": entries / (ms / 1e3), "unit": "entries/s",
        "n_gpus": 1, "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32 (regular product rules, singular Galerkin rules, unmatched close pairs); complex64 storage",
        "data": "synthetic (icosphere mesh generated in-process)",
        "config": {"workload": "icosphere s=5 (%d flat constant triangles), Helmholtz 3D SLP+DLP Galerkin, k=5" % n,
                   "n_elements": n, "entries_per_step": int(entries),
                   "l2": "256 MB written between timed steps (L2 flushed); outputs 6.7 GB >> 129 MB L2"},
        "gpu_launches": int(launches), "clocks": clk,
        "roofline": {"kernel": "k_galerkin_regular (assemble_galerkin.cu)", "bound": "hbm", "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": None,
                     "peak_source": "%s (MEASURED_PEAKS.json hbm_gbs)" % peak_kind,
                     "algorithmic_bytes_per_launch": alg_bytes, "avg_launch_ms": reg_avg,
                     "regular_pairs": n_regular, "near_pairs": int(counts[1]), "self_pairs": int(counts[0])},
        "phases": {kk: {"ms_per_step": v[0] / args.steps, "launches": v[1]} for kk, v in prof.items()},
    }
    L.nihu_gb_device_free(ctx.handle, ps)
    L.nihu_gb_device_free(ctx.handle, pd)
    dm.close()
    ctx.close()
    if not args.no_cpu:
        from oracle import oracle
        oracle.build()
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        for op in (oracle.SLP, oracle.DLP):
            oracle.assemble_galerkin(mesh, mesh, oracle.HELMHOLTZ, op, k, rows=(0, 1))
        per_row = time.perf_counter() - t0
        rows = int(max(threads, min(4096, args.cpu_seconds * threads / max(per_row, 1e-6))))
        rows = max(threads, (rows // threads) * threads)
        t0 = time.perf_counter()
        for op in (oracle.SLP, oracle.DLP):
            oracle.assemble_galerkin(mesh, mesh, oracle.HELMHOLTZ, op, k, rows=(0, rows), threads=threads)
        el = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": 2.0 * rows * n / el, "unit": "entries/s", "cores": threads, "kind": "port",
                               "sample": "%d full rows x %d columns x (SLP, DLP), FP64 Galerkin oracle, %.1f s"
                                         % (rows, n, el)}
    return out


def run_profile(args):
    """Per-phase device times of the collocational assembly, and a small
    target for ncu.  Assembles the Helmholtz (--laplace: Laplace) SLP and DLP
    matrices of an icosphere (--subdiv) or a quad cylinder (--cylinder), or
    with --bm the two Burton-Miller system matrices, --reps times.  With
    --budget-mb the context's HBM budget forces host output in column panels,
    so that every kernel launch covers one panel of the full-size problem and
    the device holds only about the budget: small enough for an ncu capture
    of single launches.  Without it both matrices are assembled into device
    memory in one launch each.  --sweep N solves N wave numbers uniform in
    [0.1, 10] on one icosphere and --sweep-config4 the 256-instance sweep
    (nihu_gb_solve_sweep_batched, run --reps times; the first call builds the
    near-pair lists).  Returns the per-phase times of the last repetition."""
    import nihu_gb300 as g
    from nihu_gb300 import _capi as C
    from nihu_gb300 import api, meshes

    if args.sweep or args.sweep_config4:
        rng = np.random.default_rng(2026)
        if args.sweep_config4:
            mesh_list = [api.create_mesh(*meshes.icosphere(s_)) for s_ in (2, 3, 4)]
            ks = rng.uniform(0.1, 10.0, 256)
            mesh_of = np.arange(256) % 3
        else:
            mesh_list = [api.create_mesh(*meshes.icosphere(args.subdiv))]
            ks = rng.uniform(0.1, 10.0, args.sweep)
            mesh_of = np.zeros(args.sweep, np.int32)
        ctx = api.Context(0)
        ctx.set_profiling(True)
        for _ in range(max(1, args.reps)):
            ctx.profile_reset()
            P, it, rel, conv = api.solve_sweep_batched(mesh_list, ks, mesh_of, restart=50, max_iters=1000, tol=1e-6,
                                                       ctx=ctx, check=False)
        prof = ctx.profile()
        ctx.close()
        return {"config": "profile (sweep)", "instances": len(ks), "meshes": [m.num_elements for m in mesh_list],
                "iterations_total": int(np.sum(it)), "converged": int(np.sum(conv)),
                "phases_ms": {k: round(v[0], 4) for k, v in prof.items()},
                "launches": {k: v[1] for k, v in prof.items()}}

    if args.gemm:
        return profile_gemm(args)

    if args.cylinder:
        nt = args.cylinder
        nodes, elems = meshes.cylinder(nt, int(1.25 * nt), max(2, round(15 * nt / 160)))
    else:
        nodes, elems = meshes.icosphere(args.subdiv)
    ctx = api.Context(0, hbm_budget_bytes=args.budget_mb << 20)
    L = g.lib()
    dm = api.DeviceMesh(ctx, nodes, elems)
    n = dm.n
    fam = C.LAPLACE_3D if args.laplace else C.HELMHOLTZ_3D
    prec = C.REGULAR_FP64 if args.fp64 else C.REGULAR_FP32
    if args.budget_mb:
        hs = np.zeros((n, n), np.complex64, order="F")
        hd = np.zeros((n, n), np.complex64, order="F")
        ps, pd, where = hs.ctypes.data, hd.ctypes.data, C.HOST
    else:
        ps, pd = ctypes.c_void_p(), ctypes.c_void_p()
        ctx.check(L.nihu_gb_device_alloc(ctx.handle, 8 * n * n, ctypes.byref(ps)))
        ctx.check(L.nihu_gb_device_alloc(ctx.handle, 8 * n * n, ctypes.byref(pd)))
        where = C.DEVICE
    ctx.set_profiling(True)
    for _ in range(max(1, args.reps)):
        ctx.profile_reset()
        if args.bm:
            c = api.burton_miller_coupling(args.k) if fam == C.HELMHOLTZ_3D else 1.0 + 0.0j
            ctx.check(L.nihu_gb_assemble_burton_miller(ctx.handle, dm.handle, fam, args.k, c.real, c.imag, prec,
                                                       C.C64, pd, ps, n, where))
        else:
            ctx.check(L.nihu_gb_assemble(ctx.handle, dm.handle, dm.handle, fam, C.SLP | C.DLP, args.k, 1.0, 0.0, prec,
                                         C.C64, ps, pd, n, 0, where))
    prof = ctx.profile()
    if not args.budget_mb:
        L.nihu_gb_device_free(ctx.handle, ps)
        L.nihu_gb_device_free(ctx.handle, pd)
    dm.close()
    ctx.close()
    return {"config": "profile (assembly)", "n_elements": n, "where": "host panels" if args.budget_mb else "device",
            "phases_ms": {k: round(v[0], 4) for k, v in prof.items()},
            "launches": {k: v[1] for k, v in prof.items()}}


def profile_gemm(args):
    """--config profile --gemm M N NRHS: nihu_gb_gemm on device buffers,
    --reps times, timed with CUDA events on the context's stream."""
    import nihu_gb300 as g
    from nihu_gb300 import _capi as C
    from nihu_gb300 import api

    m, n, nrhs = args.gemm
    ctx = api.Context(0)
    L = g.lib()
    rng = np.random.default_rng(7)
    bufs = []

    def dev(host):
        p = ctypes.c_void_p()
        ctx.check(L.nihu_gb_device_alloc(ctx.handle, host.nbytes, ctypes.byref(p)))
        ctx.check(L.nihu_gb_memcpy(ctx.handle, p, C.DEVICE, host.ctypes.data, C.HOST, host.nbytes))
        bufs.append(p)
        return p

    A = dev((rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n))).astype(np.complex64, order="F"))
    X = dev(np.asfortranarray(rng.standard_normal((n, nrhs)) + 1j * rng.standard_normal((n, nrhs))))
    Y = dev(np.zeros((m, nrhs), np.complex128, order="F"))
    times = []
    for _ in range(max(1, args.reps)):
        t0 = time.perf_counter()
        ctx.check(L.nihu_gb_gemm(ctx.handle, args.gemm_mode, A, m, n, m, X, n, nrhs, Y, m, 1.0, 0.0, 0.0, 0.0,
                                 C.DEVICE))
        times.append((time.perf_counter() - t0) * 1e3)
    for p in bufs:
        L.nihu_gb_device_free(ctx.handle, p)
    ctx.close()
    return {"config": "profile (gemm)", "m": m, "n": n, "nrhs": nrhs, "mode": args.gemm_mode,
            "host_ms": [round(t, 4) for t in times], "a_bytes": 8 * m * n}


def other_configs(args):
    """Short runs of the other configurations, summarised for the headline
    line: the plain small solve, the multi-RHS solve, the batched sweep and
    the served stream (300 requests), each with its comparison against the
    plain single-instance GPU path where it has one.  A failing leg is
    reported as an error string and does not stop the others."""
    import copy

    def sub(**kw):
        a = copy.copy(args)
        for k_, v_ in kw.items():
            setattr(a, k_, v_)
        return a

    def keep(d, keys):
        return {k_: d[k_] for k_ in keys if k_ in d}

    res = {}
    legs = (
        ("small", lambda: run_small(sub(steps=5, warmup=3)),
         ("metric", "value", "unit", "higher_is_better", "n_elements", "k", "dtype", "e2e", "phases_ms",
          "pressure_error_vs_analytic", "pressure_gpu_vs_cpu_oracle", "cpu_baseline")),
        ("multirhs", lambda: run_multirhs(sub(steps=1, warmup=1)),
         ("metric", "value", "unit", "n_elements", "nrhs", "k", "assembly_ms", "rhs_gemm_ms", "solve_ms",
          "solve_status", "outer_iterations", "inner_iterations", "max_rel_residual", "err_per_rhs", "gemm",
          "solves_per_s")),
        ("sweep", lambda: run_sweep(sub(steps=3, warmup=2)),
         ("metric", "value", "unit", "instances", "meshes", "batched_seconds", "plain_solves_per_s",
          "speedup_vs_plain_gpu", "batched_vs_plain_max_rel_difference", "phases_ms", "plan_tuning")),
        ("serve", lambda: run_serve(sub(requests=300, plain_sample=3)),
         ("metric", "value", "unit", "requests", "arrival_rate_per_s", "latency_ms", "converged",
          "plain_solves_per_s", "speedup_vs_plain_gpu", "served_vs_plain_max_rel_difference", "rounds",
          "phases_ms", "host_s", "hbm_floor", "plain_seconds_per_request", "per_mesh")),
    )
    for name, fn, keys in legs:
        t0 = time.perf_counter()
        try:
            d = fn()
            res[name] = keep(d, keys)
        except Exception as e:  # reported, not fatal for the headline
            res[name] = {"error": "%s: %s" % (type(e).__name__, e)}
        res[name]["wall_s"] = round(time.perf_counter() - t0, 2)
    return res


def main():
    args = parse()
    runs = {"multirhs": run_multirhs, "small": run_small, "sweep": run_sweep, "serve": run_serve, "bm": run_bm,
            "p2p": run_p2p, "galerkin": run_galerkin, "profile": run_profile}
    if args.config in runs:
        out = runs[args.config](args)
        if out is not None:
            print(json.dumps(out), flush=True)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
