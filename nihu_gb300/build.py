"""Build the in-tree CUDA library ``nihu_gb300/libnihu_gb300.so`` for sm_103a.

Every translation unit is compiled by its own nvcc process (in parallel) and
linked into one shared library with the CUDA runtime linked statically.  The
output stays inside the package directory so the loader finds it in-tree.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libnihu_gb300.so")
SOURCES = ["mesh.cu", "classify.cu", "assemble_regular.cu", "assemble_singular.cu", "linalg.cu", "capi.cu",
           "noalloc.cu", "multi.cu", "gemm_tc.cu", "solve_persistent.cu", "assemble_bm.cu",
           "assemble_pairs.cu", "assemble_galerkin.cu"]
HEADERS = ["common.cuh", "geom.cuh", "classify.cuh", "kernels.h", "linalg.h", "quad_rules.h", "solve_persistent.h",
           "planar.cuh", "singular_schemes.cuh", "bm_schemes.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]


def nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if not os.path.exists(LIB):
        force = True  # objects from another machine or toolchain are never reused
    common = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(HERE, "..", "include", "nihu_gb300.h")]
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        if force or _stale(o, [s] + common):
            jobs.append([nvcc(), *ARCH, *FLAGS, "-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
        for cmd, r in zip(jobs, results):
            if verbose or r.returncode:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode:
                raise RuntimeError("nvcc failed: " + " ".join(cmd))
    objs = [os.path.join(BUILD, s.replace(".cu", ".o")) for s in SOURCES]
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        cuda_lib = os.path.join(os.path.dirname(os.path.dirname(nvcc())), "lib64")
        cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", *objs, "-o", tmp, "-lcublas",
               "-Xlinker", "-rpath", "-Xlinker", cuda_lib]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
