"""The C++ front end (include/nihu_gb300/nihu.hpp): NiHu-shaped user code
compiled with g++ against the C ABI, run on the GPU, checked against the
FP64 oracle and the analytic pulsating sphere."""
import os
import subprocess

import numpy as np
import pytest

from nihu_gb300 import meshes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_shim(tmp):
    exe = os.path.join(tmp, "test_shim")
    lib_dir = os.path.join(ROOT, "nihu_gb300")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", os.path.join(ROOT, "tests", "cpp", "test_shim.cpp"),
                           "-I", os.path.join(ROOT, "include"), "-L", lib_dir, "-lnihu_gb300",
                           "-Wl,-rpath," + lib_dir, "-o", exe])
    return exe


def test_shim_compiles(tmp_path):
    """The header is plain C++17 and links against the library (no GPU needed)."""
    build_shim(str(tmp_path))


@pytest.mark.gpu
def test_shim_acoustic_bem_sequence(tmp_path, oracle):
    exe = build_shim(str(tmp_path))
    nodes, elems = meshes.icosphere(2)
    mesh_bin = tmp_path / "mesh.bin"
    with open(mesh_bin, "wb") as f:
        f.write(np.array([len(nodes), len(elems)], np.int64).tobytes())
        f.write(np.ascontiguousarray(nodes, np.float64).tobytes())
        f.write(np.ascontiguousarray(elems, np.int32).tobytes())
    out_bin = tmp_path / "out.bin"
    k = 1.0
    r = subprocess.run([exe, str(mesh_bin), str(k), str(out_bin)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    n = len(elems)
    raw = np.fromfile(out_bin, dtype=np.complex128)
    Ls = raw[:n * n].reshape(n, n, order="F")
    Ms = raw[n * n:2 * n * n].reshape(n, n, order="F")
    p = raw[2 * n * n:2 * n * n + n]
    o = 2 * n * n + n
    Gs = raw[o:o + n * n].reshape(n, n, order="F")
    Hs = raw[o + n * n:o + 2 * n * n].reshape(n, n, order="F")
    p_bm = raw[o + 2 * n * n:o + 2 * n * n + n]
    o2 = o + 2 * n * n + n
    Lg = raw[o2:o2 + n * n].reshape(n, n, order="F")
    Mg = raw[o2 + n * n:o2 + 2 * n * n].reshape(n, n, order="F")
    Ig = raw[o2 + 2 * n * n:o2 + 3 * n * n].reshape(n, n, order="F")
    p_g = raw[o2 + 3 * n * n:]
    mesh = (nodes, elems)
    L = oracle.assemble(mesh, mesh, oracle.HELMHOLTZ, oracle.SLP, k, threads=8)
    M = oracle.assemble(mesh, mesh, oracle.HELMHOLTZ, oracle.DLP, k, threads=8) - 0.5 * np.eye(n)
    assert np.abs(Ls - L).max() / np.abs(L).max() < 1e-5
    assert np.abs(Ms - M).max() / np.abs(M).max() < 1e-5
    p_ref = np.linalg.solve(M, L @ np.ones(n))
    assert np.abs(p - p_ref).max() / np.abs(p_ref).max() < 1e-4
    # the Burton-Miller branch of the same application
    c = -1j / k
    D = oracle.assemble(mesh, mesh, oracle.HELMHOLTZ, oracle.HSP, k, threads=8)
    Ht = oracle.assemble(mesh, mesh, oracle.HELMHOLTZ, oracle.DLPT, k, threads=8)
    G_ref = L + c * Ht + 0.5 * c * np.eye(n)
    H_ref = M + c * D
    assert np.abs(Gs - G_ref).max() / np.abs(G_ref).max() < 1e-5
    assert np.abs(Hs - H_ref).max() / np.abs(H_ref).max() < 1e-5
    p_bm_ref = np.linalg.solve(H_ref, G_ref @ np.ones(n))
    assert np.abs(p_bm - p_bm_ref).max() / np.abs(p_bm_ref).max() < 1e-4
    # the Galerkin formalism of the reference's own pulsating-sphere test
    Lgr = oracle.assemble_galerkin(mesh, mesh, oracle.HELMHOLTZ, oracle.SLP, k, threads=8)
    Mgr = oracle.assemble_galerkin(mesh, mesh, oracle.HELMHOLTZ, oracle.DLP, k, threads=8)
    c = nodes[elems[:, 1:4]]
    area = 0.5 * np.linalg.norm(np.cross(c[:, 1] - c[:, 0], c[:, 2] - c[:, 0]), axis=1)
    assert np.allclose(np.diag(Ig).real, area, rtol=1e-12) and np.count_nonzero(Ig) == n
    assert np.abs(Lg - Lgr).max() / np.abs(Lgr).max() < 1e-5
    assert np.abs(Mg - Mgr).max() / np.abs(Mgr).max() < 1e-5
    p_gr = np.linalg.solve(Mgr - 0.5 * np.diag(area), Lgr @ np.ones(n))
    assert np.abs(p_g - p_gr).max() / np.abs(p_gr).max() < 1e-4
