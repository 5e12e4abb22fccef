"""ctypes access to the FP64 CPU oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module; the product library never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
SOURCES = [os.path.join(HERE, "nihu_oracle.c")]
HELMHOLTZ, LAPLACE = 0, 1
SLP, DLP, DLPT, HSP = 1, 2, 4, 8


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (no external dependencies)."""
    newest = max(os.path.getmtime(s) for s in SOURCES + [os.path.join(HERE, "..", "nihu_gb300", "csrc", "quad_rules.h")])
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < newest:
        tmp = LIB_PATH + ".tmp%d" % os.getpid()
        subprocess.check_call(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", *SOURCES, "-o", tmp, "-lm"])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None
_lock = threading.Lock()


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            dp, ip = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
            c_int, c_double, c_long = ctypes.c_int, ctypes.c_double, ctypes.c_long
            L.oracle_assemble.argtypes = [dp, c_int, ip, c_int, c_int, dp, c_int, ip, c_int, c_int,
                                          c_int, c_int, c_int, c_double, c_double, c_double, c_double,
                                          c_int, c_int, c_int, c_int, dp, c_long, c_int]
            L.oracle_assemble.restype = c_int
            L.oracle_assemble_pairs.argtypes = [dp, c_int, ip, c_int, c_int, dp, c_int, ip, c_int, c_int,
                                                c_int, c_int, c_int, c_double, c_double, ctypes.c_long, ip, ip, dp]
            L.oracle_assemble_pairs.restype = c_int
            L.oracle_assemble_galerkin.argtypes = [dp, c_int, ip, c_int, c_int, dp, c_int, ip, c_int, c_int, c_int,
                                                   c_int, c_int, c_double, c_double, c_double, c_double, c_int, c_int,
                                                   c_int,
                                                   c_int, dp, ctypes.c_long, c_int]
            L.oracle_assemble_galerkin.restype = c_int
            L.oracle_galerkin_rule.argtypes = [c_int, dp]
            L.oracle_galerkin_rule.restype = c_int
            L.oracle_galerkin_quad_rule.argtypes = [c_int, dp]
            L.oracle_galerkin_quad_rule.restype = c_int
            L.oracle_classify.argtypes = [dp, c_int, ip, c_int, c_int, dp, c_int, ip, c_int, c_int,
                                          c_int, c_int, c_int, ip]
            L.oracle_classify.restype = c_int
            L.oracle_elem_integral.argtypes = [dp, c_int, dp, c_int, c_int, c_double, c_double, c_int, c_int, dp]
            L.oracle_elem_integral.restype = c_int
            L.oracle_elem_integral_nx.argtypes = [dp, c_int, dp, dp, c_int, c_int, c_double, c_double, c_int, c_int,
                                                  dp]
            L.oracle_elem_integral_nx.restype = c_int
            L.oracle_degree.argtypes = [dp, c_int, ip, c_int, c_int, dp, c_int, ip, c_int, c_int,
                                        c_int, c_int, c_int, c_int, ip]
            L.oracle_degree.restype = c_int
            L.oracle_elem_geometry.argtypes = [dp, c_int, dp]
            L.oracle_last_error.restype = ctypes.c_char_p
            _lib = L
    return _lib


def _ptr(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


def _mesh_args(nodes, elems):
    nodes = np.ascontiguousarray(nodes, dtype=np.float64)
    elems = np.ascontiguousarray(elems, dtype=np.int32)
    return nodes, elems, [_ptr(nodes, ctypes.c_double), len(nodes), _ptr(elems, ctypes.c_int), len(elems), elems.shape[1]]


def assemble(test_mesh, trial_mesh, family, op, k, same_mesh=None, rows=None, alpha=1.0, threads=1, cols=None):
    """Dense operator block (rows x cols, default all) as complex128 in
    column-major order (Fortran array)."""
    tn, te, targs = _mesh_args(*test_mesh)
    rn, re_, rargs = _mesh_args(*trial_mesh)
    if same_mesh is None:
        same_mesh = test_mesh is trial_mesh
    r0, r1 = (0, len(te)) if rows is None else rows
    c0, c1 = (0, len(re_)) if cols is None else cols
    m, n = r1 - r0, c1 - c0
    out = np.zeros((m, n), dtype=np.complex128, order="F")
    alpha = complex(alpha)
    L = lib()

    errors = []

    def work(a, b):
        buf = np.zeros((b - a, n), dtype=np.complex128, order="F")
        ptr = ctypes.cast(buf.ctypes.data, ctypes.POINTER(ctypes.c_double))
        ok = L.oracle_assemble(*targs, *rargs, int(same_mesh), family, op, complex(k).real, complex(k).imag, alpha.real, alpha.imag,
                               a, b, c0, c1, ptr, b - a, 0)
        if not ok:
            errors.append(RuntimeError(L.oracle_last_error().decode()))
            return
        out[a - r0:b - r0] = buf

    if threads <= 1 or m < 2:
        work(r0, r1)
    else:
        bounds = np.linspace(r0, r1, threads + 1).astype(int)
        ts = [threading.Thread(target=work, args=(int(bounds[i]), int(bounds[i + 1]))) for i in range(threads)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
    if errors:
        raise errors[0]
    return out


def assemble_galerkin(test_mesh, trial_mesh, family, op, k, same_mesh=None, rows=None, alpha=1.0, threads=1):
    """Dense Galerkin operator block (SLP or DLP, constant elements; singular
    quadrature for matched triangles of one mesh) as complex128, Fortran order."""
    tn, te, targs = _mesh_args(*test_mesh)
    rn, re_, rargs = _mesh_args(*trial_mesh)
    if same_mesh is None:
        same_mesh = test_mesh is trial_mesh
    r0, r1 = (0, len(te)) if rows is None else rows
    m, n = r1 - r0, len(re_)
    out = np.zeros((m, n), dtype=np.complex128, order="F")
    alpha = complex(alpha)
    L = lib()
    errors = []

    def work(a, b):
        buf = np.zeros((b - a, n), dtype=np.complex128, order="F")
        ok = L.oracle_assemble_galerkin(*targs, *rargs, int(same_mesh), family, op, complex(k).real, complex(k).imag, alpha.real, alpha.imag,
                                        a, b, 0, n, ctypes.cast(buf.ctypes.data, ctypes.POINTER(ctypes.c_double)),
                                        b - a, 0)
        if not ok:
            errors.append(RuntimeError(L.oracle_last_error().decode()))
            return
        out[a - r0:b - r0] = buf

    if threads <= 1 or m < 2:
        work(r0, r1)
    else:
        bounds = np.linspace(r0, r1, threads + 1).astype(int)
        ts = [threading.Thread(target=work, args=(int(bounds[i]), int(bounds[i + 1]))) for i in range(threads)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
    if errors:
        raise errors[0]
    return out


def galerkin_rule(match, quad=False):
    """The singular Galerkin rule of a triangle (or quad) pair for match 2
    (face), 1 (edge), 0 (corner): array of (test xi, eta, trial xi, eta, w)."""
    L = lib()
    fn = L.oracle_galerkin_quad_rule if quad else L.oracle_galerkin_rule
    n = fn(match, None)
    out = np.zeros((n, 5))
    fn(match, ctypes.cast(out.ctypes.data, ctypes.POINTER(ctypes.c_double)))
    return out


def assemble_pairs(test_mesh, trial_mesh, family, op, k, rows, cols, same_mesh=None, threads=1):
    """Entries of the pair list (rows[p], cols[p]) with the full singular
    check (complex128, one per pair): the FMM near-field evaluation."""
    tn, te, targs = _mesh_args(*test_mesh)
    rn, re_, rargs = _mesh_args(*trial_mesh)
    if same_mesh is None:
        same_mesh = test_mesh is trial_mesh
    rows = np.ascontiguousarray(rows, dtype=np.int32)
    cols = np.ascontiguousarray(cols, dtype=np.int32)
    n = len(rows)
    out = np.zeros(n, dtype=np.complex128)
    L = lib()
    errors = []

    def work(a, b):
        buf = np.zeros(b - a, dtype=np.complex128)
        ok = L.oracle_assemble_pairs(*targs, *rargs, int(same_mesh), family, op, complex(k).real, complex(k).imag, b - a,
                                     _ptr(rows[a:b], ctypes.c_int), _ptr(cols[a:b], ctypes.c_int),
                                     ctypes.cast(buf.ctypes.data, ctypes.POINTER(ctypes.c_double)))
        if not ok:
            errors.append(RuntimeError(L.oracle_last_error().decode()))
            return
        out[a:b] = buf

    if threads <= 1 or n < 2:
        work(0, n)
    else:
        bounds = np.linspace(0, n, threads + 1).astype(int)
        ts = [threading.Thread(target=work, args=(int(bounds[i]), int(bounds[i + 1]))) for i in range(threads)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
    if errors:
        raise errors[0]
    return out


def classify(test_mesh, trial_mesh, same_mesh=None, rows=None):
    tn, te, targs = _mesh_args(*test_mesh)
    rn, re_, rargs = _mesh_args(*trial_mesh)
    if same_mesh is None:
        same_mesh = test_mesh is trial_mesh
    r0, r1 = (0, len(te)) if rows is None else rows
    out = np.zeros((r1 - r0, len(re_)), dtype=np.int32)
    if not lib().oracle_classify(*targs, *rargs, int(same_mesh), r0, r1, _ptr(out, ctypes.c_int)):
        raise RuntimeError(lib().oracle_last_error().decode())
    return out


def elem_integral(coords, x0, family, op, k, kind, degree=0, nx=None):
    """kind: 0 regular(degree), 1 nearly singular dispatch, 2 self, 3 planar near scheme.
    nx: unit normal at the collocation point (DLPT and HSP)."""
    coords = np.ascontiguousarray(coords, dtype=np.float64)
    x0 = np.ascontiguousarray(x0, dtype=np.float64)
    out = np.zeros(2)
    if nx is None:
        ok = lib().oracle_elem_integral(_ptr(coords, ctypes.c_double), coords.shape[0], _ptr(x0, ctypes.c_double),
                                        family, op, complex(k).real, complex(k).imag, kind, degree, _ptr(out, ctypes.c_double))
    else:
        nx = np.ascontiguousarray(nx, dtype=np.float64)
        ok = lib().oracle_elem_integral_nx(_ptr(coords, ctypes.c_double), coords.shape[0],
                                           _ptr(x0, ctypes.c_double), _ptr(nx, ctypes.c_double), family, op,
                                           complex(k).real, complex(k).imag, kind, degree, _ptr(out, ctypes.c_double))
    if not ok:
        raise RuntimeError("element integral failed")
    return complex(out[0], out[1])


def degree(test_mesh, trial_mesh, op, same_mesh=None, rows=None):
    """Quadrature degree of operator op per pair: -1 self, -2 nearly singular."""
    tn, te, targs = _mesh_args(*test_mesh)
    rn, re_, rargs = _mesh_args(*trial_mesh)
    if same_mesh is None:
        same_mesh = test_mesh is trial_mesh
    r0, r1 = (0, len(te)) if rows is None else rows
    out = np.zeros((r1 - r0, len(re_)), dtype=np.int32)
    if not lib().oracle_degree(*targs, *rargs, int(same_mesh), op, r0, r1, _ptr(out, ctypes.c_int)):
        raise RuntimeError(lib().oracle_last_error().decode())
    return out
