"""ctypes binding of the C ABI in ``include/nihu_gb300.h``.

The shared library is built in-tree by ``nihu_gb300.build``; loading fails
loudly when it is missing -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libnihu_gb300.so")

OK = 0
STATUS_NAMES = {
    0: "OK", 1: "INVALID_ARGUMENT", 2: "OUT_OF_RANGE", 3: "RUNTIME", 4: "CUDA",
    5: "OUT_OF_MEMORY", 6: "NOT_CONVERGED", 7: "NO_DEVICE",
}
TRIA_1, QUAD_1 = 32303, 32404
HELMHOLTZ_3D, LAPLACE_3D = 0, 1
SLP, DLP = 1, 2
DLPT, HSP = 4, 8  # Burton-Miller operators
C64, C128 = 0, 1
REGULAR_FP32, REGULAR_FP64 = 0, 1
GEMM_FP32, GEMM_TF32, GEMM_BF16X9, GEMM_BF16X3, GEMM_BF16X6 = 0, 1, 2, 3, 4
HOST, DEVICE = 0, 1
NOALLOC_PARTIAL_ELEMS = 1 << 20  # NIHU_GB_NOALLOC_PARTIAL_ELEMS

# every symbol include/nihu_gb300.h declares, with (restype, argtypes)
_vp, _i, _i64, _d, _sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double, ctypes.c_size_t
_ip, _dp = ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)
SIGNATURES = {
    "nihu_gb_ctx_create": (_i, [_i, _vp, _sz, ctypes.POINTER(_vp)]),
    "nihu_gb_ctx_destroy": (None, [_vp]),
    "nihu_gb_last_error": (ctypes.c_char_p, [_vp]),
    "nihu_gb_ctx_stream": (_vp, [_vp]),
    "nihu_gb_ctx_device_bytes": (_sz, [_vp]),
    "nihu_gb_ctx_launch_count": (_i64, [_vp]),
    "nihu_gb_ctx_set_profiling": (_i, [_vp, _i]),
    "nihu_gb_ctx_profile": (_i, [_vp, _i, ctypes.POINTER(ctypes.c_char_p), _dp, ctypes.POINTER(ctypes.c_int64)]),
    "nihu_gb_ctx_profile_reset": (None, [_vp]),
    "nihu_gb_host_alloc": (_i, [_vp, _sz, ctypes.POINTER(_vp)]),
    "nihu_gb_host_free": (None, [_vp]),
    "nihu_gb_device_alloc": (_i, [_vp, _sz, ctypes.POINTER(_vp)]),
    "nihu_gb_device_free": (None, [_vp, _vp]),
    "nihu_gb_memcpy": (_i, [_vp, _vp, _i, _vp, _i, _sz]),
    "nihu_gb_mesh_create": (_i, [_vp, _vp, _i64, _vp, _i64, _i64, ctypes.POINTER(_vp)]),
    "nihu_gb_mesh_destroy": (None, [_vp]),
    "nihu_gb_mesh_num_elements": (_i64, [_vp]),
    "nihu_gb_assemble": (_i, [_vp, _vp, _vp, _i, _i, _d, _d, _d, _i, _i, _vp, _vp, _i64, _i, _i]),
    "nihu_gb_assemble_c": (_i, [_vp, _vp, _vp, _i, _i, _d, _d, _d, _d, _i, _i, _vp, _vp, _i64, _i, _i]),
    "nihu_gb_add_identity": (_i, [_vp, _vp, _d, _d, _i, _vp, _i64, _i]),
    "nihu_gb_pair_statistics": (_i, [_vp, _vp, _vp, ctypes.POINTER(ctypes.c_int64)]),
    "nihu_gb_near_pairs": (_i, [_vp, _vp, _vp, ctypes.POINTER(ctypes.c_int64), _vp, _vp]),
    "nihu_gb_matvec": (_i, [_vp, _i, _vp, _i64, _i64, _i64, _vp, _vp, _d, _d, _d, _d, _i]),
    "nihu_gb_matvec_noalloc": (_i, [_i, _vp, _i64, _i64, _i64, _vp, _vp, _d, _d, _d, _d, _vp]),
    "nihu_gb_gmres": (_i, [_vp, _i, _vp, _i64, _i64, _vp, _vp, _i, _i, _d, _ip, _dp, _i]),
    "nihu_gb_gemm": (_i, [_vp, _i, _vp, _i64, _i64, _i64, _vp, _i64, _i64, _vp, _i64, _d, _d, _d, _d, _i]),
    "nihu_gb_solve_multi": (_i, [_vp, _vp, _i64, _i64, _vp, _vp, _i64, _i, _i, _i, _i, _d, _d, _ip, _ip, _dp, _i]),
    "nihu_gb_assemble_sweep": (_i, [_vp, _vp, _vp, _i, _i, _dp, _i, _i, _i, _vp, _vp, _i64, _i64]),
    "nihu_gb_solve_sweep": (_i, [_vp, _vp, _i, _dp, _i, _i, _vp, _i, _vp, _i, _i, _d, _ip, _ip, _dp]),
    "nihu_gb_solve_batched": (_i, [_vp, _i, _vp, _vp, _vp, _vp, _vp, _i, _i, _d, _vp, _vp, _vp]),
    "nihu_gb_solve_sweep_batched": (_i, [_vp, _i, _vp, _i, _i, _vp, _vp, _i, _vp, _vp, _i, _i, _d, _vp, _vp, _vp]),
    "nihu_gb_lu_solve": (_i, [_vp, _vp, _i64, _i64, _vp, _vp, _i]),
    "nihu_gb_sweep_plan_create": (_i, [_vp, _i, _vp, _i, _i, _vp, _d, _i, _i, _i, _d, ctypes.POINTER(_vp)]),
    "nihu_gb_sweep_plan_run": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "nihu_gb_sweep_plan_host_buffers": (_i, [_vp, ctypes.POINTER(_vp), ctypes.POINTER(_vp)]),
    "nihu_gb_sweep_plan_tuning": (_i, [_vp, _vp, _vp, _vp]),
    "nihu_gb_sweep_plan_destroy": (None, [_vp]),
    "nihu_gb_server_create": (_i, [_vp, _i, _vp, _i, _i, _sz, _i, _i, _i, _d, _i, ctypes.POINTER(_vp)]),
    "nihu_gb_server_destroy": (None, [_vp]),
    "nihu_gb_server_reserve": (_i, [_vp, _sz]),
    "nihu_gb_server_submit": (_i, [_vp, _i, _d, _vp, ctypes.POINTER(ctypes.c_int64)]),
    "nihu_gb_server_step": (_i, [_vp, _ip, _ip, _ip]),
    "nihu_gb_server_take": (_i, [_vp, ctypes.POINTER(ctypes.c_int64), _vp, _i64, _ip, _dp, _ip]),
    "nihu_gb_solve_cbie": (_i, [_vp, _vp, _i, _d, _i, _i, _vp, _vp, _i, _i, _i, _d, _ip, _dp]),
    "nihu_gb_solve_cbie_c": (_i, [_vp, _vp, _i, _d, _d, _i, _i, _vp, _vp, _i, _i, _i, _d, _ip, _dp]),
    "nihu_gb_assemble_galerkin": (_i, [_vp, _vp, _vp, _i, _i, _d, _d, _d, _i, _i, _vp, _vp, _i64, _i, _i]),
    "nihu_gb_assemble_galerkin_c": (_i, [_vp, _vp, _vp, _i, _i, _d, _d, _d, _d, _i, _i, _vp, _vp, _i64, _i, _i]),
    "nihu_gb_add_mass": (_i, [_vp, _vp, _d, _d, _i, _vp, _i64, _i]),
    "nihu_gb_assemble_bm": (_i, [_vp, _vp, _vp, _i, _i, _d, _d, _d, _i, _i, _vp, _vp, _i64, _i, _i]),
    "nihu_gb_assemble_burton_miller": (_i, [_vp, _vp, _i, _d, _d, _d, _i, _i, _vp, _vp, _i64, _i]),
    "nihu_gb_assemble_pairs": (_i, [_vp, _vp, _vp, _i, _i, _d, _vp, _vp, _i, _i, _i64, _vp, _vp, _vp, _vp, _i]),
    "nihu_gb_solve_burton_miller": (_i, [_vp, _vp, _i, _d, _d, _d, _i, _i, _vp, _vp, _i, _i, _i, _d, _ip, _dp]),
    "nihu_gb_assemble_bm_c": (_i, [_vp, _vp, _vp, _i, _i, _d, _d, _d, _d, _i, _i, _vp, _vp, _i64, _i, _i]),
    "nihu_gb_assemble_burton_miller_c": (_i, [_vp, _vp, _i, _d, _d, _d, _d, _i, _i, _vp, _vp, _i64, _i]),
    "nihu_gb_assemble_pairs_c": (_i, [_vp, _vp, _vp, _i, _i, _d, _d, _vp, _vp, _i, _i, _i64, _vp, _vp, _vp, _vp, _i]),
    "nihu_gb_solve_burton_miller_c": (_i, [_vp, _vp, _i, _d, _d, _d, _d, _i, _i, _vp, _vp, _i, _i, _i, _d, _ip, _dp]),
}

_lib = None
_lock = threading.Lock()


class NihuError(RuntimeError):
    """A failed library call; ``status`` holds the C status code."""

    def __init__(self, status, message):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), message))
        self.status = status


class InvalidArgumentError(NihuError, ValueError):
    """Bad argument (the reference raises std::invalid_argument / logic_error)."""


class OutOfRangeError(NihuError, IndexError):
    """The reference's std::out_of_range (e.g. quadrature degree above 14)."""


class NotConvergedError(NihuError):
    """An iterative solve stopped at its iteration limit."""


_ERRORS = {1: InvalidArgumentError, 2: OutOfRangeError, 6: NotConvergedError}


def lib():
    """The loaded CUDA library (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError("libnihu_gb300.so is not built; run nihu_gb300.build.build() "
                                  "(the GPU path has no CPU fallback)")
            L = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def check(ctx, status):
    if status != OK:
        msg = lib().nihu_gb_last_error(ctx).decode() if ctx else ""
        raise _ERRORS.get(status, NihuError)(status, msg)
