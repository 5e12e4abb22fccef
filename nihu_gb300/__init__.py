"""GB300-native dense collocation BEM (NiHu's collocational SLP/DLP assembly
and the GMRES matvec) on hand-written sm_103a CUDA kernels behind a C ABI.

The C ABI is declared in ``include/nihu_gb300.h``; ``include/nihu_gb300/nihu.hpp``
is the C++ front end shaped like NiHu's integral-operator API; this package
is the Python front end with the same shape.
"""
from ._capi import (C64, C128, DEVICE, DLP, DLPT, HSP, GEMM_BF16X3, GEMM_BF16X6, GEMM_BF16X9, GEMM_FP32, GEMM_TF32, HELMHOLTZ_3D, HOST, LAPLACE_3D, QUAD_1, REGULAR_FP32, REGULAR_FP64, SLP,
                    TRIA_1, InvalidArgumentError, NihuError, NotConvergedError, OutOfRangeError, lib)
from .api import (Context, DeviceMesh, Mesh, Server, SweepPlan, assemble_burton_miller, assemble_pairs, burton_miller_coupling,
                  constant_view, create_integral_operator, create_mesh, default_context,
                  dirac, gemm, gmres, helmholtz_3d_DLP_kernel, helmholtz_3d_DLPt_kernel, helmholtz_3d_HSP_kernel,
                  helmholtz_3d_SLP_kernel, identity_integral_operator, laplace_3d_DLP_kernel, laplace_3d_DLPt_kernel,
                  laplace_3d_HSP_kernel, laplace_3d_SLP_kernel, lu_solve, matvec, near_pairs, pair_statistics, solve_burton_miller, solve_cbie,
                  solve_batched, solve_multi, solve_sweep, solve_sweep_batched)
from . import meshes

__all__ = [
    "C64", "C128", "DEVICE", "DLP", "GEMM_BF16X3", "GEMM_BF16X6", "GEMM_BF16X9", "GEMM_FP32", "GEMM_TF32", "gemm", "solve_batched", "solve_multi", "solve_sweep", "solve_sweep_batched", "HELMHOLTZ_3D", "HOST", "LAPLACE_3D", "QUAD_1", "REGULAR_FP32", "REGULAR_FP64",
    "SLP", "TRIA_1", "InvalidArgumentError", "NihuError", "NotConvergedError", "OutOfRangeError", "lib", "Context", "Server", "SweepPlan",
    "DeviceMesh", "Mesh", "constant_view", "create_integral_operator", "create_mesh", "default_context", "dirac",
    "gmres", "helmholtz_3d_DLP_kernel", "helmholtz_3d_SLP_kernel", "identity_integral_operator",
    "laplace_3d_DLP_kernel", "laplace_3d_SLP_kernel", "lu_solve", "matvec", "near_pairs", "pair_statistics", "solve_cbie", "meshes",
    "DLPT", "HSP", "helmholtz_3d_DLPt_kernel", "helmholtz_3d_HSP_kernel", "laplace_3d_DLPt_kernel", "laplace_3d_HSP_kernel",
    "assemble_burton_miller", "assemble_pairs", "burton_miller_coupling", "solve_burton_miller",
]
