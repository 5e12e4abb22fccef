"""NiHu-shaped Python front end of the GPU library.

Mirrors the reference's user API for the collocation path
(nihu/core/weighted_residual.hpp, integral_operator.hpp, function_space.hpp,
mesh.hpp) so code reads like NiHu:

    mesh = create_mesh(nodes, elements)
    sp = constant_view(mesh)
    Lop = create_integral_operator(helmholtz_3d_SLP_kernel(k))
    Ls = np.zeros((n, n), complex, order="F")
    Ls << dirac(sp) * Lop[sp]          # accumulates, like NiHu's operator<<

Every evaluation runs on the GPU through the C ABI; results land in the
caller's matrix with "+=" semantics (nihu/util/matrix_block.hpp).
"""
from __future__ import annotations

import ctypes
import weakref

import numpy as np

from . import _capi as C

_default_ctx = None


class Context:
    """One GPU, one stream (nihu_gb_ctx)."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0, stream=None):
        L = C.lib()
        h = ctypes.c_void_p()
        st = L.nihu_gb_ctx_create(device, stream, hbm_budget_bytes, ctypes.byref(h))
        if st != C.OK:
            raise C._ERRORS.get(st, C.NihuError)(st, "nihu_gb_ctx_create failed (device %d)" % device)
        self.handle = h
        self._meshes = weakref.WeakValueDictionary()

    def close(self):
        if self.handle:
            for dm in list(self._meshes.values()):
                dm.close()
            C.lib().nihu_gb_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return C.lib().nihu_gb_ctx_stream(self.handle) or 0

    @property
    def device_bytes(self) -> int:
        return C.lib().nihu_gb_ctx_device_bytes(self.handle)

    @property
    def launch_count(self) -> int:
        return C.lib().nihu_gb_ctx_launch_count(self.handle)

    def check(self, status):
        C.check(self.handle, status)

    def set_profiling(self, enable: bool = True):
        self.check(C.lib().nihu_gb_ctx_set_profiling(self.handle, int(enable)))

    def profile(self) -> dict:
        """{phase: (total device ms, launches)} accumulated while profiling."""
        out, i = {}, 0
        name, ms, n = ctypes.c_char_p(), ctypes.c_double(), ctypes.c_int64()
        while C.lib().nihu_gb_ctx_profile(self.handle, i, ctypes.byref(name), ctypes.byref(ms), ctypes.byref(n)) == 0:
            out[name.value.decode()] = (ms.value, n.value)
            i += 1
        return out

    def profile_reset(self):
        C.lib().nihu_gb_ctx_profile_reset(self.handle)


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None or _default_ctx.handle is None:
        _default_ctx = Context(0)
    return _default_ctx


class DeviceMesh:
    """A mesh uploaded to a context (nihu_gb_mesh)."""

    def __init__(self, ctx: Context, nodes: np.ndarray, elems: np.ndarray):
        nodes = np.ascontiguousarray(nodes, dtype=np.float64)
        elems = np.ascontiguousarray(elems, dtype=np.int32)
        if nodes.ndim != 2 or nodes.shape[1] != 3 or elems.ndim != 2:
            raise ValueError("nodes must be (n, 3) and elements (m, cols)")
        h = ctypes.c_void_p()
        ctx.check(C.lib().nihu_gb_mesh_create(ctx.handle, nodes.ctypes.data, len(nodes), elems.ctypes.data,
                                              len(elems), elems.shape[1], ctypes.byref(h)))
        self.ctx = ctx
        self.handle = h
        self.n = len(elems)

    def close(self):
        if self.handle:
            C.lib().nihu_gb_mesh_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            if self.ctx.handle:
                self.close()
        except Exception:
            pass


class Mesh:
    """create_mesh(nodes, elements) (nihu/core/mesh.hpp:175-193,285-290).

    ``elements`` rows are [type id, node indices...]; ids run in row order."""

    def __init__(self, nodes, elements):
        self.nodes = np.ascontiguousarray(nodes, dtype=np.float64)
        el = np.asarray(elements)
        if el.shape[1] < 5:
            pad = np.full((el.shape[0], 5 - el.shape[1]), -1, dtype=np.int32)
            el = np.hstack([el.astype(np.int32), pad])
        self.elements = np.ascontiguousarray(el, dtype=np.int32)
        self._dev = {}

    @property
    def num_elements(self) -> int:
        return len(self.elements)

    def areas(self, ctx: Context | None = None) -> np.ndarray:
        """Element areas with the one-point rule of the Galerkin identity
        (nihu/core/single_integral.hpp:97-140): |e1 x e2| / 2 on triangles,
        4 |x_xi x x_eta| at the centre on quads (nihu_gb_add_mass's weights)."""
        el = self.elements
        c = self.nodes[np.where(el[:, 1:5] >= 0, el[:, 1:5], el[:, 1:2])]
        quad = el[:, 0] == C.QUAD_1
        t1 = np.where(quad[:, None], (c[:, 1] + c[:, 2] - c[:, 0] - c[:, 3]) / 4, c[:, 1] - c[:, 0])
        t2 = np.where(quad[:, None], (c[:, 2] + c[:, 3] - c[:, 0] - c[:, 1]) / 4, c[:, 2] - c[:, 0])
        return np.linalg.norm(np.cross(t1, t2), axis=1) * np.where(quad, 4.0, 0.5)

    def device(self, ctx: Context) -> DeviceMesh:
        key = id(ctx)
        dm = self._dev.get(key)
        if dm is None or dm.handle is None:
            dm = DeviceMesh(ctx, self.nodes, self.elements)
            self._dev[key] = dm
            ctx._meshes[id(dm)] = dm
        return dm


def create_mesh(nodes, elements) -> Mesh:
    return Mesh(nodes, elements)


class FunctionSpace:
    """constant_view(mesh): DOF = element id (nihu/core/function_space.hpp:263)."""

    def __init__(self, mesh: Mesh):
        self.mesh = mesh

    def get_num_dofs(self) -> int:
        return self.mesh.num_elements

    def __mul__(self, transform):
        return _make_wr(self, transform)


class DiracSpace:
    """dirac(space): collocation at element centres (nihu/core/function_space.hpp:355)."""

    def __init__(self, space: FunctionSpace):
        self.space = space
        self.mesh = space.mesh

    def get_num_dofs(self) -> int:
        return self.space.get_num_dofs()

    def __mul__(self, transform):
        return _make_wr(self, transform)


def constant_view(mesh: Mesh) -> FunctionSpace:
    return FunctionSpace(mesh)


def dirac(space: FunctionSpace) -> DiracSpace:
    return DiracSpace(space)


class Kernel:
    """A kernel with its wave number: real, or complex for a lossy medium (the
    reference's kernels take a complex WaveNumber type,
    nihu/library/helmholtz_kernel.hpp:42-54)."""

    def __init__(self, family: int, op: int, k: complex = 0.0, name: str = ""):
        kc = complex(k)
        self.family, self.op, self.name = family, op, name
        self.k = kc.real if kc.imag == 0 else kc

    def get_wave_number(self):
        return self.k


def helmholtz_3d_SLP_kernel(k: float) -> Kernel:
    return Kernel(C.HELMHOLTZ_3D, C.SLP, k, "helmholtz_3d_SLP")


def helmholtz_3d_DLP_kernel(k: float) -> Kernel:
    return Kernel(C.HELMHOLTZ_3D, C.DLP, k, "helmholtz_3d_DLP")


def laplace_3d_SLP_kernel() -> Kernel:
    return Kernel(C.LAPLACE_3D, C.SLP, 0.0, "laplace_3d_SLP")


def laplace_3d_DLP_kernel() -> Kernel:
    return Kernel(C.LAPLACE_3D, C.DLP, 0.0, "laplace_3d_DLP")


def helmholtz_3d_DLPt_kernel(k: float) -> Kernel:
    """dG/dn_x (nihu/library/helmholtz_kernel.hpp:326-328); constant triangle trial elements."""
    return Kernel(C.HELMHOLTZ_3D, C.DLPT, k, "helmholtz_3d_DLPt")


def helmholtz_3d_HSP_kernel(k: float) -> Kernel:
    """d2G/dn_x dn_y (nihu/library/helmholtz_kernel.hpp:332-334); constant triangle trial elements."""
    return Kernel(C.HELMHOLTZ_3D, C.HSP, k, "helmholtz_3d_HSP")


def laplace_3d_DLPt_kernel() -> Kernel:
    return Kernel(C.LAPLACE_3D, C.DLPT, 0.0, "laplace_3d_DLPt")


def laplace_3d_HSP_kernel() -> Kernel:
    return Kernel(C.LAPLACE_3D, C.HSP, 0.0, "laplace_3d_HSP")


class IntegralOperator:
    """create_integral_operator(kernel), with scalar scaling (nihu/core/integral_operator.hpp:131-194,324-329)."""

    def __init__(self, kernel: Kernel, scale: complex = 1.0):
        self.kernel, self.scale = kernel, complex(scale)

    def __rmul__(self, alpha):
        return IntegralOperator(self.kernel, self.scale * complex(alpha))

    __mul__ = __rmul__

    def __getitem__(self, trial_space):
        return IntegralTransform(self, trial_space)


class IdentityOperator:
    """identity_integral_operator() (nihu/core/integral_operator.hpp:215-238)."""

    def __init__(self, scale: complex = 1.0):
        self.scale = complex(scale)

    def __rmul__(self, alpha):
        return IdentityOperator(self.scale * complex(alpha))

    __mul__ = __rmul__

    def __getitem__(self, trial_space):
        return IntegralTransform(self, trial_space)


def create_integral_operator(kernel: Kernel) -> IntegralOperator:
    return IntegralOperator(kernel)


def identity_integral_operator() -> IdentityOperator:
    return IdentityOperator()


class IntegralTransform:
    """op[trial_space]; sums of transforms are evaluated term by term."""

    def __init__(self, op, trial_space, terms=None):
        self.terms = terms if terms is not None else [(op, trial_space)]

    def __add__(self, other):
        return IntegralTransform(None, None, self.terms + other.terms)


def _make_wr(test, transform):
    if not isinstance(transform, IntegralTransform):
        return NotImplemented
    return WeightedResidual(test, transform)


def _space_mesh(space):
    return space.mesh


class WeightedResidual:
    """test_space * Op[trial_space] (nihu/core/weighted_residual.hpp:176-186).

    ``result << wr`` adds the operator matrix into ``result`` in place
    (nihu/core/weighted_residual.hpp:197-206).  Options (``precision``:
    "fp32" regular quadrature, the default, or "fp64") can be given with
    ``wr.eval_into(result, precision=...)``."""

    __array_ufunc__ = None  # make numpy defer ``ndarray << wr`` to __rlshift__

    def __init__(self, test, transform: IntegralTransform):
        self.test, self.transform = test, transform

    def __rlshift__(self, result):
        return self.eval_into(result)

    def eval_into(self, result: np.ndarray, precision: str = "fp32", ctx: Context | None = None):
        ctx = ctx or default_context()
        if not isinstance(result, np.ndarray) or result.ndim != 2:
            raise TypeError("result must be a 2D numpy array (a dynamic matrix, nihu/core/result_matrix.hpp)")
        test_mesh = _space_mesh(self.test)
        # a function-space test space is the Galerkin formalism, dirac(...) collocation
        # (nihu/core/formalism.hpp)
        galerkin = not isinstance(self.test, DiracSpace)
        for op, trial_space in self.transform.terms:
            trial_mesh = _space_mesh(trial_space)
            m, n = test_mesh.num_elements, trial_mesh.num_elements
            if result.shape != (m, n):
                raise ValueError("result is %s, operator is %dx%d" % (result.shape, m, n))
            if isinstance(op, IdentityOperator):
                if test_mesh is not trial_mesh:
                    continue  # the identity only couples coinciding elements of one mesh
                idx = np.arange(m)
                result[idx, idx] += op.scale * (test_mesh.areas(ctx) if galerkin else 1.0)
                continue
            _assemble_into(ctx, result, test_mesh, trial_mesh, op.kernel.family, op.kernel.op, op.kernel.k,
                           op.scale, precision, galerkin)
        return result


def _assemble_into(ctx, result, test_mesh, trial_mesh, family, op, k, alpha, precision, galerkin=False):
    L = C.lib()
    if result.dtype == np.complex64:
        dtype, target = C.C64, result
    elif result.dtype == np.complex128:
        dtype, target = C.C128, result
    elif result.dtype in (np.float32, np.float64) and family == C.LAPLACE_3D and complex(alpha).imag == 0:
        dtype = C.C64 if result.dtype == np.float32 else C.C128
        target = None
    else:
        raise TypeError("result dtype %s not supported for this kernel" % result.dtype)
    tdm, rdm = test_mesh.device(ctx), trial_mesh.device(ctx)
    same = test_mesh is trial_mesh
    rdm_handle = tdm.handle if same else rdm.handle
    prec = C.REGULAR_FP64 if precision == "fp64" else C.REGULAR_FP32
    if target is not None and target.flags.f_contiguous:
        buf, accumulate = target, 1
    else:
        cdt = np.complex64 if dtype == C.C64 else np.complex128
        buf, accumulate = np.zeros(result.shape, dtype=cdt, order="F"), 0
    if op in (C.SLP, C.DLP):
        out_s = buf.ctypes.data if op == C.SLP else None
        out_d = buf.ctypes.data if op == C.DLP else None
        kc = complex(k)
        if kc.imag != 0:
            fn = L.nihu_gb_assemble_galerkin_c if galerkin else L.nihu_gb_assemble_c
            ctx.check(fn(ctx.handle, tdm.handle, rdm_handle, family, op, kc.real, kc.imag, alpha.real, alpha.imag,
                         prec, dtype, out_s, out_d, max(result.shape[0], 1), accumulate, C.HOST))
        else:
            fn = L.nihu_gb_assemble_galerkin if galerkin else L.nihu_gb_assemble
            ctx.check(fn(ctx.handle, tdm.handle, rdm_handle, family, op, kc.real, alpha.real, alpha.imag, prec,
                         dtype, out_s, out_d, max(result.shape[0], 1), accumulate, C.HOST))
    elif galerkin:
        raise NotImplementedError("Galerkin formalism: SLP and DLP kernels only")
    else:
        kc = complex(k)
        out_t = buf.ctypes.data if op == C.DLPT else None
        out_h = buf.ctypes.data if op == C.HSP else None
        ctx.check(L.nihu_gb_assemble_bm_c(ctx.handle, tdm.handle, rdm_handle, family, op, kc.real, kc.imag,
                                          alpha.real, alpha.imag, prec, dtype, out_t, out_h,
                                          max(result.shape[0], 1), accumulate, C.HOST))
    if buf is not result:
        if target is None:
            result += buf.real.astype(result.dtype)
        else:
            result += buf


# -------------------------------------------------------------- linear algebra

def _c128(v):
    return np.ascontiguousarray(v, dtype=np.complex128)


def matvec(A: np.ndarray, x: np.ndarray, ctx: Context | None = None) -> np.ndarray:
    """y = A x on the GPU (A complex64 or complex128, Fortran order)."""
    ctx = ctx or default_context()
    A = np.asfortranarray(A)
    dtype = C.C64 if A.dtype == np.complex64 else C.C128
    if A.dtype not in (np.complex64, np.complex128):
        raise TypeError("A must be complex64 or complex128")
    x = _c128(x)
    y = np.zeros(A.shape[0], dtype=np.complex128)
    ctx.check(C.lib().nihu_gb_matvec(ctx.handle, dtype, A.ctypes.data, A.shape[0], A.shape[1], max(A.shape[0], 1),
                                     x.ctypes.data, y.ctypes.data, 1.0, 0.0, 0.0, 0.0, C.HOST))
    return y


def gmres(A: np.ndarray, b: np.ndarray, x0=None, restart: int = 50, max_iters: int = 1000, tol: float = 1e-6,
          ctx: Context | None = None):
    """Restarted GMRES on the GPU; returns (x, iterations, relative residual estimate)."""
    ctx = ctx or default_context()
    A = np.asfortranarray(A)
    if A.dtype not in (np.complex64, np.complex128):
        raise TypeError("A must be complex64 or complex128")
    dtype = C.C64 if A.dtype == np.complex64 else C.C128
    b = _c128(b)
    x = _c128(np.zeros_like(b) if x0 is None else x0).copy()
    it, res = ctypes.c_int(0), ctypes.c_double(0.0)
    ctx.check(C.lib().nihu_gb_gmres(ctx.handle, dtype, A.ctypes.data, A.shape[0], max(A.shape[0], 1), b.ctypes.data,
                                    x.ctypes.data, restart, max_iters, tol, ctypes.byref(it), ctypes.byref(res),
                                    C.HOST))
    return x, it.value, res.value


def lu_solve(A: np.ndarray, b: np.ndarray, ctx: Context | None = None) -> np.ndarray:
    """x = A^{-1} b by FP64 LU with partial pivoting on the GPU (A is not modified)."""
    ctx = ctx or default_context()
    A = np.asfortranarray(A, dtype=np.complex128)
    b = _c128(b)
    x = np.zeros_like(b)
    ctx.check(C.lib().nihu_gb_lu_solve(ctx.handle, A.ctypes.data, A.shape[0], max(A.shape[0], 1), b.ctypes.data,
                                       x.ctypes.data, C.HOST))
    return x


def gemm(A: np.ndarray, X: np.ndarray, mode: int = C.GEMM_FP32, ctx: Context | None = None) -> np.ndarray:
    """Y = A X on the GPU for many right-hand sides (A complex64, X complex128 n x nrhs)."""
    ctx = ctx or default_context()
    A = np.asfortranarray(A, dtype=np.complex64)
    X = np.asfortranarray(X, dtype=np.complex128)
    m, n = A.shape
    nrhs = X.shape[1]
    Y = np.zeros((m, nrhs), np.complex128, order="F")
    ctx.check(C.lib().nihu_gb_gemm(ctx.handle, mode, A.ctypes.data, m, n, max(m, 1), X.ctypes.data, max(n, 1), nrhs,
                                   Y.ctypes.data, max(m, 1), 1.0, 0.0, 0.0, 0.0, C.HOST))
    return Y


def solve_multi(A: np.ndarray, B: np.ndarray, inner_mode: int = C.GEMM_TF32, restart: int = 30, max_outer: int = 20,
                tol: float = 1e-6, inner_tol: float = 1e-3, residual_mode: int = C.GEMM_FP32,
                ctx: Context | None = None):
    """A X = B for many right-hand sides by mixed-precision iterative refinement
    (tensor-core GMRES inner solves, FP64-accumulated residuals).
    Returns (X, outer iterations, inner iterations, relative residual per column)."""
    ctx = ctx or default_context()
    A = np.asfortranarray(A, dtype=np.complex64)
    B = np.asfortranarray(B, dtype=np.complex128)
    n, nrhs = B.shape
    X = np.zeros_like(B, order="F")
    oi, ii = ctypes.c_int(0), ctypes.c_int(0)
    res = np.zeros(nrhs)
    ctx.check(C.lib().nihu_gb_solve_multi(ctx.handle, A.ctypes.data, n, max(n, 1), B.ctypes.data, X.ctypes.data, nrhs,
                                          inner_mode, residual_mode, restart, max_outer, tol, inner_tol,
                                          ctypes.byref(oi),
                                          ctypes.byref(ii), res.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                          C.HOST))
    return X, oi.value, ii.value, res


def solve_cbie(mesh: Mesh, k: float, q, family: int = C.HELMHOLTZ_3D, dtype: int = C.C64, solver: str = "gmres",
               precision: str = "fp32", restart: int = 50, max_iters: int = 1000, tol: float = 1e-6,
               ctx: Context | None = None, check: bool = True):
    """Exterior CBIE (DLP - I/2) p = SLP q on the GPU; returns (p, iterations, residual)."""
    ctx = ctx or default_context()
    q = _c128(q)
    p = np.zeros_like(q)
    it, res = ctypes.c_int(0), ctypes.c_double(0.0)
    dm = mesh.device(ctx)
    kc = complex(k)  # a complex k is a lossy medium
    st = C.lib().nihu_gb_solve_cbie_c(ctx.handle, dm.handle, family, kc.real, kc.imag,
                                      C.REGULAR_FP64 if precision == "fp64" else C.REGULAR_FP32, dtype,
                                      q.ctypes.data, p.ctypes.data, 0 if solver == "gmres" else 1, restart,
                                      max_iters, tol, ctypes.byref(it), ctypes.byref(res))
    if st != C.OK and (check or st != 6):
        ctx.check(st)
    return p, it.value, res.value


def assemble_pairs(test: Mesh, trial: Mesh, rows, cols, ops: int, k: complex = 0.0, family: int = C.HELMHOLTZ_3D,
                   coef=None, ident=None, dtype: int = C.C128, precision: str = "fp32", ctx: Context | None = None):
    """Entries of the element pairs (rows[p], cols[p]) with the full singular
    check, as the FMM near field (nihu/fmm/p2p_precompute.hpp):
    a[p] = c_DLP DLP + c_HSP HSP (+ ident[0] on self pairs),
    b[p] = c_SLP SLP + c_DLPt DLPt (+ ident[1]).  coef: dict or 4-sequence of
    complex scales for (SLP, DLP, DLPt, HSP) (default 1).  Returns (a, b), None
    for an output the operators do not touch."""
    ctx = ctx or default_context()
    rows = np.ascontiguousarray(rows, dtype=np.int32)
    cols = np.ascontiguousarray(cols, dtype=np.int32)
    if rows.shape != cols.shape or rows.ndim != 1:
        raise ValueError("rows and cols must be 1D arrays of one length")
    if isinstance(coef, dict):
        coef = [coef.get(op, 1.0) for op in (C.SLP, C.DLP, C.DLPT, C.HSP)]
    c = None if coef is None else np.array([[complex(v).real, complex(v).imag] for v in coef], np.float64).ravel()
    idn = None if ident is None else np.array([[complex(v).real, complex(v).imag] for v in ident], np.float64).ravel()
    n = len(rows)
    cdt = np.complex64 if dtype == C.C64 else np.complex128
    need_a = bool(ops & (C.DLP | C.HSP))
    need_b = bool(ops & (C.SLP | C.DLPT))
    a = np.zeros(n, cdt) if need_a else None
    b = np.zeros(n, cdt) if need_b else None
    tdm = test.device(ctx)
    rdm = tdm if trial is test else trial.device(ctx)
    kc = complex(k)
    ctx.check(C.lib().nihu_gb_assemble_pairs_c(
        ctx.handle, tdm.handle, rdm.handle, family, ops, kc.real, kc.imag, None if c is None else c.ctypes.data,
        None if idn is None else idn.ctypes.data, C.REGULAR_FP64 if precision == "fp64" else C.REGULAR_FP32, dtype,
        n, rows.ctypes.data, cols.ctypes.data, None if a is None else a.ctypes.data,
        None if b is None else b.ctypes.data, C.HOST))
    return a, b


def burton_miller_coupling(k: complex) -> complex:
    """The reference application's coupling constant -i/k
    (nihu/applications/helmholtz/helmholtz_3d_coll.cpp:44), k real or complex."""
    return -1j / complex(k)


def assemble_burton_miller(mesh: Mesh, k: complex, coupling=None, family: int = C.HELMHOLTZ_3D, dtype: int = C.C64,
                           precision: str = "fp32", ctx: Context | None = None):
    """The Burton-Miller system matrices A = DLP - I/2 + c HSP and B = SLP + c DLPt + c/2 I
    (c = -i/k by default), assembled on the GPU in one pass; returns (A, B)."""
    ctx = ctx or default_context()
    c = burton_miller_coupling(k) if coupling is None else complex(coupling)
    n = mesh.num_elements
    cdt = np.complex64 if dtype == C.C64 else np.complex128
    A = np.zeros((n, n), cdt, order="F")
    B = np.zeros((n, n), cdt, order="F")
    dm = mesh.device(ctx)
    kc = complex(k)
    ctx.check(C.lib().nihu_gb_assemble_burton_miller_c(ctx.handle, dm.handle, family, kc.real, kc.imag, c.real,
                                                       c.imag, C.REGULAR_FP64 if precision == "fp64" else C.REGULAR_FP32,
                                                       dtype, A.ctypes.data, B.ctypes.data, max(n, 1), C.HOST))
    return A, B


def solve_burton_miller(mesh: Mesh, k: complex, q, coupling=None, family: int = C.HELMHOLTZ_3D, dtype: int = C.C64,
                        solver: str = "gmres", precision: str = "fp32", restart: int = 50, max_iters: int = 1000,
                        tol: float = 1e-6, ctx: Context | None = None, check: bool = True):
    """Burton-Miller exterior solve A p = B q on the GPU (c = -i/k by default);
    returns (p, iterations, residual)."""
    ctx = ctx or default_context()
    c = burton_miller_coupling(k) if coupling is None else complex(coupling)
    q = _c128(q)
    p = np.zeros_like(q)
    it, res = ctypes.c_int(0), ctypes.c_double(0.0)
    dm = mesh.device(ctx)
    kc = complex(k)
    st = C.lib().nihu_gb_solve_burton_miller_c(ctx.handle, dm.handle, family, kc.real, kc.imag, c.real, c.imag,
                                               C.REGULAR_FP64 if precision == "fp64" else C.REGULAR_FP32, dtype,
                                             q.ctypes.data, p.ctypes.data, 0 if solver == "gmres" else 1, restart,
                                             max_iters, tol, ctypes.byref(it), ctypes.byref(res))
    if st != C.OK and (check or st != 6):
        ctx.check(st)
    return p, it.value, res.value


def solve_sweep(mesh: Mesh, ks, q, family: int = C.HELMHOLTZ_3D, precision: str = "fp32", restart: int = 30,
                max_cycles: int = 50, tol: float = 1e-6, ctx: Context | None = None, check: bool = True):
    """(DLP - I/2) p_f = SLP q_f for every wave number ks[f] on one mesh, batched on
    the GPU (frequency-batched assembly, one persistent GMRES launch).  q: (n,)
    broadcast or (n, nk).  Returns (P (n x nk), largest restart-cycle count,
    largest iteration count, relative residual estimates).  With check=False an iteration
    limit is not an error: the residuals tell which columns converged."""
    ctx = ctx or default_context()
    ks = np.ascontiguousarray(ks, dtype=np.float64)
    nk = len(ks)
    q = np.asarray(q, dtype=np.complex128)
    q_cols = 1 if q.ndim == 1 else q.shape[1]
    q = np.asfortranarray(q.reshape(q.shape[0], q_cols))
    n = mesh.num_elements
    P = np.zeros((n, nk), np.complex128, order="F")
    cyc, it = ctypes.c_int(0), ctypes.c_int(0)
    res = np.zeros(nk)
    dm = mesh.device(ctx)
    st = C.lib().nihu_gb_solve_sweep(ctx.handle, dm.handle, family, ks.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                     nk, C.REGULAR_FP64 if precision == "fp64" else C.REGULAR_FP32, q.ctypes.data,
                                     q_cols, P.ctypes.data, restart, max_cycles, tol, ctypes.byref(cyc),
                                     ctypes.byref(it), res.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    if st != C.OK and (check or st != 6):
        ctx.check(st)
    return P, cyc.value, it.value, res


def solve_batched(As, bs, restart: int = 50, max_iters: int = 1000, tol: float = 1e-6, ctx: Context | None = None,
                  check: bool = True):
    """Solve the independent systems As[f] x = bs[f] (any sizes) with GMRES in one
    persistent GPU launch (nihu_gb_solve_batched).  As: complex64 matrices;
    bs: vectors.  Returns (xs, iterations, relative residual estimates,
    converged flags).  With check=False an iteration limit is not an error."""
    ctx = ctx or default_context()
    L = C.lib()
    count = len(As)
    if len(bs) != count:
        raise ValueError("one right-hand side per matrix")
    mats = [np.asfortranarray(A, dtype=np.complex64) for A in As]
    rhs = [_c128(b) for b in bs]
    for A, b in zip(mats, rhs):
        if A.ndim != 2 or A.shape[0] != A.shape[1] or b.shape != (A.shape[0],):
            raise ValueError("square matrices with matching right-hand sides expected")
    ptrs = []

    def dev(nbytes):
        p = ctypes.c_void_p()
        ctx.check(L.nihu_gb_device_alloc(ctx.handle, max(nbytes, 16), ctypes.byref(p)))
        ptrs.append(p)
        return p

    try:
        dA, db, dx = [], [], []
        for A, b in zip(mats, rhs):
            pa, pb, px = dev(A.nbytes), dev(b.nbytes), dev(b.nbytes)
            ctx.check(L.nihu_gb_memcpy(ctx.handle, pa, C.DEVICE, A.ctypes.data, C.HOST, A.nbytes))
            ctx.check(L.nihu_gb_memcpy(ctx.handle, pb, C.DEVICE, b.ctypes.data, C.HOST, b.nbytes))
            dA.append(pa.value)
            db.append(pb.value)
            dx.append(px.value)
        arr = lambda v: (ctypes.c_void_p * max(count, 1))(*v)
        n = np.array([A.shape[0] for A in mats] or [0], dtype=np.int64)
        lda = np.maximum(n, 1)
        it = np.zeros(max(count, 1), np.int32)
        rel = np.zeros(max(count, 1))
        conv = np.zeros(max(count, 1), np.int32)
        st = L.nihu_gb_solve_batched(ctx.handle, count, arr(dA), n.ctypes.data, lda.ctypes.data, arr(db), arr(dx),
                                     restart, max_iters, tol, it.ctypes.data, rel.ctypes.data, conv.ctypes.data)
        if st != C.OK and (check or st != 6):
            ctx.check(st)
        xs = []
        for f, b in enumerate(rhs):
            x = np.zeros_like(b)
            ctx.check(L.nihu_gb_memcpy(ctx.handle, x.ctypes.data, C.HOST, dx[f], C.DEVICE, x.nbytes))
            xs.append(x)
        return xs, it[:count], rel[:count], conv[:count].astype(bool)
    finally:
        for p in ptrs:
            L.nihu_gb_device_free(ctx.handle, p)


def solve_sweep_batched(meshes, ks, mesh_of, q=None, family: int = C.HELMHOLTZ_3D, precision: str = "fp32",
                        restart: int = 50, max_iters: int = 1000, tol: float = 1e-6, ctx: Context | None = None,
                        check: bool = True):
    """(DLP - I/2) p_f = SLP q_f for instance f on meshes[mesh_of[f]] at wave number
    ks[f], all instances assembled per mesh in frequency batches and solved in
    one persistent launch.  q: None (q = 1, the pulsating sphere) or a list of
    per-instance vectors.  Returns (list of p_f, iterations, relative residual
    estimates, converged flags)."""
    ctx = ctx or default_context()
    ks = np.ascontiguousarray(ks, dtype=np.float64)
    mesh_of = np.ascontiguousarray(mesh_of, dtype=np.int32)
    nk = len(ks)
    if mesh_of.shape != (nk,):
        raise ValueError("one mesh index per wave number")
    dms = [m.device(ctx) for m in meshes]
    sizes = [m.num_elements for m in meshes]
    ns = [sizes[i] for i in mesh_of]
    if q is None:
        qf = np.ones(sum(ns), np.complex128)
    else:
        qf = np.concatenate([_c128(v) for v in q]) if nk else np.zeros(0, np.complex128)
        if qf.shape != (sum(ns),):
            raise ValueError("q: one vector per instance with its mesh's element count")
    pf = np.zeros_like(qf)
    handles = (ctypes.c_void_p * len(dms))(*[d.handle.value if hasattr(d.handle, "value") else d.handle for d in dms])
    it = np.zeros(nk, np.int32)
    rel = np.zeros(nk)
    conv = np.zeros(nk, np.int32)
    st = C.lib().nihu_gb_solve_sweep_batched(
        ctx.handle, len(dms), handles, family, nk, ks.ctypes.data, mesh_of.ctypes.data,
        C.REGULAR_FP64 if precision == "fp64" else C.REGULAR_FP32, qf.ctypes.data, pf.ctypes.data, restart, max_iters,
        tol, it.ctypes.data, rel.ctypes.data, conv.ctypes.data)
    if st != C.OK and (check or st != 6):
        ctx.check(st)
    out = np.split(pf, np.cumsum(ns)[:-1]) if nk else []
    return out, it, rel, conv.astype(bool)


class SweepPlan:
    """A frequency sweep over fixed meshes captured once as a CUDA graph
    (nihu_gb_sweep_plan_*): instance f on meshes[mesh_of[f]]; run(ks, q)
    replays assembly, right-hand sides and one persistent GMRES launch for a
    new set of wave numbers (|k| <= k_max) and Neumann data."""

    def __init__(self, meshes, mesh_of, k_max: float, family: int = C.HELMHOLTZ_3D, precision: str = "fp32",
                 restart: int = 50, max_iters: int = 1000, tol: float = 1e-6, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self.meshes = list(meshes)
        self._dms = [m.device(self.ctx) for m in self.meshes]
        self.mesh_of = np.ascontiguousarray(mesh_of, dtype=np.int32)
        self.nk = len(self.mesh_of)
        self.sizes = [self.meshes[i].num_elements for i in self.mesh_of]
        handles = (ctypes.c_void_p * len(self._dms))(*[d.handle.value for d in self._dms])
        h = ctypes.c_void_p()
        self.ctx.check(C.lib().nihu_gb_sweep_plan_create(
            self.ctx.handle, len(self._dms), handles, family, self.nk, self.mesh_of.ctypes.data, float(k_max),
            C.REGULAR_FP64 if precision == "fp64" else C.REGULAR_FP32, restart, max_iters, tol, ctypes.byref(h)))
        self.handle = h
        # the plan's pinned staging (instance order): Neumann data are written
        # and solutions read in place, with no further host copy
        self._off = np.concatenate([[0], np.cumsum(self.sizes)]).astype(np.int64)
        total = int(self._off[-1])
        qp, pp = ctypes.c_void_p(), ctypes.c_void_p()
        self.ctx.check(C.lib().nihu_gb_sweep_plan_host_buffers(h, ctypes.byref(qp), ctypes.byref(pp)))
        self._qptr, self._pptr = qp, pp
        self._q = np.frombuffer((ctypes.c_double * (2 * total)).from_address(qp.value), np.complex128)
        self._p = np.frombuffer((ctypes.c_double * (2 * total)).from_address(pp.value), np.complex128)

    def run(self, ks, q=None, check: bool = True, copy: bool = True):
        """Returns (list of p_f, iterations, relative residual estimates, converged).
        copy=False returns views of the plan's pinned staging (no host copy),
        valid until the next run or close()."""
        ks = np.ascontiguousarray(ks, dtype=np.float64)
        if ks.shape != (self.nk,):
            raise ValueError("one wave number per instance")
        if q is None:
            self._q[:] = 1.0
        else:
            if len(q) != self.nk or [np.shape(v) for v in q] != [(n,) for n in self.sizes]:
                raise ValueError("q: one vector per instance with its mesh's element count")
            np.concatenate(q, out=self._q)  # one pass, straight into the pinned staging
        it = np.zeros(self.nk, np.int32)
        rel = np.zeros(self.nk)
        conv = np.zeros(self.nk, np.int32)
        st = C.lib().nihu_gb_sweep_plan_run(self.handle, ks.ctypes.data, self._qptr, self._pptr,
                                            it.ctypes.data, rel.ctypes.data, conv.ctypes.data)
        if st != C.OK and (check or st != 6):
            self.ctx.check(st)
        return np.split(self._p.copy() if copy else self._p, self._off[1:-1]), it, rel, conv.astype(bool)

    def tuning(self) -> dict:
        """The launch set-up the plan's autotuner chose at creation."""
        c, f, ms = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_double(0.0)
        self.ctx.check(C.lib().nihu_gb_sweep_plan_tuning(self.handle, ctypes.byref(c), ctypes.byref(f),
                                                         ctypes.byref(ms)))
        return {"cluster": c.value, "freq_per_block": f.value, "replay_ms": ms.value}

    def close(self):
        if getattr(self, "handle", None):
            self._q = self._p = None  # views of the plan's staging
            C.lib().nihu_gb_sweep_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            if self.ctx.handle:
                self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching serving loop of CBIE solves (DLP - I/2) p = SLP q
    (nihu_gb_server_*).  Requests wait in a FIFO queue until the HBM budget
    holds them; each step() admits what fits, assembles the new requests (one
    frequency batch per mesh), advances every admitted system by at most
    `quantum` GMRES steps in one persistent launch and retires the finished
    ones, whose results take() returns.  A request's result does not depend
    on what else is in flight."""

    def __init__(self, meshes, family: int = C.HELMHOLTZ_3D, precision: str = "fp32",
                 hbm_budget_bytes: int = 150 << 30, max_active: int = 1024, restart: int = 50, max_iters: int = 1000,
                 tol: float = 1e-6, quantum: int = 8, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self.meshes = list(meshes)
        self._dms = [m.device(self.ctx) for m in self.meshes]
        self.sizes = [m.num_elements for m in self.meshes]
        handles = (ctypes.c_void_p * len(self._dms))(*[d.handle.value for d in self._dms])
        h = ctypes.c_void_p()
        self.ctx.check(C.lib().nihu_gb_server_create(
            self.ctx.handle, len(self._dms), handles, family, C.REGULAR_FP64 if precision == "fp64" else C.REGULAR_FP32,
            int(hbm_budget_bytes), max_active, restart, max_iters, tol, quantum, ctypes.byref(h)))
        self.handle = h
        self._mesh_of = {}

    def reserve(self, nbytes: int = 0):
        """Map nbytes (0: the whole budget) of device memory into the server's
        pool now, so that admissions inside the serving loop map none."""
        self.ctx.check(C.lib().nihu_gb_server_reserve(self.handle, int(nbytes)))

    def submit(self, mesh: int, k: float, q) -> int:
        q = _c128(q)
        if q.shape != (self.sizes[mesh],):
            raise ValueError("q must have the mesh's element count")
        rid = ctypes.c_int64(-1)
        self.ctx.check(C.lib().nihu_gb_server_submit(self.handle, mesh, float(k), q.ctypes.data, ctypes.byref(rid)))
        self._mesh_of[rid.value] = mesh
        return rid.value

    def step(self):
        """One round; returns (queued, active, finished-but-not-taken)."""
        a, b, c = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
        self.ctx.check(C.lib().nihu_gb_server_step(self.handle, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def take(self):
        """The oldest finished request as (id, p, iterations, relative residual,
        converged), or None."""
        cap = max(self.sizes)
        p = np.zeros(cap, np.complex128)
        rid, it, conv = ctypes.c_int64(-1), ctypes.c_int(0), ctypes.c_int(0)
        rel = ctypes.c_double(0.0)
        self.ctx.check(C.lib().nihu_gb_server_take(self.handle, ctypes.byref(rid), p.ctypes.data, cap, ctypes.byref(it),
                                                   ctypes.byref(rel), ctypes.byref(conv)))
        if rid.value < 0:
            return None
        n = self.sizes[self._mesh_of.pop(rid.value)]
        return rid.value, p[:n].copy(), it.value, rel.value, bool(conv.value)

    def close(self):
        if getattr(self, "handle", None):
            C.lib().nihu_gb_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            if self.ctx.handle:
                self.close()
        except Exception:
            pass


def near_pairs(test: Mesh, trial: Mesh, ctx: Context | None = None) -> tuple[np.ndarray, np.ndarray]:
    """The nearly singular pair list of (test, trial): (col_ptr, rows), the
    rows of trial column j in increasing order at rows[col_ptr[j]:col_ptr[j+1]]."""
    ctx = ctx or default_context()
    tdm = test.device(ctx)
    rdm = tdm if test is trial else trial.device(ctx)
    nnz = ctypes.c_int64()
    ctx.check(C.lib().nihu_gb_near_pairs(ctx.handle, tdm.handle, rdm.handle, ctypes.byref(nnz), None, None))
    col_ptr = np.zeros(rdm.n + 1, np.int64)
    rows = np.zeros(max(nnz.value, 1), np.int32)
    ctx.check(C.lib().nihu_gb_near_pairs(ctx.handle, tdm.handle, rdm.handle, ctypes.byref(nnz),
                                         col_ptr.ctypes.data, rows.ctypes.data))
    return col_ptr, rows[:nnz.value]


def pair_statistics(test: Mesh, trial: Mesh, ctx: Context | None = None) -> np.ndarray:
    """[self, near, regular (SLP level, DLP level) 3x3] pair counts."""
    ctx = ctx or default_context()
    out = (ctypes.c_int64 * 11)()
    tdm = test.device(ctx)
    rdm = tdm if test is trial else trial.device(ctx)
    ctx.check(C.lib().nihu_gb_pair_statistics(ctx.handle, tdm.handle, rdm.handle, out))
    return np.array(list(out), dtype=np.int64)
