"""The allocation-free matvec entry point, nihu_gb_matvec_noalloc.

Callers that cannot allocate device memory -- hosts that reserve all of it for
their own pool, request loops that must never wait on the allocator, plug-in
hosts whose memory manager forbids allocations behind their back -- use this
entry point: it takes device buffers from the caller and keeps its partial
sums in one fixed static device array.  These tests check it through the
C ABI against the allocating entry point nihu_gb_matvec, on two calls in a
row (the second call reuses the scratch the first one left behind).

The file is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

import nihu_gb300 as g
from nihu_gb300 import _capi as C

pytestmark = pytest.mark.gpu


def _device_copy(ctx, arr):
    L = g.lib()
    p = ctypes.c_void_p()
    ctx.check(L.nihu_gb_device_alloc(ctx.handle, max(arr.nbytes, 16), ctypes.byref(p)))
    ctx.check(L.nihu_gb_memcpy(ctx.handle, p, C.DEVICE, arr.ctypes.data, C.HOST, arr.nbytes))
    return p


def _to_host(ctx, p, like):
    out = np.empty_like(like)
    ctx.check(g.lib().nihu_gb_memcpy(ctx.handle, out.ctypes.data, C.HOST, p, C.DEVICE, out.nbytes))
    return out


@pytest.mark.parametrize("dt,m,n", [(np.complex64, 3000, 2500), (np.complex128, 1500, 1700)])
def test_noalloc_matches_allocating_matvec_twice(dt, m, n):
    L = g.lib()
    ctx = g.Context(0)
    ptrs = []
    try:
        rng = np.random.default_rng(11)
        A = np.asfortranarray((rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n))).astype(dt))
        dtype = C.C64 if dt == np.complex64 else C.C128
        tol = 1e-5 if dt == np.complex64 else 1e-13
        dA = _device_copy(ctx, A)
        ptrs.append(dA)
        for call in range(2):  # two calls in a row share the static scratch
            x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
            y0 = rng.standard_normal(m) + 1j * rng.standard_normal(m)
            alpha, beta = complex(0.7, -0.2), complex(0.3 * call, 0.1)
            dx = _device_copy(ctx, x)
            dy_ref = _device_copy(ctx, y0)
            dy = _device_copy(ctx, y0)
            ptrs += [dx, dy_ref, dy]
            ctx.check(L.nihu_gb_matvec(ctx.handle, dtype, dA, m, n, m, dx, dy_ref, alpha.real, alpha.imag,
                                       beta.real, beta.imag, C.DEVICE))
            st = L.nihu_gb_matvec_noalloc(dtype, dA, m, n, m, dx, dy, alpha.real, alpha.imag, beta.real, beta.imag,
                                          ctx.stream)
            assert st == C.OK
            got = _to_host(ctx, dy, y0)  # the copy runs on the same stream, after the product
            ref = _to_host(ctx, dy_ref, y0)
            assert np.abs(got - ref).max() / np.abs(ref).max() < tol
            exact = alpha * (A.astype(np.complex128) @ x) + beta * y0
            assert np.abs(got - exact).max() / np.abs(exact).max() < tol
    finally:
        for p in ptrs:
            L.nihu_gb_device_free(ctx.handle, p)
        ctx.close()


def test_noalloc_allocates_nothing_and_rejects_oversize():
    torch = pytest.importorskip("torch")
    L = g.lib()
    ctx = g.Context(0)
    ptrs = []
    try:
        m, n = 1024, 512
        rng = np.random.default_rng(3)
        A = np.asfortranarray((rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n))).astype(np.complex64))
        dA = _device_copy(ctx, A)
        dx = _device_copy(ctx, np.ones(n, np.complex128))
        dy = _device_copy(ctx, np.zeros(m, np.complex128))
        ptrs += [dA, dx, dy]
        args = (C.C64, dA, m, n, m, dx, dy, 1.0, 0.0, 0.0, 0.0, ctx.stream)
        assert L.nihu_gb_matvec_noalloc(*args) == C.OK  # first call on the device: address set-up
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info(0)[0]
        bytes_before = ctx.device_bytes
        for _ in range(3):
            assert L.nihu_gb_matvec_noalloc(*args) == C.OK
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info(0)[0] == free_before
        assert ctx.device_bytes == bytes_before
        # more rows than the static scratch can hold: clear error, nothing launched
        big = C.NOALLOC_PARTIAL_ELEMS + 1
        assert L.nihu_gb_matvec_noalloc(C.C64, dA, big, 1, big, dx, dy, 1.0, 0.0, 0.0, 0.0, ctx.stream) == 2
        assert L.nihu_gb_matvec_noalloc(C.C64, None, 10, 10, 10, dx, dy, 1.0, 0.0, 0.0, 0.0, ctx.stream) == 1
    finally:
        for p in ptrs:
            L.nihu_gb_device_free(ctx.handle, p)
        ctx.close()
