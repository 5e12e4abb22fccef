"""The C-ABI library loads and exports every symbol include/nihu_gb300.h declares (CPU, no compute)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "nihu_gb300.h")).read()
    return sorted(set(re.findall(r"\b(nihu_gb_\w+)\s*\(", txt)))


def test_header_and_binding_agree():
    from nihu_gb300 import _capi
    assert declared_symbols() == sorted(_capi.SIGNATURES)


def test_binding_argument_counts_match_header():
    from nihu_gb300 import _capi
    txt = open(os.path.join(ROOT, "include", "nihu_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    decls = dict(re.findall(r"\b(nihu_gb_\w+)\s*\(([^;{]*?)\)\s*;", txt))
    assert sorted(decls) == sorted(_capi.SIGNATURES)
    for name, params in decls.items():
        params = params.strip()
        count = 0 if params in ("", "void") else params.count(",") + 1
        assert count == len(_capi.SIGNATURES[name][1]), name


def test_library_exports_all_symbols():
    import nihu_gb300
    L = nihu_gb300.lib()
    for name in declared_symbols():
        assert hasattr(L, name), name


def test_no_device_is_reported_not_faked():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import nihu_gb300
    L = nihu_gb300.lib()
    h = ctypes.c_void_p()
    assert L.nihu_gb_ctx_create(0, None, 0, ctypes.byref(h)) == 7  # NIHU_GB_ERR_NO_DEVICE
    with pytest.raises(nihu_gb300.NihuError):
        nihu_gb300.Context(0)
