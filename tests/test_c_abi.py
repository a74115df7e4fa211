"""The C-ABI library builds, loads and exports every symbol declared in
include/*.h; argument checks that need no GPU behave."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols(header=None):
    names = [header] if header else sorted(f for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h"))
    out = set()
    for h in names:
        src = open(os.path.join(ROOT, "include", h)).read()
        out |= set(re.findall(r"\b(mrg_[a-z_0-9]+)\s*\(", src))
    return sorted(out)


def test_header_and_binding_list_agree():
    from mray_gb300 import _native as N
    assert declared_symbols("mray_gb300.h") == sorted(N.EXPORTED)
    tracer = [n for n in declared_symbols("mray_gb300_tracer.h") if n.startswith("mrg_tracer_")]
    assert tracer == sorted(N.TRACER_EXPORTED)


def test_library_exports_every_declared_symbol(cuda_lib):
    lib = C.CDLL(cuda_lib)
    for s in declared_symbols():
        assert hasattr(lib, s), s


def test_no_gpu_paths_fail_cleanly(cuda_lib):
    from mray_gb300 import _native as N
    L = N.lib()
    assert L.mrg_create(None, None) == N.MRG_ERR_INVALID_ARG
    assert b"null" in L.mrg_last_error()
    assert L.mrg_build(None) == N.MRG_ERR_INVALID_ARG
    assert L.mrg_cast_closest(None, None, None, 0, None, None, None) == N.MRG_ERR_INVALID_ARG
    assert L.mrg_destroy(None) == N.MRG_OK
    assert L.mrg_status_string(N.MRG_ERR_TRAVERSAL) == b"traversal error"


def test_create_without_gpu_reports_error(cuda_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    from mray_gb300 import _native as N
    h = C.c_void_p()
    p = N.MrgParams(device=0)
    st = N.lib().mrg_create(C.byref(p), C.byref(h))
    assert st in (N.MRG_ERR_CUDA, N.MRG_ERR_INVALID_ARG)
    assert not h.value
