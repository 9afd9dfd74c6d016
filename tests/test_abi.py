"""The C-ABI library loads without a GPU and exports every entry point that
include/*.h declares; host-side argument checks fail cleanly."""
import ctypes
import glob
import os
import re

import pytest

from sw2_gb300 import build, lib
from sw2_gb300.formats import CaseParams

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(sw2g_\w+)\s*\(", text))
    return sorted(names)


@pytest.fixture(scope="module")
def L():
    build.build()
    return lib.load()


def test_library_exports_every_declared_symbol(L):
    names = declared()
    assert len(names) >= 15
    for n in names:
        assert hasattr(L, n), n
    assert set(lib.SYMBOLS) <= set(names)


def test_status_strings(L):
    assert lib.status_string(lib.OK) == "ok"
    assert "CFL" in lib.status_string(lib.ERR_CFL)
    assert "volume" in lib.status_string(lib.ERR_FORCING)
    assert lib.status_string(99) == "unknown status"


def test_device_gaussian_rejects_bad_arguments_before_the_gpu(L):
    L.sw2g_add_gaussian.argtypes = [ctypes.c_void_p, ctypes.POINTER(lib.Gaussian)]
    g = lib.Gaussian(lon=0.0, lat=0.0, amp=1.0, sigma=1e6, radius=3e6, inject=0.0, volume=1.0, images=0)
    assert L.sw2g_add_gaussian(None, ctypes.byref(g)) == lib.ERR_BAD_ARG


def test_create_rejects_bad_cases_without_touching_the_gpu(L):
    bad = [dict(nx=2, ny=8), dict(nx=8, ny=8, sch=10), dict(nx=8, ny=8, Dt=-1.0),
           dict(nx=8, ny=8, lat0=-95.0), dict(nx=8, ny=8, hypernu=(0.0, -1.0, 0.0))]
    for kw in bad:
        p = CaseParams(**kw)
        h = ctypes.c_void_p()
        c = lib.case_struct(p)
        assert L.sw2g_create(ctypes.byref(c), lib.FP64, 0, ctypes.byref(h)) == lib.ERR_BAD_ARG
        assert not h.value
    # unknown flags and precision
    c = lib.case_struct(CaseParams(nx=8, ny=8), flags=0x80)
    assert L.sw2g_create(ctypes.byref(c), lib.FP64, 0, ctypes.byref(ctypes.c_void_p())) == lib.ERR_BAD_ARG
    c = lib.case_struct(CaseParams(nx=8, ny=8))
    assert L.sw2g_create(ctypes.byref(c), 7, 0, ctypes.byref(ctypes.c_void_p())) == lib.ERR_BAD_ARG


def test_null_context_calls_are_rejected(L):
    assert L.sw2g_step(None, 1) == lib.ERR_BAD_ARG
    assert L.sw2g_download(None, None, None, None, None) == lib.ERR_BAD_ARG
    assert L.sw2g_error_step(None) == -1
    L.sw2g_destroy(None)


def test_host_array_step_and_add_selfcheck_reject_bad_arguments(L):
    """Checked on the host before any CUDA call."""
    buf = (ctypes.c_double * 16)()
    p = ctypes.cast(buf, ctypes.POINTER(ctypes.c_double))
    assert L.sw2g_step_host(None, p, p, p, 1) == lib.ERR_BAD_ARG
    L.sw2g_selfcheck_add.argtypes = [ctypes.c_longlong, ctypes.c_ulonglong, ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_longlong)]
    out = ctypes.c_longlong(-7)
    assert L.sw2g_selfcheck_add(0, 1, 0, ctypes.byref(out)) == lib.ERR_BAD_ARG
    assert L.sw2g_selfcheck_add(10, 1, 0, None) == lib.ERR_BAD_ARG
    assert out.value == -7
