"""sw2g_energy_noalloc: the energy diagnostic for callers that cannot let the
library allocate device memory (a pool allocator owns the device, a time loop
must not synchronise on cudaMalloc/cudaFree, or a tool owns its buffers and has
no sw2g context). Its scratch lives in a fixed static device array instead.

Checked through the C ABI against sw2g_diag on the same fields, twice in a row
(the second call must not see anything left over from the first), with the
tolerance the other energy tests use (relative 1e-12); with NULL winds and
bottom on a case that has none; for the argument checks it shares with
sw2g_create (rejected before anything is launched, so tiny buffers suffice);
and for the property that defines it: a call leaves the device's free memory
unchanged. This file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

from sw2_gb300 import cases, lib
from sw2_gb300.formats import CaseParams

pytestmark = pytest.mark.gpu

REL = 1e-12


def _noalloc():
    L = lib.load()
    f = L.sw2g_energy_noalloc
    vp = ctypes.c_void_p
    f.argtypes = [ctypes.POINTER(lib.Case), vp, vp, vp, vp, vp, vp, vp, vp]
    f.restype = ctypes.c_int
    return f


def _dev(torch, a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda:0")


def _check_against_diag(torch, case, hB, null_aux):
    s = lib.Solver(case.params)
    s.upload(case.eta, case.u, case.v, None, case.windx, case.windy, hB)
    fn = _noalloc()
    c = lib.case_struct(case.params)
    aux = [None, None, None] if null_aux else [_dev(torch, case.windx), _dev(torch, case.windy), _dev(torch, hB)]
    ptr = lambda t: None if t is None else t.data_ptr()
    out = torch.zeros(3, dtype=torch.float64, device="cuda:0")
    for call in range(2):
        assert s.step(7) == lib.OK
        ref = s.diag()
        st = s.download()
        eta, u, v = _dev(torch, st["eta"]), _dev(torch, st["u"]), _dev(torch, st["v"])
        out.fill_(float("nan"))
        torch.cuda.synchronize()
        rc = fn(ctypes.byref(c), eta.data_ptr(), u.data_ptr(), v.data_ptr(), ptr(aux[0]), ptr(aux[1]), ptr(aux[2]),
                out.data_ptr(), None)
        torch.cuda.synchronize()
        assert rc == lib.OK
        got = out.cpu().numpy()
        for g, r in zip(got, ref):
            assert abs(g - r) <= REL * abs(r), (call, g, r)
    s.close()


def test_energy_noalloc_matches_diag_two_calls():
    torch = pytest.importorskip("torch")
    wind = np.stack([np.arange(-180.0, 181.0), 25 * np.cos(np.deg2rad(np.arange(-180.0, 181.0)) * 2)], axis=1)
    case = cases.make_case(nx=200, ny=96, sch=2, seed=31, bumps=2, wind=wind)
    ny, nx = case.eta.shape
    jj = np.arange(ny)[:, None]
    hB = 50.0 * np.cos(2 * np.pi * jj / ny) * np.ones((1, nx))
    _check_against_diag(torch, case, hB, null_aux=False)


def test_energy_noalloc_null_winds_and_bottom_read_as_zero():
    torch = pytest.importorskip("torch")
    # more rows than one launch carries in its parameters (1024), so the row
    # geometry travels in two launches
    case = cases.make_case(nx=64, ny=1500, sch=2, seed=5, bumps=1)
    assert not np.any(case.windx) and not np.any(case.windy)
    _check_against_diag(torch, case, np.zeros_like(case.eta), null_aux=True)


def _rejects(torch, p, flags=0):
    fn = _noalloc()
    c = lib.case_struct(p, flags)
    buf = torch.zeros(8, dtype=torch.float64, device="cuda:0")
    rc = fn(ctypes.byref(c), buf.data_ptr(), buf.data_ptr(), buf.data_ptr(), None, None, None, buf.data_ptr(), None)
    torch.cuda.synchronize()
    return rc == lib.ERR_BAD_ARG


def test_energy_noalloc_rejects_bad_grids_before_launching():
    torch = pytest.importorskip("torch")
    # beyond its fixed scratch
    assert _rejects(torch, CaseParams(nx=4, ny=8193))
    # few rows but a row so long that padded cell indices leave 32 bits
    assert _rejects(torch, CaseParams(nx=300_000_000, ny=8))
    # a band that reaches a pole, in degrees and in radians
    assert _rejects(torch, CaseParams(nx=16, ny=8, lat0=-90.0, lat1=70.0))
    assert _rejects(torch, CaseParams(nx=16, ny=8, lat0=-1.0, lat1=np.pi / 2), flags=lib.FLAG_RADIANS)
    # polar caps (their gravity is a two-dimensional field)
    for pole in (1, -1):
        assert _rejects(torch, CaseParams(nx=16, ny=16, polar=pole, angleSim=20.0, BetaSp=15.0, SigSp=1e-4))
    # grids smaller than 3x3
    assert _rejects(torch, CaseParams(nx=2, ny=8))


def test_energy_noalloc_leaves_free_device_memory_unchanged():
    torch = pytest.importorskip("torch")
    case = cases.make_case(nx=128, ny=64, sch=2, seed=9, bumps=1)
    fn = _noalloc()
    c = lib.case_struct(case.params)
    eta, u, v = _dev(torch, case.eta), _dev(torch, case.u), _dev(torch, case.v)
    out = torch.zeros(3, dtype=torch.float64, device="cuda:0")
    args = (ctypes.byref(c), eta.data_ptr(), u.data_ptr(), v.data_ptr(), None, None, None, out.data_ptr(), None)
    assert fn(*args) == lib.OK  # the first call on the device loads the module
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(0)
    for _ in range(3):
        assert fn(*args) == lib.OK
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0
    assert np.all(np.isfinite(out.cpu().numpy()))
