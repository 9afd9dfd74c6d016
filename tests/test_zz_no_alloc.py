"""sw2g_energy_noalloc: the energy diagnostic for callers that cannot let the
library allocate device memory (a pool allocator owns the device, a time loop
must not synchronise on cudaMalloc/cudaFree, or a tool owns its buffers and has
no sw2g context). Its scratch lives in a fixed static device array instead.

Checked through the C ABI against sw2g_diag on the same fields, twice in a row
(the second call must not see anything left over from the first), with the
tolerance the other energy tests use (relative 1e-12). This file is named to be
collected last.
"""
import ctypes

import numpy as np
import pytest

from sw2_gb300 import cases, lib

pytestmark = pytest.mark.gpu

REL = 1e-12


def _noalloc():
    L = lib.load()
    f = L.sw2g_energy_noalloc
    vp = ctypes.c_void_p
    f.argtypes = [ctypes.POINTER(lib.Case), vp, vp, vp, vp, vp, vp, vp, vp]
    f.restype = ctypes.c_int
    return f


def test_energy_noalloc_matches_diag_two_calls():
    torch = pytest.importorskip("torch")
    wind = np.stack([np.arange(-180.0, 181.0), 25 * np.cos(np.deg2rad(np.arange(-180.0, 181.0)) * 2)], axis=1)
    case = cases.make_case(nx=200, ny=96, sch=2, seed=31, bumps=2, wind=wind)
    ny, nx = case.eta.shape
    jj = np.arange(ny)[:, None]
    hB = 50.0 * np.cos(2 * np.pi * jj / ny) * np.ones((1, nx))
    s = lib.Solver(case.params)
    s.upload(case.eta, case.u, case.v, None, case.windx, case.windy, hB)
    fn = _noalloc()
    c = lib.case_struct(case.params)
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda:0")
    wx, wy, hb = dev(case.windx), dev(case.windy), dev(hB)
    out = torch.zeros(3, dtype=torch.float64, device="cuda:0")
    for call in range(2):
        assert s.step(7) == lib.OK
        ref = s.diag()
        st = s.download()
        eta, u, v = dev(st["eta"]), dev(st["u"]), dev(st["v"])
        out.fill_(float("nan"))
        torch.cuda.synchronize()
        rc = fn(ctypes.byref(c), eta.data_ptr(), u.data_ptr(), v.data_ptr(), wx.data_ptr(), wy.data_ptr(),
                hb.data_ptr(), out.data_ptr(), None)
        torch.cuda.synchronize()
        assert rc == lib.OK
        got = out.cpu().numpy()
        for g, r in zip(got, ref):
            assert abs(g - r) <= REL * abs(r), (call, g, r)


def test_energy_noalloc_rejects_rows_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    fn = _noalloc()
    from sw2_gb300.formats import CaseParams

    p = CaseParams(nx=4, ny=8193)
    c = lib.case_struct(p)
    buf = torch.zeros(8, dtype=torch.float64, device="cuda:0")
    rc = fn(ctypes.byref(c), buf.data_ptr(), buf.data_ptr(), buf.data_ptr(), None, None, None, buf.data_ptr(), None)
    assert rc == lib.ERR_BAD_ARG
