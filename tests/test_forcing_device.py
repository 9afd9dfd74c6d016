"""sw2g_add_gaussian: a Gaussian injection evaluated on the device
(perturbs.c:199-364). The runner tests hold its results against the
reference's frames; here its failure paths: an injection whose volume finds
no cell inside the radius is the reference's "total injected volume is 0"
(perturbs.c:316), returned at once between steps and by sw2g_step_close
inside an opened step, with the context still usable; a volume below the
reference's 1e-7 threshold leaves eta unchanged."""
import math

import numpy as np
import pytest

from sw2_gb300 import cases, lib

pytestmark = pytest.mark.gpu


def solver(precision=lib.FP64):
    case = cases.make_case(nx=64, ny=32, sch=2, seed=5)
    flags = lib.FLAG_VANLEER_SAFE if precision == lib.FP32 else 0
    s = lib.Solver(case.params, precision=precision, flags=flags)
    s.upload(*case.fields())
    return case, s


def between_columns(case):
    """A longitude half a column from the cell centres, and a radius of one metre:
    no cell centre lies inside."""
    p = case.params
    dlon = (p.lon1 - p.lon0) / p.nx
    return math.radians(p.lon0 + 10.0 * dlon)  # the edge between the centres of columns 10 and 11


@pytest.mark.parametrize("precision", [lib.FP64, lib.FP32])
def test_no_cell_inside_the_radius_is_a_forcing_error(precision):
    case, s = solver(precision)
    p = case.params
    lat_row = math.radians(p.lat0 + (p.lat1 - p.lat0) * 15.5 / p.ny)  # a row's centre latitude
    g = lib.Gaussian(lon=between_columns(case), lat=lat_row, amp=1.0, sigma=1e6, radius=1.0, inject=0.0,
                     volume=1.0, images=0)
    assert s.add_gaussian(g) == lib.ERR_FORCING  # the device found V = 0
    g.lat = math.radians(p.lat0 + (p.lat1 - p.lat0) * 15.0 / p.ny)  # on a row boundary: no row within reach
    assert s.add_gaussian(g) == lib.ERR_FORCING
    # inside an opened step the failure comes back from sw2g_step_close
    lib.load().sw2g_step_open.argtypes = [lib.ctypes.c_void_p]
    lib.load().sw2g_step_close.argtypes = [lib.ctypes.c_void_p]
    assert lib.load().sw2g_step_open(s.h) == lib.OK
    g.lat = lat_row
    assert s.add_gaussian(g) == lib.OK
    assert lib.load().sw2g_step_close(s.h) == lib.ERR_FORCING
    # the context goes on
    assert s.step(2) == lib.OK


def test_small_volume_leaves_eta_and_sets_the_tracer():
    case, s = solver()
    p = case.params
    before = s.download()
    g = lib.Gaussian(lon=math.radians(0.5 * (p.lon0 + p.lon1)), lat=0.0, amp=0.0, sigma=2e6, radius=6e6,
                     inject=0.75, volume=0.0, images=0)
    assert s.add_gaussian(g) == lib.OK
    after = s.download()
    assert np.array_equal(after["eta"], before["eta"])
    inside = after["tracer"] != before["tracer"]
    assert inside.any()
    assert np.all(after["tracer"][inside] <= 0.75) and np.all(after["tracer"][inside] > 0.0)
