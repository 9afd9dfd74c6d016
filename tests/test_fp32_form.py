"""FP32 precision form against the FP64 reference-exact step.

The FP32 form runs the same algorithm (including the reference's halo and wall
semantics) with FP32 stencils and FP64 state accumulation. Checks:
  * after a few steps every padded cell (halos included) is within FP32
    round-off of the FP64 result, so any error in the halo images, the seam
    ghosts or the wall fixes would show up as an O(1) difference;
  * after many steps the relative L2 error of h = eta + depth is below 1e-5
    (the stated bar), and u, v stay close.
"""
import dataclasses

import numpy as np
import pytest

from sw2_gb300 import cases, lib
from tests import golden_cases as gc

pytestmark = pytest.mark.gpu


def run(case, precision, n, flags=0):
    s = lib.Solver(case.params, precision=precision, flags=flags)
    s.upload(*case.fields())
    rc = s.step(n)
    assert rc == lib.OK, (rc, s.error_step())
    return s, s.download()


def rel_l2(a, b):
    a, b = a[2:-2, 2:-2], b[2:-2, 2:-2]
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("sch", [2, 1, 0, 3, 4, 7])
def test_fp32_all_cells_close_after_few_steps(sch):
    case = cases.make_case(nx=97, ny=45, sch=sch, seed=40 + sch, bumps=3, sigma_km=(3000.0, 6000.0))
    flags = lib.FLAG_VANLEER_SAFE if sch == 3 else 0
    _, a = run(case, lib.FP32, 4, flags)
    _, b = run(case, lib.FP64, 4, flags)
    depth = case.params.depth
    assert np.max(np.abs(a["eta"] - b["eta"])) <= 2e-6 * depth
    for k in ("u", "v"):
        scale = np.max(np.abs(b["u"]))
        assert np.max(np.abs(a[k] - b[k])) <= 2e-5 * scale, (k, np.max(np.abs(a[k] - b[k])))


def test_fp32_halos_follow_the_reference_quirks():
    """Row ny of v: interior zeroed by the wall, x-halo columns keep the
    pre-wall Coriolis value (calc.c:600-649 after the halo update)."""
    case = cases.make_case(nx=64, ny=32, sch=2, seed=5, bumps=2)
    _, a = run(case, lib.FP32, 3)
    _, b = run(case, lib.FP64, 3)
    ny = case.params.ny
    row = ny + 1
    assert np.all(a["v"][row, 2:-2] == 0) and np.all(b["v"][row, 2:-2] == 0)
    stale = b["v"][row, [0, 1, -2, -1]]
    assert np.any(stale != 0)
    assert np.allclose(a["v"][row, [0, 1, -2, -1]], stale, rtol=1e-4, atol=1e-6 * np.max(np.abs(b["v"])))


@pytest.mark.parametrize("nx,ny", [(3, 3), (33, 9), (130, 66)])
def test_fp32_odd_sizes(nx, ny):
    case = cases.make_case(nx=nx, ny=ny, sch=1, seed=8, bumps=1, sigma_km=(8000.0, 8000.0))
    _, a = run(case, lib.FP32, 5)
    _, b = run(case, lib.FP64, 5)
    assert np.max(np.abs(a["eta"] - b["eta"])) <= 2e-6 * case.params.depth
    assert np.max(np.abs(a["u"] - b["u"])) <= 2e-5 * max(1.0, np.max(np.abs(b["u"])))


def test_fp32_winds_and_nu2():
    wind = np.stack([np.arange(-180.0, 181.0), 20 * np.cos(np.deg2rad(np.arange(-180.0, 181.0)) * 4)], axis=1)
    case = cases.make_case(nx=80, ny=40, sch=2, seed=9, wind=wind)
    nu4 = case.params.hypernu[1]
    case.params.hypernu = (1e-3 * nu4 ** 0.5, nu4, 0.0)
    _, a = run(case, lib.FP32, 4)
    _, b = run(case, lib.FP64, 4)
    assert np.max(np.abs(a["eta"] - b["eta"])) <= 2e-6 * case.params.depth
    assert np.max(np.abs(a["u"] - b["u"])) <= 2e-5 * np.max(np.abs(b["u"]))


def test_fp32_nu2_nu4_nu6():
    """All three hyperviscosity orders (laplacian_vels applied three times,
    core.c:233-268): the third level is the Laplacian of the second, with the
    same halo images and wall fixes, added to the partial tendencies."""
    case = cases.make_case(nx=96, ny=48, sch=1, seed=12)
    nu4 = case.params.hypernu[1]  # grid-scale e-folding time 10 Dt
    # nu6 with a grid-scale e-folding time of 20 Dt, so that it matters
    nu6 = 0.5 * nu4 ** 1.5 * (10.0 * case.params.Dt) ** 0.5
    case.params.hypernu = (2.0e-3 * nu4 ** 0.5, 0.5 * nu4, nu6)
    _, a = run(case, lib.FP32, 6)
    _, b = run(case, lib.FP64, 6)
    assert np.max(np.abs(a["eta"] - b["eta"])) <= 2e-6 * case.params.depth
    assert np.max(np.abs(a["u"] - b["u"])) <= 2e-5 * np.max(np.abs(b["u"]))
    assert np.max(np.abs(a["v"] - b["v"])) <= 2e-5 * max(1.0, np.max(np.abs(b["v"])))
    # and it matters: without nu6 the FP64 step ends elsewhere
    case.params.hypernu = (2.0e-3 * nu4 ** 0.5, 0.5 * nu4, 0.0)
    _, c = run(case, lib.FP64, 6)
    assert np.max(np.abs(c["u"] - b["u"])) > 10 * np.max(np.abs(a["u"] - b["u"]))


@pytest.mark.parametrize("sch", [1, 2, 3])
def test_fp32_tracer_with_winds(sch):
    """The tracer (BODYTRACER, calc.c:117-163; AB and update, core.c:161-182)
    advected by the flow plus a zonal wind, with its dissipation: FP64 state,
    FP32 fluxes, within the tolerance of the other fields."""
    wind = np.stack([np.arange(-180.0, 181.0), 25 * np.cos(np.deg2rad(np.arange(-180.0, 181.0)) * 3)], axis=1)
    case = cases.make_case(nx=64, ny=32, sch=sch, seed=21, wind=wind, tracer=True, TracerDis=2.0e-6)
    flags = lib.FLAG_VANLEER_SAFE if sch == 3 else 0
    _, a = run(case, lib.FP32, 8, flags=flags)
    _, b = run(case, lib.FP64, 8, flags=flags)
    assert np.max(np.abs(b["tracer"])) > 0.1
    assert np.max(np.abs(a["tracer"] - b["tracer"])) <= 2e-5 * np.max(np.abs(b["tracer"]))
    assert np.max(np.abs(a["eta"] - b["eta"])) <= 2e-6 * case.params.depth
    # the tracer moved: it differs from its initial field
    assert np.max(np.abs(b["tracer"] - case.tracer)) > 1e-3 * np.max(np.abs(b["tracer"]))


def test_fp32_rejects_what_it_does_not_cover():
    case = cases.make_case(nx=16, ny=8, sch=2, seed=1)
    with pytest.raises(lib.SW2GError):
        lib.Solver(case.params, precision=lib.FP32, flags=lib.FLAG_LAPE_ETA)


def _polar_pair(params, fields):
    flags = lib.FLAG_VANLEER_SAFE if params.sch == 3 else 0
    a = lib.Solver(params, precision=lib.FP32, flags=flags)
    b = lib.Solver(params, precision=lib.FP64, flags=flags)
    for s in (a, b):
        s.upload(*fields, mode=lib.UPLOAD_FRAME)
    return a, b


def _pole_distance(params):
    """Distance of every padded cell from the cap's pole (the grid's centre), in cells."""
    H, W = params.ny + 4, params.nx + 4
    jj, ii = np.mgrid[0:H, 0:W]
    return np.hypot(jj - (H - 1) / 2.0, ii - (W - 1) / 2.0)


def _check_fp32_polar(ga, gb, depth, mask=None):
    m = np.ones(ga["eta"].shape, bool) if mask is None else mask
    assert np.max(np.abs(ga["eta"] - gb["eta"])[m]) <= 2e-6 * depth
    for k in ("u", "v", "tracer"):
        scale = max(float(np.max(np.abs(gb[k]))), 1e-300)
        err = np.max(np.abs(ga[k] - gb[k])[m])
        assert err <= 2e-4 * scale, (k, err / scale)


@pytest.mark.parametrize("name", gc.polar_cases())
def test_fp32_polar_caps(name):
    """Polar caps (init.c:66-79) in the FP32 form: per-cell gravity, Coriolis
    and sponge factors, turned winds, no walls (every halo wraps, and the
    Laplacian intermediates of the halo rows are those of the rows they wrap
    from), against the FP64 form and the reference's own frames at every
    saved frame.

    Limiter 2 (calc.c:54-63, psi(r) = r below 1, no lower bound) makes the
    limited slope psi(r)*d jump from 0 to the upwind difference n when the
    face difference d changes sign. At the pole the turned winds of mirrored
    cells are equal up to FP64 rounding, so the FP64 form (like the
    reference) follows the sign of a rounding residue where the FP32 shadows
    hold an exact zero. With that limiter the FP32 form stays within its
    tolerance 12 cells or more from the pole, and within a bound set by the
    wind's Courant number (1e-3 of eta's range, 2e-3 of the velocity range)
    at the pole."""
    entry, case, frames = gc.load_case(name)
    a, b = _polar_pair(case.params, case.fields())
    depth = case.params.depth
    near = _pole_distance(case.params) <= 12
    for fr in frames:
        assert a.step(entry["save_every"]) == lib.OK
        assert b.step(entry["save_every"]) == lib.OK
        ga, gb = a.download(), b.download()
        assert np.max(np.abs(gb["eta"][2:-2, 2:-2] - fr["eta"])) <= 1e-9 * depth
        if case.params.sch != 2:
            _check_fp32_polar(ga, gb, depth)
            assert np.max(np.abs(ga["eta"][2:-2, 2:-2] - fr["eta"])) <= 2e-6 * depth
            continue
        _check_fp32_polar(ga, gb, depth, mask=~near)
        assert np.max(np.abs(ga["eta"] - gb["eta"])) <= 1e-3 * float(np.ptp(gb["eta"]))
        for k in ("u", "v"):
            assert np.max(np.abs(ga[k] - gb[k])) <= 2e-3 * float(np.max(np.abs(gb[k])))
    ka, pa, ma = a.diag()
    kb, pb, mb = b.diag()
    assert abs(ma - mb) <= 1e-8 * abs(mb)


def test_fp32_polar_cap_bounded_limiter():
    """The north cap with limiter 1 (superbee, a bounded psi) in place of
    limiter 2: every padded cell of the FP32 form within tolerance of the
    FP64 form, the pole included, over 60 steps."""
    entry, case, _ = gc.load_case("p01_north_minmod_nu4")
    params = dataclasses.replace(case.params, sch=1)
    a, b = _polar_pair(params, case.fields())
    for _ in range(3):
        assert a.step(20) == lib.OK and b.step(20) == lib.OK
        _check_fp32_polar(a.download(), b.download(), params.depth)


@pytest.mark.slow
def test_fp32_band256_500_steps_error_bar():
    case = cases.config_case("band256")
    sa, a = run(case, lib.FP32, 500)
    sb, b = run(case, lib.FP64, 500)
    d = case.params.depth
    e_h = rel_l2(a["eta"] + d, b["eta"] + d)
    assert e_h <= 1e-5, e_h
    assert rel_l2(a["u"], b["u"]) <= 1e-3
    ka, pa, ma = sa.diag()
    kb, pb, mb = sb.diag()
    assert abs(ma - mb) <= 1e-9 * abs(mb)


def test_fp32_bounded_tile_wait_reports_timeout():
    """Failure path of the FP32 form's bounded device waits (TMA tile loads on
    an mbarrier): tiles that never complete make every block give up after
    its wait limit and the step return SW2G_ERR_TIMEOUT, with the device and
    the library still usable afterwards."""
    case = cases.make_case(nx=64, ny=32, sch=2, seed=4)
    s = lib.Solver(case.params, precision=lib.FP32)
    s.upload(*case.fields())
    assert s.step(2) == lib.OK
    s.test_tile_timeout(3)
    with pytest.raises(lib.SW2GError) as err:
        s.step(1)
    assert err.value.code == lib.ERR_TIMEOUT
    s.test_tile_timeout(0)
    s.upload(*case.fields())
    assert s.step(3) == lib.OK
    # a fresh context of either form runs normally on the same device
    s64 = lib.Solver(case.params)
    s64.upload(*case.fields())
    assert s64.step(3) == lib.OK
    with pytest.raises(lib.SW2GError):
        s64.test_tile_timeout(3)  # FP64 contexts have no such waits
