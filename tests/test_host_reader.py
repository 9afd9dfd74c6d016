"""The case-file front end on the CPU (libsw2host.so): the m4 subset, the
'<expression>' evaluator, the reader's tag sequence (init.c:48-237) against
the case writer, and the host forcing fields (perturbs.c) against their
defining properties. The GPU runs of the same cases are tests/test_runner.py."""
import math
import os

import numpy as np
import pytest

from sw2_gb300 import cases, formats, hostlib
from tests import golden_cases as gc


@pytest.fixture(scope="module", autouse=True)
def built():
    if not os.path.exists(hostlib.LIB_PATH):
        pytest.skip("libsw2host.so not built")


@pytest.mark.parametrize("expr,value", [
    ("86400*20", 1728000.0), ("12*3600/50", 864.0), ("2+3^2", 11.0), ("-2^2", 4.0), ("2^3^2", 64.0),
    ("7 % 3", 1.0), ("(1+2)*(3+4)", 21.0), ("2*pi", 2 * math.pi), ("e", math.e), ("log(1000)", 3.0),
    ("ln(e)", 1.0), ("sqrt(16)+abs(-2)", 6.0), ("pow(2,10)", 1024.0), ("atan2(1,1)*4", math.pi),
    ("sin 0", 0.0), ("fac(5)", 120.0), ("ncr(6,2)", 15.0), ("1.5e3/3", 500.0), ("-(-3)", 3.0), ("1,2,3", 3.0),
])
def test_expressions(expr, value):
    assert hostlib.evaluate(expr) == pytest.approx(value, rel=1e-15, abs=1e-15)


@pytest.mark.parametrize("bad", ["", "2+", "(1", "foo(2)", "2 3"])
def test_bad_expressions(bad):
    with pytest.raises(ValueError):
        hostlib.evaluate(bad)


def test_m4_define_include_comments(tmp_path):
    (tmp_path / "planet.inc").write_text("rE R # radius, R stays in comments\n")
    (tmp_path / "c.sw").write_text("define(R,7.1492e7)\ndefine(TWO, 2)\ninclude(planet.inc)\nx TWO TWOX R\n")
    out = hostlib.m4(str(tmp_path / "c.sw"))
    assert "rE 7.1492e7 # radius, R stays in comments" in out
    assert "x 2 TWOX 7.1492e7" in out


def test_reader_expressions_and_macros(tmp_path):
    p = formats.CaseParams(nx=24, ny=12, nsteps=30, Dt=50.0)
    path = tmp_path / "c.sw"
    formats.write_sw(str(path), p)
    text = path.read_text().replace("\nt1 ", "\nt1 <DAY*20> # ", 1).replace("Dt 50.0", "Dt DT")
    path.write_text("define(DAY,86400)\ndefine(DT,50)\n" + text)
    c = hostlib.Case(str(path))
    assert c.t1 == 1728000.0 and c.Dt == 50.0 and c.N == 34560


@pytest.mark.parametrize("name", gc.forcing_cases() + ["g11_wind_tracer", "g14_oblate_nu2"])
def test_reader_reads_what_the_writer_wrote(tmp_path, name):
    p = gc.forcing_params(name) if name.startswith("f") else gc.params_of(gc.manifest()[name])
    path = tmp_path / "c.sw"
    formats.write_sw(str(path), p)
    c = hostlib.Case(str(path))
    d2r = lambda a: a * ((4.0 * math.atan(1.0)) / 180.0)  # noqa: E731 (sw.h:108)
    assert (c.nx, c.ny, c.sch, c.polar) == (p.nx, p.ny, p.sch, 0)
    assert (c.lon0, c.lon1, c.lat0, c.lat1) == tuple(d2r(x) for x in (p.lon0, p.lon1, p.lat0, p.lat1))
    assert (c.t0, c.t1, c.Dt, c.CFL) == (p.t0, p.t1, p.Dt, p.CFL)
    assert c.N == int((p.t1 - p.t0) / p.Dt) == p.nsteps
    assert (c.nu2, c.nu4, c.nu6) == tuple(p.hypernu)
    assert c.sigma_dis == (0.0 if p.Tau > 1e10 else 1.0 / p.Tau)
    assert (c.IteInfo, c.saveEvery, c.loadFrom) == (p.IteInfo, p.SaveEvery, p.LoadFrom)
    assert (c.Omega, c.rE, c.rP, c.gE, c.depth, c.tracer_dis) == (p.Omega, p.rE, p.rP, p.gE, p.depth, p.TracerDis)
    assert np.array_equal(c.table("gaussians"), np.array(p.gaussians).reshape(-1, 12))
    assert np.array_equal(c.table("vortices"), np.array(p.vortices).reshape(-1, 7))
    w = p.wind if p.wind is not None else np.array([[-180.0, 0.0], [180.0, 0.0]])
    assert np.array_equal(c.table("wind"), w)


@pytest.mark.parametrize("name", gc.polar_cases())
def test_reader_reads_polar_caps(tmp_path, name):
    """A polar cap's file (init.c:66-74, 154-157): the square -angleSim..angleSim
    around the pole, n cells a side, the sponge values, and the turned winds
    the reference ran the cap with."""
    entry, case, _ = gc.load_case(name)
    p = case.params
    path = tmp_path / "c.sw"
    formats.write_sw(str(path), p)
    c = hostlib.Case(str(path))
    a = p.angleSim * ((4.0 * math.atan(1.0)) / 180.0)
    assert (c.nx, c.ny, c.polar) == (p.nx, p.ny, p.polar) and p.nx == p.ny
    assert (c.lon0, c.lon1, c.lat0, c.lat1) == (-a, a, -a, a)
    assert (c.beta_sponge, c.sigma_sponge) == (p.BetaSp, p.SigSp)
    wx, wy = c.winds(c.beta_sponge)
    assert np.array_equal(wx, case.windx) and np.array_equal(wy, case.windy)


def test_windx_matches_the_python_restatement(tmp_path):
    p = gc.params_of(gc.manifest()["g11_wind_tracer"])
    path = tmp_path / "c.sw"
    formats.write_sw(str(path), p)
    wx, _ = cases.wind_fields(p)
    got = hostlib.Case(str(path)).windx()
    # the Python restatement also applies do_channel's wall copies (calc.c:600-649),
    # which the runner leaves to the GPU step's start-up
    I = slice(2, p.nx + 2)
    got[1, I] = got[2, I]
    got[0, I] = got[1, I]
    got[p.ny + 2, I] = got[p.ny + 1, I]
    got[p.ny + 3, I] = got[p.ny + 2, I]
    assert np.array_equal(got, wx)


def _case(tmp_path, name):
    path = tmp_path / "c.sw"
    formats.write_sw(str(path), gc.forcing_params(name))
    return hostlib.Case(str(path))


def test_gaussian_injects_its_volume(tmp_path):
    c = _case(tmp_path, "f01_gauss_static")
    f = hostlib.Forcing(c)
    p = gc.forcing_params("f01_gauss_static")
    rc, rf, pert, tracer, mask, perturbs = f.gaussian(0, p.Dt, 3 * p.Dt)
    assert rc == 0 and rf > 0
    g = cases.Grid(p)
    rows = g.rows()
    dlat = (g.lat1 - g.lat0) / p.ny
    s = np.array([rows["dxe"][j + 1] * dlat * g.rM(g.latn(j - 1)) for j in range(-1, p.ny + 3)])
    vol = float(np.sum(rf * pert * s[:, None]))
    assert vol == pytest.approx(p.Dt * p.gaussians[0][7], rel=1e-12)
    assert mask.sum() > 0 and np.all(perturbs[mask == 1] == 1.0) and np.all(pert[mask == 0] == 0.0)
    # inactive after t1
    assert f.gaussian(0, p.Dt, 21 * p.Dt)[0] == 1


def test_gaussian_near_the_seam_wraps(tmp_path):
    c = _case(tmp_path, "f02_gauss_moving_tracer")
    p = gc.forcing_params("f02_gauss_moving_tracer")
    rc, rf, pert, tracer, mask, _ = hostlib.Forcing(c).gaussian(0, p.Dt, 10 * p.Dt)
    cols = np.nonzero(mask.any(axis=0))[0]
    assert cols.min() <= 3 and cols.max() >= p.nx  # both ends of the band: the periodic image
    assert np.all(tracer[mask == 1] > 0) and np.all(tracer[mask == 1] <= 1.0)


def test_vortex_fields(tmp_path):
    c = _case(tmp_path, "f03_vortices_wind")
    deta, du, dv = hostlib.Forcing(c).vortex(0)
    inner = (slice(2, -2), slice(2, -2))
    assert np.all(np.isfinite(deta)) and np.abs(deta[inner]).max() > 1.0
    assert np.abs(du[inner]).max() > 0 and np.abs(dv[inner]).max() > 0
    assert np.all(deta[0:2] == 0) and np.all(du[:, 0:2] == 0)  # halos untouched (the step wraps them)


def _brute_gaussian_mask(c, f, G, Dt, t):
    """The cells inside the radius by the reference's expression evaluated at
    every interior cell (perturbs.c:22-364, polar 0), with the per-row and
    per-column values the C code tabulates."""
    w = f.w
    nx, ny = c.c.nx, c.c.ny
    R = (c.c.rE + c.c.rP) / 2.0
    pi = 4.0 * math.atan(1.0)
    deg = lambda a: a * (pi / 180.0)
    t0 = G[0]
    lon, lat = deg(G[3]), deg(G[4])
    rZ = lambda la: c.c.rE / math.sqrt(1.0 + (math.tan(la) * math.tan(la)) / c.c.epsilon2)
    om = G[6] / rZ(lat) if int(G[5]) == 0 else deg(G[6])
    lon = lon + om * (t - t0)
    radius = G[10]
    if int(G[8]) == 1:
        radius = radius / 360.0 * 2 * pi * (c.c.rE + c.c.rP) / 2.0
    while lon < c.c.lon0:
        lon += (c.c.lon1 - c.c.lon0)
    while lon > c.c.lon1:
        lon -= (c.c.lon1 - c.c.lon0)
    centres = [lon]
    if (lon + radius / rZ(lat)) >= c.c.lon1:
        centres.append(lon - (c.c.lon1 - c.c.lon0))
    if (lon - radius / rZ(lat)) <= c.c.lon0:
        centres.append(lon + (c.c.lon1 - c.c.lon0))
    plat = math.atan(1.0 / c.c.epsilon2 * math.tan(lat))
    mask = np.zeros((ny + 4, nx + 4), np.uint8)
    for lc in centres:
        for j in range(1, ny + 1):
            sj, cj = w.row_sin[j], w.row_cos[j]
            for i in range(1, nx + 1):
                x = math.sin(plat) * sj + math.cos(plat) * cj * math.cos(w.col_lonc[i] - lc)
                r = R * math.acos(x) if -1.0 <= x <= 1.0 else float("nan")
                if r < radius:
                    mask[j + 1, i + 1] = 1
    return mask


@pytest.mark.parametrize("lon,lat,sigma,radius", [
    (100.0, 10.0, 2.0, 5.0),      # interior
    (1.0, -5.0, 3.0, 8.0),        # across the periodic seam (west)
    (358.5, 20.0, 3.0, 12.0),     # across the seam (east)
    (200.0, 55.0, 4.0, 15.0),     # against the northern wall
    (60.0, 0.0, 20.0, 200.0),     # radius beyond the planet: every cell
    (33.75, -27.5, 0.5, 1.0),     # small: one cell
])
def test_gaussian_skips_only_cells_outside_the_radius(tmp_path, lon, lat, sigma, radius):
    """The Gaussian evaluation skips cells that cannot lie inside the radius;
    its cells must be exactly those where the reference's distance, evaluated
    at every cell, is below the radius, and its list must match its fields."""
    p = gc.forcing_params("f01_gauss_static")
    p.gaussians = [[0.0, 20 * p.Dt, 0.0, lon, lat, 0, 0.0, 2.5e13 / p.Dt, 1, sigma, radius, 1.0]]
    path = tmp_path / "c.sw"
    formats.write_sw(str(path), p)
    c = hostlib.Case(str(path))
    f = hostlib.Forcing(c)
    for t in (3 * p.Dt, 4 * p.Dt):  # twice: the second call must clear the first's cells
        rc, rf, pert, tracer, mask, _ = f.gaussian(0, p.Dt, t)
        assert rc == 0 and rf > 0
        ref = _brute_gaussian_mask(c, f, p.gaussians[0], p.Dt, t)
        assert np.array_equal(mask, ref)
        assert np.all(pert[mask == 0] == 0.0)
        idx, cp, ct = f.cells()
        assert np.array_equal(idx, np.sort(np.nonzero(mask.ravel())[0]))
        assert np.array_equal(cp, pert.ravel()[idx]) and np.array_equal(ct, tracer.ravel()[idx])
