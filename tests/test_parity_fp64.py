"""Parity of the FP64 CUDA step (through the C ABI) with the reference.

Bar: bit-identical. Every padded cell of eta, u, v and tracer (halos included)
must equal the CPU oracle's, and the interiors must equal the frames the
reference itself wrote (tests/golden). Energy diagnostics use compensated
sums instead of the reference's sequential ones: relative tolerance 1e-12.
"""
import dataclasses
import hashlib

import numpy as np
import pytest

from oracle import oracle as orc
from sw2_gb300 import cases, lib
from tests import golden_cases as gc

pytestmark = pytest.mark.gpu

FIELDS = ("eta", "u", "v", "tracer")


def same(a, b):
    """Bitwise-equal up to the sign of zero (NaNs equal to NaNs)."""
    return np.array_equal(a, b, equal_nan=True)


def run_both(case, nsteps, flags=0, chunk=None):
    s = lib.Solver(case.params, flags=flags)
    s.upload(*case.fields(), mode=lib.UPLOAD_FRAME)
    o = orc.Oracle(case.params)
    o.load(case.fields())
    chunk = chunk or nsteps
    done = 0
    while done < nsteps:
        n = min(chunk, nsteps - done)
        assert s.step(n) == lib.OK
        rc, bad = o.step(n)
        assert rc == 0, (rc, bad)
        done += n
    return s, o


@pytest.mark.parametrize("name", gc.array_cases())
def test_gpu_matches_reference_frames(name):
    entry, case, frames = gc.load_case(name)
    s = lib.Solver(case.params)
    s.upload(*case.fields(), mode=lib.UPLOAD_FRAME)
    for fr in frames:
        assert s.step(entry["save_every"]) == lib.OK
        got = s.download()
        for k in FIELDS:
            g = got[k][2:-2, 2:-2]
            assert np.array_equal(g, fr[k]), f"{k}: max|d|={np.max(np.abs(g - fr[k]))}"


@pytest.mark.parametrize("name", gc.polar_cases())
def test_gpu_polar_caps_match_reference_frames(name):
    """Polar caps (2-D gravity, Coriolis and sponge fields, turned winds, no
    walls) against the reference's own frames, bit for bit, and its ENERGY
    lines to their printed digits."""
    entry, case, frames = gc.load_case(name)
    s = lib.Solver(case.params)
    s.upload(*case.fields(), mode=lib.UPLOAD_FRAME)
    energies = [s.diag()]
    for fr in frames:
        assert s.step(entry["save_every"]) == lib.OK
        got = s.download()
        for k in FIELDS:
            g = got[k][2:-2, 2:-2]
            assert np.array_equal(g, fr[k]), f"{k}: max|d|={np.max(np.abs(g - fr[k]))}"
        energies.append(s.diag())
    printed = entry["energy_printed"]
    printed = [printed[0]] + printed[2:]
    for (t, ke, ape, tot), (gke, gape, _m) in zip(printed, energies):
        assert float(f"{gke:e}") == ke and float(f"{gape:e}") == ape


@pytest.mark.parametrize("sch", range(10))
def test_gpu_matches_oracle_all_cells(sch):
    flags = lib.FLAG_VANLEER_SAFE if sch == 3 else 0
    case = cases.make_case(nx=61, ny=29, sch=sch, seed=100 + sch, bumps=2, tracer=(sch % 2 == 0),
                           TracerDis=1e-6, Tau=2e6 if sch % 3 == 0 else 1e20)
    if sch == 3:
        pytest.skip("reference Van Leer aborts; safe variant is covered separately")
    s, o = run_both(case, 25, flags=flags, chunk=7)
    got = s.download()
    for k in FIELDS:
        assert same(got[k], o.field(k)), k


@pytest.mark.parametrize("nx,ny", [(3, 3), (4, 5), (129, 7), (257, 33)])
def test_gpu_matches_oracle_odd_sizes(nx, ny):
    case = cases.make_case(nx=nx, ny=ny, sch=1, seed=7, bumps=1, sigma_km=(8000.0, 8000.0))
    nu4 = case.params.hypernu[1]
    case.params.hypernu = (1e-3 * nu4 ** 0.5, nu4, 1e-4 * nu4 ** 1.5)
    s, o = run_both(case, 12, chunk=5)
    got = s.download()
    for k in FIELDS:
        assert same(got[k], o.field(k)), k


def test_gpu_wind_tracer():
    wind = np.stack([np.arange(-180.0, 181.0), 30 * np.cos(np.deg2rad(np.arange(-180.0, 181.0)) * 3)], axis=1)
    case = cases.make_case(nx=48, ny=20, sch=7, seed=5, wind=wind, tracer=True, TracerDis=3e-6)
    s, o = run_both(case, 20)
    got = s.download()
    for k in FIELDS:
        assert same(got[k], o.field(k)), k


def test_gpu_vanleer_aborts_where_reference_aborts():
    entry = gc.manifest()["c01_vanleer_nan"]
    p = gc.params_of(entry)
    z = np.load(f"{gc.GOLDEN}/c01_vanleer_nan.npz")
    f = [gc.padded(z["init_" + k]) for k in FIELDS]
    s = lib.Solver(p)
    s.upload(*f)
    assert s.step(entry["nsteps"]) == lib.ERR_NONFINITE
    assert s.error_step() + 1 == entry["abort_step"]
    # the safe variant runs through
    s2 = lib.Solver(p, flags=lib.FLAG_VANLEER_SAFE)
    s2.upload(*f)
    assert s2.step(entry["nsteps"]) == lib.OK
    assert all(np.isfinite(a).all() for a in s2.download().values())


def test_gpu_cfl_abort_step_matches_oracle():
    case = cases.make_case(nx=40, ny=20, sch=2, seed=22, cfl=0.4, nsteps=200)
    s = lib.Solver(case.params)
    s.upload(*case.fields())
    o = orc.Oracle(case.params)
    o.load(case.fields())
    rc, bad = o.step(200)
    assert rc == 1
    assert s.step(200) == lib.ERR_CFL
    assert s.error_step() == bad
    # an oversized Dt fails on the first step
    case.params.Dt *= 100
    s3 = lib.Solver(case.params)
    s3.upload(*case.fields())
    assert s3.step(3) == lib.ERR_CFL and s3.error_step() == 0


@pytest.mark.parametrize("plant", ["nan_u", "nan_v_first", "nan_eta_first", "inf_v", "big_eta", "negzero"])
def test_gpu_nonfinite_values_follow_the_reference_checks(plant):
    """The CFL maxima skip NaNs and keep infinities (calc.c:705-712); the range
    check aborts on a non-finite first value or a value beyond 1e10 and is
    blind to later NaNs (sppde_core.c:346-395). Planted values must give the
    oracle's status, abort step and fields."""
    case = cases.make_case(nx=40, ny=20, sch=2, seed=23)
    f = list(case.fields())
    names = ("eta", "u", "v")
    where = {"nan_u": (1, 9, 5, np.nan), "nan_v_first": (2, 0, 0, np.nan), "nan_eta_first": (0, 0, 0, np.nan),
             "inf_v": (2, 13, 4, np.inf), "big_eta": (0, 20, 10, 2e10), "negzero": (1, 7, 3, -0.0)}[plant]
    k, i, j, val = where
    arr = f[k].copy()
    arr[j + 2, i + 2] = val
    f[k] = arr
    s = lib.Solver(case.params)
    s.upload(*f, mode=lib.UPLOAD_FRAME)
    o = orc.Oracle(case.params)
    o.load(f)
    rc_o, bad = o.step(6)
    rc = s.step(6)
    want = {0: lib.OK, 1: lib.ERR_CFL, 2: lib.ERR_NONFINITE}[rc_o]
    assert rc == want, (names[k], rc, rc_o)
    if rc != lib.OK:
        assert s.error_step() == bad
    else:
        got = s.download()
        for q in FIELDS:
            assert same(got[q], o.field(q)), q


def test_gpu_range_check_sees_the_wall_row_after_do_channel():
    """A value beyond 1e10 that only ever reaches v on the north wall row
    (from a huge eta in the halo row above it, kept by a raw upload) is zeroed
    by do_channel before the range check runs (core.c:303-312), so the
    reference does not abort; neither may the check fused into the step."""
    case = cases.make_case(nx=40, ny=20, sch=2, seed=24)
    f = [a.copy() for a in case.fields()]
    f[0][case.params.ny + 2, 2:-2] = 1e17  # eta, halo row j = ny+1
    s = lib.Solver(case.params)
    s.upload(*f, mode=lib.UPLOAD_RAW)
    o = orc.Oracle(case.params)
    o.load(f, raw=True)
    rc_o, bad = o.step(6)
    assert rc_o == 0, bad
    assert s.step(6) == lib.OK
    got = s.download()
    for q in FIELDS:
        assert same(got[q], o.field(q)), q


def test_gpu_energy_matches_oracle():
    case = cases.make_case(nx=96, ny=48, sch=2, seed=3, bumps=3)
    s, o = run_both(case, 30)
    ke, ape, m = s.diag()
    oke, oape, om = o.energy()
    for a, b in ((ke, oke), (ape, oape), (m, om)):
        assert abs(a - b) <= 1e-12 * abs(b), (a, b)


def test_gpu_raw_upload_round_trip_and_resume():
    case = cases.make_case(nx=32, ny=16, sch=2, seed=9)
    s = lib.Solver(case.params)
    s.upload(*case.fields(), mode=lib.UPLOAD_RAW)
    back = s.download()
    for k in FIELDS:
        assert np.array_equal(back[k], getattr(case, k))
    # stepping 10 then 10 equals stepping 20 (history kept across calls)
    s.step(10)
    s.step(10)
    a = s.download()
    s2 = lib.Solver(case.params)
    s2.upload(*case.fields(), mode=lib.UPLOAD_RAW)
    s2.step(20)
    b = s2.download()
    for k in FIELDS:
        assert same(a[k], b[k])


def test_gpu_rest_state_stays_at_rest():
    case = cases.make_case(nx=64, ny=32, sch=1, seed=1, jet="none", bumps=0)
    s = lib.Solver(case.params)
    s.upload(*case.fields())
    assert s.step(50) == lib.OK
    got = s.download()
    assert np.all(got["u"] == 0) and np.all(got["v"] == 0)
    assert np.all(got["eta"][2:-2, 2:-2] == case.eta[2:-2, 2:-2])


@pytest.mark.slow
def test_gpu_band2048_matches_oracle():
    """The drop-in configuration at its stated length: 2048x1024, minmod, nu4,
    2000 steps, bit-identical to the oracle in every padded cell after 40 steps
    and after 2000, with equal energy and mass. The fields being identical, the
    sums differ only by their order: the oracle adds the 2M cells in sequence,
    as the reference does, the GPU with compensated sums, so they agree to
    relative 1e-10 (a sequential sum of 2M terms carries up to ~1e-10)."""
    case = cases.config_case("band2048")
    s, o = run_both(case, 40, chunk=20)
    got = s.download()
    for k in ("eta", "u", "v"):
        assert same(got[k], o.field(k)), k
    assert s.step(1960) == lib.OK
    rc, bad = o.step(1960)
    assert rc == 0, (rc, bad)
    got = s.download()
    for k in ("eta", "u", "v"):
        assert same(got[k], o.field(k)), k
    for g, r in zip(s.diag(), o.energy()):
        assert abs(g - r) <= 1e-10 * abs(r)


@pytest.mark.slow
def test_gpu_band256_500_steps_matches_reference_hash():
    """The 256x128 minmod configuration at its stated length (500 steps): the
    interiors of eta, u and v after the last step hash to the SHA-256 of the
    reference's own final frame, and the energy matches its printed ENERGY line."""
    entry = gc.manifest()["h01_band256"]
    case = cases.make_case(**entry["make_case"])
    for k, h in entry["init_sha256"].items():
        assert hashlib.sha256(np.ascontiguousarray(getattr(case, k)[2:-2, 2:-2]).tobytes()).hexdigest() == h
    s = lib.Solver(case.params)
    s.upload(*case.fields(), mode=lib.UPLOAD_FRAME)
    assert s.step(entry["nsteps"]) == lib.OK
    got = s.download()
    for k, h in entry["sha256"].items():
        assert hashlib.sha256(np.ascontiguousarray(got[k][2:-2, 2:-2]).tobytes()).hexdigest() == h, k
    ke, ape, _mass = s.diag()
    t, pke, pape, _tot = entry["energy_printed"][-1]
    assert float(f"{ke:e}") == pke and float(f"{ape:e}") == pape


def test_sw_struct_conventions():
    # a caller that fills the case from the reference's sw struct passes the
    # band limits in radians and sigma_dis instead of Tau: same bits
    case = cases.make_case(nx=40, ny=18, sch=2, seed=31, Tau=4e5)
    a = lib.Solver(case.params)
    a.upload(*case.fields())
    assert a.step(9) == lib.OK
    p = case.params
    q = dataclasses.replace(p, Tau=1.0 / p.Tau)
    q.lon0, q.lon1, q.lat0, q.lat1 = (cases.deg2rad(x) for x in (p.lon0, p.lon1, p.lat0, p.lat1))
    b = lib.Solver(q, flags=lib.FLAG_RADIANS | lib.FLAG_SIGMA)
    b.upload(*case.fields())
    assert b.step(9) == lib.OK
    ga, gb = a.download(), b.download()
    for k in FIELDS:
        assert same(ga[k], gb[k]), k


def test_gpu_eta_hyperviscosity_of_eta():
    """SW2G_FLAG_LAPE_ETA: the eta hyperviscosity takes eta as its source
    instead of u (the reference's calc.c:332). Bit-identical to the oracle run
    the same way, and different from the default run."""
    case = cases.make_case(nx=64, ny=32, sch=2, seed=5)
    nu4 = case.params.hypernu[1]
    case.params.hypernu = (1e-3 * nu4 ** 0.5, nu4, 1e-4 * nu4 ** 1.5)
    s = lib.Solver(case.params, flags=lib.FLAG_LAPE_ETA)
    s.upload(*case.fields(), mode=lib.UPLOAD_FRAME)
    assert s.step(30) == lib.OK
    got = s.download()
    o = orc.Oracle(case.params, lape_eta=True)
    o.load(case.fields())
    assert o.step(30) == (0, -1)
    for k in FIELDS:
        assert same(got[k], o.field(k)), k
    d = orc.Oracle(case.params)
    d.load(case.fields())
    d.step(30)
    assert not np.array_equal(got["eta"], d.field("eta"))


@pytest.mark.parametrize("winds", [False, True])
def test_gpu_checkpoint_restart_is_exact(winds):
    """A checkpoint taken mid-run and loaded into a fresh context continues bit
    for bit as the uninterrupted run (every padded cell), unlike the
    reference's frame restart, whose Euler step departs from it."""
    wind = None
    if winds:
        lat = np.arange(-180.0, 181.0)
        wind = np.stack([lat, 20 * np.cos(np.deg2rad(lat) * 3)], axis=1)
    case = cases.make_case(nx=48, ny=24, sch=1, seed=13, tracer=winds, TracerDis=2e-6, wind=wind)
    a = lib.Solver(case.params)
    a.upload(*case.fields(), mode=lib.UPLOAD_FRAME)
    assert a.step(9) == lib.OK
    buf = a.checkpoint()
    assert a.step(11) == lib.OK
    want = a.download()
    b = lib.Solver(case.params)
    b.restore(buf)
    assert b.step(11) == lib.OK
    got = b.download()
    for k in FIELDS:
        assert np.array_equal(got[k], want[k]), k
    # a frame restart (interior, Euler step) differs
    c = lib.Solver(case.params)
    first = lib.Solver(case.params)
    first.upload(*case.fields(), mode=lib.UPLOAD_FRAME)
    first.step(9)
    mid = first.download()
    c.upload(mid["eta"], mid["u"], mid["v"], mid["tracer"], *case.fields()[4:], mode=lib.UPLOAD_FRAME)
    c.step(11)
    assert not np.array_equal(c.download()["u"], want["u"])
    # a checkpoint of another grid is refused
    other = lib.Solver(cases.make_case(nx=40, ny=24, sch=1, seed=13).params)
    with pytest.raises(lib.SW2GError):
        other.restore(np.concatenate([buf[:8], np.zeros(15 * 44 * 28)]))


@pytest.mark.parametrize("orders", [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 0), (0, 1, 1)])
def test_gpu_hyperviscosity_orders_match_oracle(orders):
    """The step's kernels are specialised on which hyperviscosity orders are
    in use (and the Adams-Bashforth tails fuse them from the third step):
    every combination, with and without Tau damping, matches the oracle in
    every padded cell."""
    case = cases.make_case(nx=45, ny=22, sch=1, seed=60 + sum(k << i for i, k in enumerate(orders)),
                           Tau=3e5 if orders[0] else 1e20)
    nu4 = case.params.hypernu[1]
    scale = (1e-3 * nu4 ** 0.5, nu4, 1e-4 * nu4 ** 1.5)
    case.params.hypernu = tuple(s * k for s, k in zip(scale, orders))
    s, o = run_both(case, 14, chunk=5)
    got = s.download()
    for k in FIELDS:
        assert same(got[k], o.field(k)), k
