"""sw2g_step_host: the per-step call on the caller's own padded host arrays.

It must leave in those arrays exactly what sw2g_upload(CONTINUE) +
sw2g_step + sw2g_download leave, which the FP64 form pins to the reference
bit for bit (here against the CPU oracle and the reference's own frames),
including the Euler and AB2 start-up steps, the fused AB3 steps, multi-step
calls, a tracer that stays on the device, and a failing step.
"""
import numpy as np
import pytest

from oracle import oracle as orc
from sw2_gb300 import cases, lib
from tests import golden_cases as gc

pytestmark = pytest.mark.gpu


def same(a, b):
    return np.array_equal(a, b, equal_nan=True)


def host_arrays(case):
    return [np.ascontiguousarray(getattr(case, k), dtype=np.float64).copy() for k in ("eta", "u", "v")]


@pytest.mark.parametrize("sch,tracer,winds", [(2, False, False), (1, False, False), (7, True, False), (0, True, True)])
def test_gpu_step_host_matches_oracle_every_step(sch, tracer, winds):
    wind = None
    if winds:
        lat = np.arange(-180.0, 181.0)
        wind = np.stack([lat, 20 * np.cos(np.deg2rad(lat) * 3)], axis=1)
    case = cases.make_case(nx=61, ny=29, sch=sch, seed=40 + sch, bumps=2, tracer=tracer, TracerDis=2e-6,
                           wind=wind)
    s = lib.Solver(case.params)
    s.upload(*case.fields(), mode=lib.UPLOAD_FRAME)
    o = orc.Oracle(case.params)
    o.load(case.fields())
    # the frame upload refreshed the halos: start from the device's state
    d = s.download()
    eta, u, v = (d[k].copy() for k in ("eta", "u", "v"))
    for n in (1, 1, 1, 1, 3, 1, 5):
        assert s.step_host(eta, u, v, n) == lib.OK
        rc, bad = o.step(n)
        assert rc == 0, (rc, bad)
        for k, a in zip(("eta", "u", "v"), (eta, u, v)):
            assert same(a, o.field(k)), k
    assert same(s.download()["tracer"], o.field("tracer"))
    assert s.steps_done() == 13


@pytest.mark.parametrize("lape_eta,hyper", [(True, True), (False, False)])
def test_gpu_step_host_other_step_orders(lape_eta, hyper):
    """The eta Laplacians run first only when they read u alone: with
    SW2G_FLAG_LAPE_ETA they read eta and keep their place, and without
    hyperviscosity there are none; both still match the oracle."""
    case = cases.make_case(nx=48, ny=24, sch=2, seed=61, bumps=2, hyper=hyper)
    if hyper:
        nu4 = case.params.hypernu[1]
        case.params.hypernu = (1e-3 * nu4 ** 0.5, nu4, 1e-4 * nu4 ** 1.5)
    s = lib.Solver(case.params, flags=lib.FLAG_LAPE_ETA if lape_eta else 0)
    s.upload(*case.fields(), mode=lib.UPLOAD_FRAME)
    o = orc.Oracle(case.params, lape_eta=lape_eta)
    o.load(case.fields())
    d = s.download()
    eta, u, v = (d[k].copy() for k in ("eta", "u", "v"))
    for n in (1, 1, 2, 4):
        assert s.step_host(eta, u, v, n) == lib.OK
        assert o.step(n) == (0, -1)
        for k, a in zip(("eta", "u", "v"), (eta, u, v)):
            assert same(a, o.field(k)), k


def test_gpu_step_host_equals_upload_step_download():
    case = cases.make_case(nx=128, ny=48, sch=2, seed=3, bumps=3)
    a = lib.Solver(case.params)
    b = lib.Solver(case.params)
    for s in (a, b):
        s.upload(*case.fields(), mode=lib.UPLOAD_FRAME)
    d = a.download()
    eta, u, v = (d[k].copy() for k in ("eta", "u", "v"))
    for _ in range(6):
        assert a.step_host(eta, u, v, 1) == lib.OK
        assert b.step(1) == lib.OK
        ref = b.download()
        for k, x in zip(("eta", "u", "v"), (eta, u, v)):
            assert same(x, ref[k]), k
        # a caller may change the state between calls: it is what goes in next
        eta[5, 7] += 1e-3
        b.upload(eta, u, v, mode=lib.UPLOAD_CONTINUE)


@pytest.mark.parametrize("name", gc.polar_cases()[:1])
def test_gpu_step_host_polar_cap_matches_reference_frames(name):
    entry, case, frames = gc.load_case(name)
    s = lib.Solver(case.params)
    s.upload(*case.fields(), mode=lib.UPLOAD_FRAME)
    d = s.download()
    eta, u, v = (d[k].copy() for k in ("eta", "u", "v"))
    for fr in frames:
        assert s.step_host(eta, u, v, entry["save_every"]) == lib.OK
        for k, x in zip(("eta", "u", "v"), (eta, u, v)):
            assert np.array_equal(x[2:-2, 2:-2], fr[k]), k


def test_gpu_step_host_failure_returns_the_state():
    case = cases.make_case(nx=40, ny=20, sch=2, seed=22)
    case.params.Dt *= 100
    s = lib.Solver(case.params)
    s.upload(*case.fields())
    eta, u, v = host_arrays(case)
    assert s.step_host(eta, u, v, 3) == lib.ERR_CFL
    assert s.error_step() == 0
    d = s.download()
    for k, x in zip(("eta", "u", "v"), (eta, u, v)):
        assert same(x, d[k]), k


def test_gpu_step_host_fp32_form_matches_its_sequence():
    case = cases.make_case(nx=96, ny=40, sch=2, seed=12, bumps=2)
    a = lib.Solver(case.params, precision=lib.FP32)
    b = lib.Solver(case.params, precision=lib.FP32)
    for s in (a, b):
        s.upload(*case.fields(), mode=lib.UPLOAD_FRAME)
    d = a.download()
    eta, u, v = (d[k].copy() for k in ("eta", "u", "v"))
    for _ in range(4):
        assert a.step_host(eta, u, v, 2) == lib.OK
        b.upload(*(d[k] for k in ("eta", "u", "v")), mode=lib.UPLOAD_CONTINUE)
        assert b.step(2) == lib.OK
        d = b.download()
        for k, x in zip(("eta", "u", "v"), (eta, u, v)):
            assert same(x, d[k]), k


def test_gpu_step_host_arguments():
    case = cases.make_case(nx=16, ny=8, sch=2, seed=1)
    s = lib.Solver(case.params)
    eta, u, v = host_arrays(case)
    with pytest.raises(lib.SW2GError) as e:
        s.step_host(eta, u, v, 1)  # no upload yet
    assert e.value.code == lib.ERR_STATE
    s.upload(*case.fields())
    with pytest.raises(ValueError):
        s.step_host(eta[:, :-1], u, v, 1)
    with pytest.raises(ValueError):
        s.step_host(eta.astype(np.float32), u, v, 1)
    with pytest.raises(lib.SW2GError) as e:
        s.step_host(eta, u, v, 0)
    assert e.value.code == lib.ERR_BAD_ARG
