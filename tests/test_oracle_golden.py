"""The CPU oracle against vectors written by the reference itself.

tests/golden/make_golden.py ran the reference (built from its own sources with
a one-rank MPI stand-in) on these cases; here the C restatement must reproduce
every saved interior bit for bit, the printed ENERGY lines to their 7 digits,
and the Van Leer abort in the same step.
"""
import hashlib

import numpy as np
import pytest

from oracle import oracle as orc
from sw2_gb300 import cases
from tests import golden_cases as gc


@pytest.mark.parametrize("name", gc.array_cases())
def test_oracle_matches_reference_frames(name):
    entry, case, frames = gc.load_case(name)
    o = orc.Oracle(case.params)
    o.load(case.fields())
    every = entry["save_every"]
    energies = [o.energy()]
    for fr in frames:
        rc, bad = o.step(every)
        assert rc == 0, (rc, bad)
        for k in ("eta", "u", "v", "tracer"):
            got = o.field(k)[2:-2, 2:-2]
            assert np.array_equal(got, fr[k]), f"{k}: max|d|={np.max(np.abs(got - fr[k]))}"
        energies.append(o.energy())
    printed = entry["energy_printed"]
    printed = [printed[0]] + (printed[2:] if every > 1 else printed[1:])
    for (t, ke, ape, tot), (oke, oape, _m) in zip(printed, energies):
        assert float(f"{oke:e}") == ke
        assert float(f"{oape:e}") == ape


def test_oracle_vanleer_abort_step():
    name = "c01_vanleer_nan"
    entry = gc.manifest()[name]
    p = gc.params_of(entry)
    z = np.load(f"{gc.GOLDEN}/{name}.npz")
    f = [gc.padded(z["init_" + k]) for k in ("eta", "u", "v", "tracer")]
    zero = np.zeros_like(f[0])
    o = orc.Oracle(p)
    o.load(f + [zero, zero, zero])
    rc, bad = o.step(entry["nsteps"])
    assert rc == 2 and bad + 1 == entry["abort_step"]


@pytest.mark.slow
def test_oracle_band256_500_steps_hash():
    """The 256x128 minmod configuration, 500 steps, against the reference's final frame."""
    entry = gc.manifest()["h01_band256"]
    case = cases.make_case(**entry["make_case"])
    for k, h in entry["init_sha256"].items():
        assert hashlib.sha256(np.ascontiguousarray(getattr(case, k)[2:-2, 2:-2]).tobytes()).hexdigest() == h
    o = orc.Oracle(case.params)
    o.load(case.fields())
    rc, bad = o.step(entry["nsteps"])
    assert rc == 0
    for k, h in entry["sha256"].items():
        got = np.ascontiguousarray(o.field(k)[2:-2, 2:-2])
        assert hashlib.sha256(got.tobytes()).hexdigest() == h, k


def test_halo_wrap_matches_oracle():
    rng = np.random.default_rng(3)
    for nx, ny in ((3, 3), (5, 4), (17, 9)):
        a = rng.standard_normal((ny + 4, nx + 4))
        b = a.copy()
        cases.halo_wrap(a)
        orc.lib().sw2o_halo_update(nx, ny, orc._ptr(b))
        assert np.array_equal(a, b)
