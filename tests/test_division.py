"""The FP64 step divides by row metric factors (DXE, DYN, DXC, DYV, ...)
with multiplications and fused multiply-adds using each factor's correctly
rounded reciprocal (Markstein's method). Its quotients must equal IEEE
division bit for bit; the library's self-check draws random numerators and
numerators whose quotient lies next to a rounding midpoint. The same holds
for the additions the step computes on the integer pipe."""
import numpy as np
import pytest

from sw2_gb300 import cases, lib

pytestmark = pytest.mark.gpu


def metric_factors(name):
    p = cases.config_case(name, seed=1).params
    g = cases.Grid(p)
    dlon = (g.lon1 - g.lon0) / float(p.nx)
    dlat = (g.lat1 - g.lat0) / float(p.ny)
    out = []
    for j in range(-1, p.ny + 3):
        lc, ln, ln1 = g.latc(j), g.latn(j), g.latn(j - 1)
        dxe, dyn = dlon * g.rZ(lc), dlat * g.rM(lc)
        out += [dxe, dlon * g.rZ(ln), dyn, dlat * g.rM(ln1), dxe + dxe, g.rZ(lc), g.rZ(ln)]
    return np.array(out)


def test_metric_division_matches_ieee():
    d = np.concatenate([metric_factors("band256")])
    assert lib.selfcheck_division(d, samples=100_000, seed=11) == 0


def test_random_divisors_match_ieee():
    rng = np.random.default_rng(5)
    d = np.ldexp(rng.uniform(1.0, 2.0, 20_000), rng.integers(-30, 60, 20_000))
    # significands with all-ones tails and powers of two
    d = np.concatenate([d, np.nextafter(np.ldexp(1.0, np.arange(-20, 40)), 0), np.ldexp(1.0, np.arange(-20, 40))])
    assert lib.selfcheck_division(d, samples=5_000, seed=12) == 0


def test_divisors_near_powers_of_two_match_ieee():
    """The one-correction quotient RN(q0 + (a - b q0) y), q0 = RN(a y), can
    start more than one ulp off only when a's and b's significands are both
    within a few ulps of 2: every divisor within 512 ulps below 2 (and just
    above 1, and scaled by powers of two) against every numerator within 512
    ulps below 2 of either sign (the self-check's grid), plus random and
    near-midpoint numerators."""
    below2 = np.arange(0x3FFFFFFFFFFFFFFF - 511, 0x3FFFFFFFFFFFFFFF + 1, dtype=np.uint64).view(np.float64)
    above1 = np.arange(0x3FF0000000000000, 0x3FF0000000000000 + 512, dtype=np.uint64).view(np.float64)
    d = np.concatenate([below2, above1, np.ldexp(below2, -20), np.ldexp(below2, 37), np.ldexp(above1, 11)])
    assert lib.selfcheck_division(d, samples=2_000, seed=13) == 0


def test_integer_pipe_addition_matches_the_fp64_unit():
    """The step's additions on the integer pipe (sadd, ssub) against the FP64
    unit: 2^27 operand pairs per seed over the adder's edge cases."""
    for seed in (21, 22, 23):
        assert lib.selfcheck_add(samples=1 << 27, seed=seed) == 0
