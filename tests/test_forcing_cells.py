"""Forcing on cell lists (sw2g_add_cells, sw2g_set_cells) through the C ABI.

A Gaussian injection touches only the cells inside its radius
(perturbs.c:333-364), so only their indices and values cross to the GPU. The
result must be bit for bit that of the whole-field calls (sw2g_add_field,
sw2g_set_field_where) with the same values on the listed cells and zero
elsewhere, including the sign of zero that the reference's loop over every
cell gives (-0.0 + 0.0 = +0.0), after the halo wrap; lists that are not
increasing or name halo cells are rejected.
"""
import numpy as np
import pytest

from sw2_gb300 import cases, lib

pytestmark = pytest.mark.gpu


def _pair(case):
    a = lib.Solver(case.params)
    b = lib.Solver(case.params)
    for s in (a, b):
        s.upload(*case.fields())
    return a, b


def test_cell_lists_match_whole_field_forcing():
    case = cases.make_case(nx=40, ny=20, sch=2, seed=5, bumps=1)
    case.eta[5, 7] = -0.0  # a negative zero off the list: the whole-grid add turns it into +0.0
    case.eta[6, 9] = -0.0  # and one on it
    a, b = _pair(case)
    W = case.params.nx + 4
    rng = np.random.default_rng(3)
    js, is_ = np.meshgrid(np.arange(3, 9), np.arange(5, 16), indexing="ij")
    cells = np.sort(((is_ + 1) + (js + 1) * W).ravel()).astype(np.int32)
    cells = np.unique(np.append(cells, (9 + 1) + (6 + 1) * W)).astype(np.int32)
    vals = rng.standard_normal(cells.size) * 10.0
    vals[::7] = 0.0
    dense = np.zeros_like(case.eta)
    dense.ravel()[cells] = vals
    mask = np.zeros(case.eta.shape, np.uint8)
    mask.ravel()[cells] = 1
    for which in (0, 1, 2):
        assert a.add_cells(which, cells, vals, 0.37) == lib.OK
        b.add_field(which, dense, 0.37)
    assert a.set_cells(3, cells, vals) == lib.OK
    b.set_field_where(3, dense, mask)
    assert a.add_cells(0, np.zeros(0, np.int32), np.zeros(0), 2.0) == lib.OK  # empty list: zeros everywhere
    b.add_field(0, np.zeros_like(dense), 2.0)
    ga, gb = a.download(), b.download()
    for k in ("eta", "u", "v", "tracer"):
        assert np.array_equal(ga[k], gb[k]) and np.array_equal(np.signbit(ga[k]), np.signbit(gb[k])), k
    # the forced fields step on identically
    assert a.step(5) == lib.OK and b.step(5) == lib.OK
    ga, gb = a.download(), b.download()
    for k in ("eta", "u", "v", "tracer"):
        assert np.array_equal(ga[k], gb[k]), k


def test_cell_lists_are_checked():
    case = cases.make_case(nx=16, ny=8, sch=2, seed=6, bumps=1)
    s = lib.Solver(case.params)
    s.upload(*case.fields())
    W = case.params.nx + 4
    q = lambda i, j: (i + 1) + (j + 1) * W
    one = np.ones(2)
    assert s.add_cells(0, [q(3, 2), q(2, 2)], one) == lib.ERR_BAD_ARG   # not increasing
    assert s.add_cells(0, [q(3, 2), q(3, 2)], one) == lib.ERR_BAD_ARG   # repeated
    assert s.add_cells(0, [q(0, 2), q(3, 2)], one) == lib.ERR_BAD_ARG   # halo column
    assert s.set_cells(3, [q(3, 0), q(3, 2)], one) == lib.ERR_BAD_ARG   # halo row
    assert s.set_cells(3, [q(3, 2), q(17, 2)], one) == lib.ERR_BAD_ARG  # beyond nx
    assert s.add_cells(4, [q(3, 2), q(4, 2)], one) == lib.ERR_BAD_ARG   # not a state field
