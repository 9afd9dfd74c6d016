"""Batched ensembles of FP32-form members (sw2g_batch_*).

A batch runs the same kernels over all members' tiles in one launch per phase
and replays a captured one-step CUDA graph, so each member must end bit for
bit where it ends when stepped alone; the sweep-schedule tuner only reorders
independent blocks, so tuning must not change any result either.
"""
import numpy as np
import pytest

from sw2_gb300 import cases, lib

pytestmark = pytest.mark.gpu


def members(seed=3):
    specs = [(64, 32, 1), (97, 40, 2), (128, 64, 3)]
    out = []
    for nx, ny, k in specs:
        c = cases.make_case(nx=nx, ny=ny, sch=3, seed=seed * 10 + k, bumps=1, amp=(0.01, 0.08),
                            sigma_km=(1000.0, 3000.0))
        out.append(c)
    return out


def solo(case, n):
    s = lib.Solver(case.params, precision=lib.FP32, flags=lib.FLAG_VANLEER_SAFE)
    s.upload(*case.fields())
    assert s.step(n) == lib.OK
    return s.download()


def test_batch_matches_members_stepped_alone():
    cs = members()
    ss = []
    for c in cs:
        s = lib.Solver(c.params, precision=lib.FP32, flags=lib.FLAG_VANLEER_SAFE)
        s.upload(*c.fields())
        ss.append(s)
    b = lib.Batch(ss)
    assert b.step(7) == lib.OK
    assert b.step(9) == lib.OK
    assert b.last_launches() == 4 * 9
    for c, s in zip(cs, ss):
        got, ref = s.download(), solo(c, 16)
        for k in ("eta", "u", "v"):
            assert np.array_equal(got[k], ref[k]), k
        assert s.steps_done() == 16


def test_tuning_changes_no_result():
    cs = members(seed=5)
    ss = []
    for c in cs:
        s = lib.Solver(c.params, precision=lib.FP32, flags=lib.FLAG_VANLEER_SAFE)
        s.upload(*c.fields())
        ss.append(s)
    b = lib.Batch(ss)
    times = b.tune(3)
    assert len(times) == len(lib.Batch.TILE_ROWS) * len(lib.Batch.SCHEDULES)
    assert all(t > 0 for t in times.values())
    assert b.schedule() in lib.Batch.SCHEDULES and b.tile_rows() in lib.Batch.TILE_ROWS
    assert b.step(4) == lib.OK
    # 12 candidates x 3 steps, one untimed step per shape, and 4 more
    n = 12 * 3 + 3 + 4
    for c, s in zip(cs, ss):
        got, ref = s.download(), solo(c, n)
        for k in ("eta", "u", "v"):
            assert np.array_equal(got[k], ref[k]), k


@pytest.mark.parametrize("tile_rows", lib.Batch.TILE_ROWS)
def test_every_tile_shape_gives_the_same_bits(tile_rows):
    """Each face is computed with the same operations wherever it is
    evaluated (carried down a strip or recomputed at a strip's first row), so
    every strip height and schedule, also changed between steps, ends where
    the member stepped alone ends."""
    cs = members(seed=9)
    ss = []
    for c in cs:
        s = lib.Solver(c.params, precision=lib.FP32, flags=lib.FLAG_VANLEER_SAFE)
        s.upload(*c.fields())
        ss.append(s)
    b = lib.Batch(ss)
    b.set_schedule(tile_rows, "columns")
    assert b.step(5) == lib.OK
    b.set_schedule(lib.Batch.TILE_ROWS[(lib.Batch.TILE_ROWS.index(tile_rows) + 1) % 3], "interleaved")
    assert b.step(6) == lib.OK
    for c, s in zip(cs, ss):
        got, ref = s.download(), solo(c, 11)
        for k in ("eta", "u", "v"):
            assert np.array_equal(got[k], ref[k]), k


def test_batch_reports_the_failing_member():
    cs = members(seed=7)
    cs[1].params.Dt *= 100  # violates the CFL bound at the first step
    ss = []
    for c in cs:
        s = lib.Solver(c.params, precision=lib.FP32, flags=lib.FLAG_VANLEER_SAFE)
        s.upload(*c.fields())
        ss.append(s)
    b = lib.Batch(ss)
    assert b.step(5) == lib.ERR_CFL
    assert b.error() == (1, 0)
    assert ss[1].error_step() == 0


def test_graph_replay_equals_direct_launches():
    c = members(seed=9)[2]
    a = lib.Solver(c.params, precision=lib.FP32, flags=lib.FLAG_VANLEER_SAFE)
    a.upload(*c.fields())
    a.timers(True)  # per-kernel timers force direct launches
    assert a.step(11) == lib.OK
    assert set(a.timer_table()) == {"f32_lap1", "f32_main1", "f32_main2"}
    ref = solo(c, 11)
    got = a.download()
    for k in ("eta", "u", "v"):
        assert np.array_equal(got[k], ref[k]), k


def test_batch_rejects_mixed_members():
    c = members()[0]
    s64 = lib.Solver(c.params, precision=lib.FP64)
    s64.upload(*c.fields())
    s32 = lib.Solver(c.params, precision=lib.FP32, flags=lib.FLAG_VANLEER_SAFE)
    s32.upload(*c.fields())
    with pytest.raises(lib.SW2GError):
        lib.Batch([s32, s64])
    with pytest.raises(lib.SW2GError):
        lib.Batch([s32, s32])


def test_polar_cap_members_step_alone():
    """A polar cap's FP32 kernels read per-cell cap factors and are built for
    one member: a cap batches alone, bit for bit as stepped by itself, and a
    batch that mixes it with other members is refused."""
    from tests import golden_cases as gc

    entry, case, _ = gc.load_case("p02_south_superbee_tracer")

    def cap():
        s = lib.Solver(case.params, precision=lib.FP32)
        s.upload(*case.fields(), mode=lib.UPLOAD_FRAME)
        return s

    a, b = cap(), cap()
    with pytest.raises(lib.SW2GError):
        lib.Batch([a, fresh(members()[0])])
    bt = lib.Batch([a])
    assert bt.step(6) == lib.OK
    assert b.step(6) == lib.OK
    ga, gb = a.download(), b.download()
    for k in ("eta", "u", "v", "tracer"):
        assert np.array_equal(ga[k], gb[k]), k


def fresh(c):
    s = lib.Solver(c.params, precision=lib.FP32, flags=lib.FLAG_VANLEER_SAFE)
    s.upload(*c.fields())
    return s


def test_members_stepped_alone_between_batch_steps():
    # a member stepped through its own context (or re-uploaded) between batch
    # steps must be picked up where it is, not where the batch left it
    cs = members(seed=11)
    ss = [fresh(c) for c in cs]
    b = lib.Batch(ss)
    assert b.step(4) == lib.OK
    assert ss[0].step(3) == lib.OK
    ss[1].upload(*cs[1].fields())
    assert b.step(5) == lib.OK
    expect = [solo(cs[0], 12), solo(cs[1], 5), solo(cs[2], 9)]
    for s, ref in zip(ss, expect):
        got = s.download()
        for k in ("eta", "u", "v"):
            assert np.array_equal(got[k], ref[k]), k


def test_large_batch():
    # more than 16 members: the widest descriptor set of the launch
    cs = [cases.make_case(nx=40 + 8 * (k % 3), ny=16 + 8 * (k % 2), sch=3, seed=100 + k, bumps=1,
                          amp=(0.01, 0.08), sigma_km=(1000.0, 3000.0)) for k in range(20)]
    ss = [fresh(c) for c in cs]
    b = lib.Batch(ss)
    assert b.step(6) == lib.OK
    for k in (0, 7, 19):
        got, ref = ss[k].download(), solo(cs[k], 6)
        for f in ("eta", "u", "v"):
            assert np.array_equal(got[f], ref[f]), (k, f)


def test_check_slots_wrap():
    # per-step checks live in a ring of 1024 slots on the device: runs that
    # cross the end of the ring give the same state and still catch a failure
    c = members(seed=13)[0]
    a, one = fresh(c), fresh(c)
    assert a.step(1000) == lib.OK
    assert a.step(30) == lib.OK
    assert one.step(1030) == lib.OK
    ga, go = a.download(), one.download()
    for k in ("eta", "u", "v"):
        assert np.array_equal(ga[k], go[k]), k
    # a state far beyond the CFL bound, continued from step 1030 (slot 6 of the ring)
    a.upload(ga["eta"], ga["u"] * 1e3, ga["v"], mode=lib.UPLOAD_CONTINUE)
    assert a.step(5) == lib.ERR_CFL
    assert a.error_step() == 1030
