"""The reference built with its time loop on the GPU.

oracle/Makefile (target binding) compiles the reference's own sources where
they lie, its core.c with loop() renamed loop_cpu, and links them with
sw2_gb300/binding/sw2g_loop.c, which defines loop() on top of libsw2g.so
through include/sw2g.h only: a drop-in at the reference's seam (core.c:22,
sw.h:223). On the CPU: the binary builds against the reference's sw struct,
links the library, defines both loops, and its CPU path (SW2G_CPU=1) still
writes the reference's frames. With a GPU (where the reference's sources are
present to build it): the GPU path writes the reference's frames bit for bit
and its ENERGY lines to their printed digits. Skipped without the
reference's sources.
"""
import os
import subprocess

import numpy as np
import pytest

from sw2_gb300 import build, formats
from tests import golden_cases as gc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIN = os.path.join(ROOT, "oracle", "_ref", "SW_sw2g")
M4 = os.path.join(ROOT, "oracle", "_ref", "bin")


@pytest.fixture(scope="module")
def binary():
    build.build()
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", "binding"], capture_output=True,
                       text=True)
    if not os.path.exists(BIN):
        pytest.skip("the reference's sources are not present: the binding cannot be built (" +
                    (r.stdout + r.stderr).strip()[-200:] + ")")
    return BIN


def run_restart(binary, tmp_path, name, env_extra):
    entry, case, ref = gc.load_case(name)
    p = case.params
    p.LoadFrom, p.IteInfo = 1, entry["save_every"]
    p.SaveEvery, p.nsteps = entry["save_every"], entry["nsteps"]
    formats.write_sw(str(tmp_path / f"{name}.sw"), p)
    os.makedirs(tmp_path / "out")
    z = np.zeros_like(case.eta)
    fr = [np.zeros_like(case.eta) for _ in range(4)]
    for dst, src in zip(fr, (case.eta, case.u, case.v, case.tracer)):
        dst[2:-2, 2:-2] = src[2:-2, 2:-2]
    formats.write_frame(str(tmp_path / "out" / f"{name}.0001.bin"), 0, 0.0, p.nx, p.ny, fr + [z])
    env = dict(os.environ, PATH=M4 + os.pathsep + os.environ["PATH"], **env_extra)
    r = subprocess.run([binary, "1", "1", name, "out"], cwd=tmp_path, env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0 and "CRASH" not in r.stdout + r.stderr, (r.stdout[-1500:], r.stderr[-1500:])
    energy = [ln.split(None, 1)[1].strip() for ln in r.stdout.splitlines() if ln.startswith("ENERGY")]
    for k, rf in enumerate(ref):
        nstep, t, nx, ny, fl = formats.read_frame(str(tmp_path / "out" / f"{name}.{k + 2:04d}.bin"))
        for f in ("eta", "u", "v", "tracer"):
            assert np.array_equal(fl[f][2:-2, 2:-2], rf[f]), f"frame {k + 2} {f}"
    return entry, energy


def test_binding_links_the_library_and_keeps_both_loops(binary):
    syms = subprocess.run(["nm", binary], capture_output=True, text=True).stdout
    assert " T loop\n" in syms and " T loop_cpu\n" in syms
    assert "libsw2g.so" in subprocess.run(["ldd", binary], capture_output=True, text=True).stdout


def test_binding_cpu_path_writes_the_reference_frames(binary, tmp_path):
    run_restart(binary, tmp_path, "g01_minmod_nu4", {"SW2G_CPU": "1"})


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["g01_minmod_nu4", "g11_wind_tracer"])
def test_binding_gpu_path_writes_the_reference_frames(binary, tmp_path, name):
    entry, energy = run_restart(binary, tmp_path, name, {})
    printed = entry["energy_printed"]
    assert len(energy) == len(printed)
    for a, b in zip(energy, printed):
        va, vb = [float(x) for x in a.split()], b
        assert va[0] == vb[0] and all(abs(x - y) <= 1.5e-6 * abs(y) for x, y in zip(va[1:], vb[1:])), (a, b)
