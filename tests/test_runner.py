"""The case-file runner (sw2g-run: C front end + GPU step) against runs of
the reference executable on the same case files (tests/golden):

* forcing cases (f*): the reference starts from its own initial state
  (zero fields, zonal wind, forcing at t0, frame 0) and injects Gaussians
  and vortices during the run; every field of every frame must be bit for bit
  the reference's, and the ENERGY lines equal to their printed digits;
* restart cases (g* bands, p* polar caps): the reference loads frame 1
  (LoadFrom 1) and saves the following frames; the runner must reproduce them
  bit for bit;
* the reference's own example (examples/JupiterEnergyTest, 34,560 steps) gives
  the reference's ENERGY lines and last frame, and its known-answer file
  (enou.txt, from an older version of the code) is met within the reference's
  own agreement;
* the FP32 form runs a case file within tolerance of the FP64 step.
"""
import hashlib
import os
import shutil
import subprocess

import numpy as np
import pytest

from sw2_gb300 import formats, hostlib
from tests import golden_cases as gc

pytestmark = pytest.mark.gpu


def run(workdir, name, args=(), flags=()):
    r = subprocess.run([hostlib.RUNNER, "--quiet", *flags, *args, "1", "1", name, "out"], cwd=workdir,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    energy = [ln.split(None, 1)[1].strip() for ln in r.stdout.splitlines() if ln.startswith("ENERGY")]
    frames = {}
    pre, post = f"{name}.", ".bin"
    for fn in os.listdir(os.path.join(workdir, "out")):
        if fn.startswith(pre) and fn.endswith(post) and fn[len(pre):-len(post)].isdigit():
            frames[int(fn[len(pre):-len(post)])] = formats.read_frame(os.path.join(workdir, "out", fn))
    return energy, frames


def same_energy(a, b, rel=1.5e-6):
    va, vb = [float(x) for x in a.split()], [float(x) for x in b.split()]
    return va[0] == vb[0] and all(abs(x - y) <= rel * abs(y) for x, y in zip(va[1:], vb[1:]))


FULL = [n for n in gc.forcing_cases() if "last_frame" not in gc.manifest()[n]]
HASHED = [n for n in gc.forcing_cases() if "last_frame" in gc.manifest()[n]]


@pytest.mark.parametrize("name", FULL)
def test_forcing_cases_match_the_reference(tmp_path, name):
    p = gc.forcing_params(name)
    formats.write_sw(str(tmp_path / f"{name}.sw"), p)
    energy, frames = run(tmp_path, name)
    ref = gc.forcing_frames(name)
    assert sorted(frames) == list(range(len(ref)))
    for k, rf in enumerate(ref):
        nstep, t, nx, ny, fl = frames[k]
        assert t == float(rf["t"]), (k, t, float(rf["t"]))
        for f in ("eta", "u", "v", "tracer", "perturbs"):
            d = np.max(np.abs(fl[f] - rf[f]))
            assert np.array_equal(fl[f], rf[f]), f"frame {k} {f}: max|d|={d}"
    printed = gc.manifest()[name]["energy_printed"]
    assert len(energy) == len(printed)
    for a, b in zip(energy, printed):
        assert same_energy(a, b), (a, b)


@pytest.mark.parametrize("name", FULL)
def test_device_forcing_matches_the_reference_within_rounding(tmp_path, name):
    """--device-forcing: the Gaussians' fields, injected volume and rescale
    evaluated on the GPU (sw2g_add_gaussian). Every padded cell of every frame
    within 1e-12 of the field's largest magnitude of the reference's (the GPU's
    cos, acos and exp and the order of the volume sum differ in the last bits),
    PERTURBS and the times exact, and the ENERGY lines equal to their printed
    digits."""
    p = gc.forcing_params(name)
    formats.write_sw(str(tmp_path / f"{name}.sw"), p)
    energy, frames = run(tmp_path, name, flags=("--device-forcing",))
    ref = gc.forcing_frames(name)
    assert sorted(frames) == list(range(len(ref)))
    for k, rf in enumerate(ref):
        nstep, t, nx, ny, fl = frames[k]
        assert t == float(rf["t"])
        assert np.array_equal(fl["perturbs"], rf["perturbs"]), k
        for f in ("eta", "u", "v", "tracer"):
            scale = max(float(np.max(np.abs(rf[f]))), 1e-300)
            assert np.max(np.abs(fl[f] - rf[f])) <= 1e-12 * scale, (k, f)
    printed = gc.manifest()[name]["energy_printed"]
    assert len(energy) == len(printed)
    for a, b in zip(energy, printed):
        assert same_energy(a, b), (a, b)


def test_device_forcing_in_the_fp32_form(tmp_path):
    """--fp32 --device-forcing on the moving Gaussian with tracer injection:
    the FP32 form's tolerance of the reference's frames, as with the host
    evaluation (h relative L2 <= 1e-5, tracer within 1e-3 of its largest
    magnitude), PERTURBS exact."""
    name = "f02_gauss_moving_tracer"
    p = gc.forcing_params(name)
    formats.write_sw(str(tmp_path / f"{name}.sw"), p)
    _, frames = run(tmp_path, name, flags=("--fp32", "--device-forcing"))
    ref = gc.forcing_frames(name)
    assert sorted(frames) == list(range(len(ref)))
    inner = (slice(2, -2), slice(2, -2))
    for k, rf in enumerate(ref):
        fl = frames[k][4]
        assert np.array_equal(fl["perturbs"], rf["perturbs"]), k
        h = rf["eta"][inner] + p.depth
        assert np.linalg.norm((fl["eta"] - rf["eta"])[inner]) <= 1e-5 * np.linalg.norm(h), k
        tr = max(float(np.max(np.abs(rf["tracer"]))), 1e-300)
        assert np.max(np.abs(fl["tracer"] - rf["tracer"])) <= 1e-3 * tr, k


@pytest.mark.parametrize("name", HASHED)
def test_reference_example_run(tmp_path, name):
    """Runs kept as hashes: the reference's examples/JupiterEnergyTest case,
    all 34,560 steps (every ENERGY line as printed), and a 1024x512 band with
    three Gaussians injected every step, whose cells inside the radii reach the
    GPU as lists (ENERGY lines to their printed digits: sums over 0.5 M cells
    in another order). The last frame must be the reference's bit for bit."""
    entry = gc.manifest()[name]
    formats.write_sw(str(tmp_path / f"{name}.sw"), gc.forcing_params(name))
    energy, frames = run(tmp_path, name)
    if name == "f05_jupiter_example":
        assert energy == entry["energy_printed"]
    else:
        assert len(energy) == len(entry["energy_printed"])
        for a, b in zip(energy, entry["energy_printed"]):
            assert same_energy(a, b), (a, b)
    assert len(frames) == entry["frames"]
    nstep, t, nx, ny, fl = frames[max(frames)]
    assert t == entry["last_frame"]["t"]
    for k, h in entry["last_frame"]["sha256"].items():
        assert hashlib.sha256(np.ascontiguousarray(fl[k]).tobytes()).hexdigest() == h, k


@pytest.mark.parametrize("name", ["g01_minmod_nu4", "g11_wind_tracer", "g13_saturn_superbee"] + gc.polar_cases())
def test_restart_cases_match_the_reference(tmp_path, name):
    entry, case, ref = gc.load_case(name)
    p = case.params
    p.LoadFrom = 1
    formats.write_sw(str(tmp_path / f"{name}.sw"), p)
    os.makedirs(tmp_path / "out")
    z = np.zeros_like(case.eta)
    fr = [np.zeros_like(case.eta) for _ in range(4)]
    for dst, src in zip(fr, (case.eta, case.u, case.v, case.tracer)):
        dst[2:-2, 2:-2] = src[2:-2, 2:-2]
    formats.write_frame(str(tmp_path / "out" / f"{name}.0001.bin"), 0, 0.0, p.nx, p.ny, fr + [z])
    energy, frames = run(tmp_path, name)
    assert sorted(k for k in frames if k >= 2) == list(range(2, 2 + len(ref)))
    for k, rf in enumerate(ref):
        fl = frames[k + 2][4]
        for f in ("eta", "u", "v", "tracer"):
            assert np.array_equal(fl[f][2:-2, 2:-2], rf[f]), f"frame {k + 2} {f}"
    printed = entry["energy_printed"]
    assert len(energy) == len(printed)
    for a, b in zip(energy, printed):
        assert same_energy(a, "%e %e %e %e" % tuple(b)), (a, b)


def test_fp32_form_runs_a_polar_cap(tmp_path):
    """The south cap (superbee, tracer, nu2+nu4+nu6) from its LoadFrom frame
    through the runner in the FP32 form: every saved frame within the FP32
    form's tolerance of the reference's frames (eta within 2e-6 of the depth,
    u, v and the tracer within 2e-4 of the field's largest magnitude)."""
    name = "p02_south_superbee_tracer"
    entry, case, ref = gc.load_case(name)
    p = case.params
    p.LoadFrom = 1
    formats.write_sw(str(tmp_path / f"{name}.sw"), p)
    os.makedirs(tmp_path / "out")
    z = np.zeros_like(case.eta)
    fr = [np.zeros_like(case.eta) for _ in range(4)]
    for dst, src in zip(fr, (case.eta, case.u, case.v, case.tracer)):
        dst[2:-2, 2:-2] = src[2:-2, 2:-2]
    formats.write_frame(str(tmp_path / "out" / f"{name}.0001.bin"), 0, 0.0, p.nx, p.ny, fr + [z])
    _, frames = run(tmp_path, name, flags=("--fp32",))
    assert sorted(k for k in frames if k >= 2) == list(range(2, 2 + len(ref)))
    for k, rf in enumerate(ref):
        fl = frames[k + 2][4]
        assert np.max(np.abs(fl["eta"][2:-2, 2:-2] - rf["eta"])) <= 2e-6 * p.depth, k
        for f in ("u", "v", "tracer"):
            scale = float(np.max(np.abs(rf[f])))
            assert np.max(np.abs(fl[f][2:-2, 2:-2] - rf[f])) <= 2e-4 * scale, (k, f)


def test_checkpoint_resume_continues_exactly(tmp_path):
    """--checkpoint writes an exact-restart file beside each frame; --resume F
    continues from it and writes the uninterrupted run's later frames bit for
    bit (with its Gaussian injections and vortices on the way)."""
    name = FULL[-1]
    p = gc.forcing_params(name)
    a, b = tmp_path / "a", tmp_path / "b"
    for d in (a, b):
        os.makedirs(d / "out")
        formats.write_sw(str(d / f"{name}.sw"), p)
    _, full = run(a, name, flags=("--checkpoint",))
    last = max(full)
    assert last >= 3
    k = last // 2
    shutil.copy(a / "out" / f"{name}.{k:04d}.ckp", b / "out")
    _, tail = run(b, name, flags=("--resume", str(k)))
    assert sorted(tail) == list(range(k + 1, last + 1))
    for q in tail:
        assert tail[q][:2] == full[q][:2]
        for f in ("eta", "u", "v", "tracer", "perturbs"):
            assert np.array_equal(tail[q][4][f], full[q][4][f]), (q, f)


def test_known_answer_file(tmp_path):
    name = "f04_jupiter_box"
    formats.write_sw(str(tmp_path / f"{name}.sw"), gc.forcing_params(name))
    energy, _ = run(tmp_path, name)
    kat = gc.manifest()["kat_enou"]["energy_printed"]
    assert len(energy) >= len(kat)
    for a, b in zip(energy, kat):
        t, ke, ape, tot = (float(x) for x in a.split())
        tk, kek, apek, totk = (float(x) for x in b.split())
        assert t == tk
        assert abs(ke - kek) <= 5.5e-4 * abs(kek)
        assert abs(tot - totk) <= 2.0e-5 * abs(totk)


@pytest.mark.parametrize("name", ["g12_minmod_long", "g11_wind_tracer", "g02_superbee_nu246"])
def test_fp32_form_runs_a_case_file(tmp_path, name):
    """A case file run from its LoadFrom frame by the runner in both forms (a
    long minmod run; winds with a tracer; nu2+nu4+nu6): the FP32 form's last
    frame within its tolerance of the FP64 form's (h relative L2 <= 1e-6
    over the interior, the tracer within 1e-4 of its largest magnitude)."""
    entry, case, ref = gc.load_case(name)
    p = case.params
    p.LoadFrom = 1
    for sub in ("a", "b"):
        d = tmp_path / sub
        os.makedirs(d / "out")
        formats.write_sw(str(d / f"{name}.sw"), p)
        z = np.zeros_like(case.eta)
        fr = [np.zeros_like(case.eta) for _ in range(4)]
        for dst, src in zip(fr, (case.eta, case.u, case.v, case.tracer)):
            dst[2:-2, 2:-2] = src[2:-2, 2:-2]
        formats.write_frame(str(d / "out" / f"{name}.0001.bin"), 0, 0.0, p.nx, p.ny, fr + [z])
    _, f64 = run(tmp_path / "a", name)
    _, f32 = run(tmp_path / "b", name, ["--fp32"])
    last = max(f64)
    assert max(f32) == last
    a, b = f64[last][4], f32[last][4]
    h = a["eta"][2:-2, 2:-2] + p.depth
    err = np.linalg.norm((b["eta"] - a["eta"])[2:-2, 2:-2]) / np.linalg.norm(h)
    assert err <= 1e-6, err
    tr = float(np.max(np.abs(a["tracer"])))
    assert np.max(np.abs(b["tracer"] - a["tracer"])) <= 1e-4 * max(tr, 1e-300)


@pytest.mark.parametrize("name", FULL)
def test_fp32_form_runs_the_forcing_cases(tmp_path, name):
    """The FP32 form with forcing (Gaussians, vortices, tracer injection)
    through the runner: sw2g_step_open runs the step with the plain halo
    update of u and v, the forcing changes the FP64 state, sw2g_step_close
    makes the halo update of eta and the tracer, do_channel and the range
    checks (core.c:287-312). Every frame of the reference's run, halos
    included, within the FP32 form's tolerance: h relative L2 <= 1e-5 over
    the interior, every padded cell of u, v and the tracer within 1e-3 of the
    field's largest magnitude; the injected fields and the times exact."""
    p = gc.forcing_params(name)
    formats.write_sw(str(tmp_path / f"{name}.sw"), p)
    _, frames = run(tmp_path, name, flags=("--fp32",))
    ref = gc.forcing_frames(name)
    assert sorted(frames) == list(range(len(ref)))
    inner = (slice(2, -2), slice(2, -2))
    for k, rf in enumerate(ref):
        nstep, t, nx, ny, fl = frames[k]
        assert t == float(rf["t"])
        assert np.array_equal(fl["perturbs"], rf["perturbs"]), k
        h = rf["eta"][inner] + p.depth
        assert np.linalg.norm((fl["eta"] - rf["eta"])[inner]) <= 1e-5 * np.linalg.norm(h), k
        assert np.max(np.abs(fl["eta"] - rf["eta"])) <= 2e-6 * p.depth, k
        for f in ("u", "v", "tracer"):
            scale = float(np.max(np.abs(rf[f])))
            assert np.max(np.abs(fl[f] - rf[f])) <= 1e-3 * max(scale, 1e-300), (k, f)
