#!/usr/bin/env python3
"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs only where the reference sources are present (it builds them with
oracle/Makefile into oracle/_ref). For each case it writes a fully expanded
`.sw` file and an initial MAGICSW2 frame, runs the reference single-rank with
`LoadFrom 1` (core.c:115-118) so the frame is its initial state, reads the
frames it saves, and stores initial and saved interiors plus the ENERGY lines
it prints. It then checks the C restatement in oracle/ against the same
frames bit for bit (the oracle pin) before writing anything.

    python tests/golden/make_golden.py            # all cases
    python tests/golden/make_golden.py --forcing  # the forcing and polar cases only
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as orc  # noqa: E402
from sw2_gb300 import cases, formats  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
REF_BIN = os.path.join(ROOT, "oracle", "_ref", "SW")
REF_DIR = os.environ.get("REF", "/root/reference")
REF_PATH = os.path.join(ROOT, "oracle", "_ref", "bin")


def wind_table(amp=40.0, k=4.0):
    # the table must cover the halo rows too (io.c:201-203 reads latc(-1)..latc(ny+2))
    lat = np.arange(-130.0, 130.5, 1.0)
    return np.stack([lat, amp * np.cos(np.deg2rad(k * lat))], axis=1)


# name: (make_case kwargs, nsteps, save_every)
CASES = {
    "g01_minmod_nu4": (dict(nx=24, ny=12, sch=2, seed=11), 30, 10),
    "g02_superbee_nu246": (dict(nx=24, ny=12, sch=1, seed=12), 30, 10),
    "g03_muscl_tau": (dict(nx=32, ny=16, sch=0, seed=13, hyper=False, Tau=3.0e5), 30, 15),
    "g04_muscl": (dict(nx=16, ny=8, sch=0, seed=14), 20, 20),
    "g05_koren": (dict(nx=16, ny=8, sch=4, seed=15), 20, 20),
    "g06_ospre": (dict(nx=16, ny=8, sch=5, seed=16), 20, 20),
    "g07_vanalbada": (dict(nx=16, ny=8, sch=6, seed=17), 20, 20),
    "g08_umist": (dict(nx=16, ny=8, sch=7, seed=18), 20, 20),
    "g09_upwind": (dict(nx=16, ny=8, sch=8, seed=19), 20, 20),
    "g10_laxwendroff": (dict(nx=16, ny=8, sch=9, seed=20), 20, 20),
    "g11_wind_tracer": (dict(nx=32, ny=16, sch=2, seed=21, wind=wind_table(), tracer=True,
                             TracerDis=2.0e-6, jet="cos6"), 40, 20),
    "g12_minmod_long": (dict(nx=40, ny=20, sch=2, seed=22), 200, 100),
    "g13_saturn_superbee": (dict(nx=48, ny=24, sch=1, seed=23, planet="saturn", jet="cos4x100",
                                 bumps=3, amp=(0.03, 0.03), sigma_km=(1500.0, 1500.0)), 60, 30),
    "g14_oblate_nu2": (dict(nx=24, ny=12, sch=2, seed=24, lat0=-35.0, lat1=-10.0, lon0=0.0,
                            lon1=90.0), 30, 15),
}

# cases where the reference aborts on its field range check (core.c:309-312;
# sppde_core.c:386-395): the Van Leer limiter evaluates 0/0 at r = -1
# (calc.c:57), which any flat row with one differing cell produces.
CRASH_CASES = {
    "c01_vanleer_nan": (dict(nx=32, ny=16, sch=3, seed=13, hyper=False, Tau=3.0e5), 30),
}

# cases stored as hashes (too large to commit as arrays)
HASH_CASES = {
    "h01_band256": (dict(nx=256, ny=128, sch=2, seed=1), 500, 500),
}


# Cases with the reference's time-dependent forcing, run from the reference's
# own initial state (LoadFrom 0: zero state, winds, forcing at t0, frame 0):
# golden vectors for the case-file runner (sw2_gb300/host). Each entry gives
# make_case keyword arguments (for the grid and physics; its fields are not
# used), the number of steps, SaveEvery, IteInfo and a function that adds
# the forcing tables.
def _f01(p):
    p.gaussians = [[0.0, 20 * p.Dt, 0.0, 100.0, 10.0, 0, 0.0, 2.5e13 / p.Dt, 0, 2.0e6, 5.0e6, 0.0]]


def _f02(p):
    # moving, ramped (rise, plateau, decay), sized in degrees, across the
    # periodic seam, injecting tracer
    p.gaussians = [[0.0, 40 * p.Dt, 3 * p.Dt, 2.0, -5.0, 0, -40.0, 1.5e13 / p.Dt, 1, 3.0, 8.0, 1.0]]
    p.TracerDis = 1.0e-6


def _f03(p):
    p.vortices = [[0.0, 60.0, -20.0, 7.4, 4.7, -100.0, 2.0],
                  [10.5 * p.Dt, 200.0, 25.0, 6.0, 4.0, 80.0, 1.5]]


def _f04(p):
    # the physics of the reference's examples/JupiterEnergyTest (its .sw and
    # .planet values): a moving injection on a 90 x 25 degree box
    p.gaussians = [[0.0, 7 * 86400.0, 0.0, 45.0, -22.5, 0, -3.6, 4.52e11, 0, 3.5e6, 3.5e6, 0.0]]


def _f05(p):
    _f04(p)


def _f06(p):
    # three injections on a 1024 x 512 band for the whole run (the bench's
    # forcing workload, cases.forcing_band)
    p.gaussians = cases.forcing_band(p.nsteps, p.nx, p.ny).gaussians


FORCING_CASES = {
    "f01_gauss_static": (dict(nx=48, ny=24, sch=2, seed=31, jet="none", bumps=0, lat0=-60.0, lat1=60.0),
                         60, 20, 10, _f01),
    "f02_gauss_moving_tracer": (dict(nx=64, ny=24, sch=1, seed=32, jet="none", bumps=0, lat0=-50.0, lat1=40.0,
                                     hyper=False), 60, 20, 5, _f02),
    "f03_vortices_wind": (dict(nx=60, ny=30, sch=7, seed=33, jet="none", bumps=0, wind="table"), 40, 10, 10, _f03),
    "f04_jupiter_box": (dict(nx=50, ny=50, sch=1, seed=34, jet="none", bumps=0, hyper=False, lon0=0.0, lon1=90.0,
                             lat0=-35.0, lat1=-10.0, Dt=50.0, h0=1000.0), 2000, 500, 100, _f04),
    # the whole 20-day run of that example (34,560 steps, frames every 12 h),
    # kept as the ENERGY lines and SHA-256 digests of the last frame
    "f05_jupiter_example": (dict(nx=50, ny=50, sch=1, seed=34, jet="none", bumps=0, hyper=False, lon0=0.0,
                                 lon1=90.0, lat0=-35.0, lat1=-10.0, Dt=50.0, h0=1000.0), 34560, 864, 100, _f05),
    # injections every step on a grid large enough for the forcing's cost to
    # matter; kept as the ENERGY lines and SHA-256 digests of the last frame
    "f06_gauss_1024": (dict(nx=1024, ny=512, sch=2, seed=36, jet="none", bumps=0, lat0=-60.0, lat1=60.0),
                       30, 10, 10, _f06),
}
HASH_ONLY = {"f05_jupiter_example", "f06_gauss_1024"}


def polar_wind_table(amp=30.0, k=6.0):
    lat = np.arange(-90.0, 90.5, 1.0)
    return np.stack([lat, amp * np.cos(np.deg2rad(k * lat))], axis=1)


# Polar caps (polar = 1 north, -1 south): run from an initial frame like CASES,
# checked against the reference's frames directly (the C restatement in
# oracle/ covers the band only).
POLAR_CASES = {
    "p01_north_minmod_nu4": (dict(n=40, polar=1, sch=2, seed=41, beta_sp=15.0, sig_sp=1e-5), 60, 20),
    "p02_south_superbee_tracer": (dict(n=32, polar=-1, angle_sim=15.0, sch=1, seed=42, beta_sp=10.0, sig_sp=3e-5,
                                       tracer=True, TracerDis=2e-6, Tau=3e5), 60, 20),
}


def polar_case(name):
    kw, nsteps, every = POLAR_CASES[name]
    case = cases.make_polar_case(**kw, nsteps=nsteps, wind=polar_wind_table())
    if name == "p02_south_superbee_tracer":
        nu4 = case.params.hypernu[1]
        case.params.hypernu = (2.0e-3 * nu4 ** 0.5, nu4, 1.0e-4 * nu4 ** 1.5)
    return case


def forcing_params(name):
    """CaseParams of a forcing case (also used by the tests to write the .sw)."""
    kw, nsteps, every, ite, add = FORCING_CASES[name]
    kw = dict(kw)
    wind = kw.pop("wind", None)
    if wind == "table":
        kw["wind"] = wind_table(30.0, 3.0)
    case = cases.make_case(**kw, nsteps=nsteps)
    p = case.params
    p.nsteps, p.SaveEvery, p.IteInfo, p.LoadFrom = nsteps, every, ite, 0
    if name in ("f04_jupiter_box", "f05_jupiter_example"):
        p.Omega, p.rE, p.rP, p.gE, p.depth = 0.000176, 7.1492e7, 6.6852e7, 22.58, 1000.0
        p.CFL, p.Tau, p.hypernu = 0.25, 1e7, (0.0, 0.0, 0.0)
        p.wind = np.array([[-81.58, 0.0], [78.72, 0.0]])
    add(p)
    return p


def run_reference_forcing(name, p, workdir):
    """Run the reference from its own initial state; frames 0.. and ENERGY lines."""
    os.makedirs(os.path.join(workdir, "out"), exist_ok=True)
    formats.write_sw(os.path.join(workdir, name + ".sw"), p)
    env = dict(os.environ, PATH=REF_PATH + os.pathsep + os.environ["PATH"])
    r = subprocess.run([REF_BIN, "1", "1", name, "out"], cwd=workdir, env=env, capture_output=True, text=True)
    if r.returncode != 0 or "CRASH" in r.stdout + r.stderr:
        raise RuntimeError(f"reference failed on {name}:\n{r.stdout[-3000:]}\n{r.stderr[-2000:]}")
    energy = [ln.split(None, 1)[1].strip() for ln in r.stdout.splitlines() if ln.startswith("ENERGY")]
    frames = []
    k = 0
    while os.path.exists(os.path.join(workdir, "out", f"{name}.{k:04d}.bin")):
        frames.append(formats.read_frame(os.path.join(workdir, "out", f"{name}.{k:04d}.bin")))
        k += 1
    return energy, frames


def tweak(name, case):
    p = case.params
    if name == "g02_superbee_nu246":
        nu4 = p.hypernu[1]
        p.hypernu = (2.0e-3 * nu4 ** 0.5, nu4, 1.0e-4 * nu4 ** 1.5)
    if name == "g14_oblate_nu2":
        # oblate planet (Jupiter polar radius) to exercise epsilon2 != 1
        p.rP = 6.6852e7
        nu4 = p.hypernu[1]
        p.hypernu = (1.0e-3 * nu4 ** 0.5, nu4, 0.0)
    return case


def run_reference(name, case, nsteps, save_every, workdir):
    p = case.params
    p.nsteps = nsteps
    p.SaveEvery = save_every
    p.IteInfo = save_every
    p.LoadFrom = 1
    os.makedirs(os.path.join(workdir, "out"), exist_ok=True)
    formats.write_sw(os.path.join(workdir, name + ".sw"), p)
    z = np.zeros_like(case.eta)
    fr = [np.zeros_like(case.eta) for _ in range(4)]
    for dst, src in zip(fr, (case.eta, case.u, case.v, case.tracer)):
        dst[2:-2, 2:-2] = src[2:-2, 2:-2]
    formats.write_frame(os.path.join(workdir, "out", name + ".0001.bin"), 0, 0.0, p.nx, p.ny, fr + [z])
    env = dict(os.environ, PATH=REF_PATH + os.pathsep + os.environ["PATH"])
    r = subprocess.run([REF_BIN, "1", "1", name, "out"], cwd=workdir, env=env, capture_output=True, text=True)
    if r.returncode != 0 or "CRASH" in r.stdout + r.stderr:
        raise RuntimeError(f"reference failed on {name}:\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
    energy = [list(map(float, ln.split()[1:])) for ln in r.stdout.splitlines() if ln.startswith("ENERGY")]
    frames = []
    k = 2
    while True:
        path = os.path.join(workdir, "out", f"{name}.{k:04d}.bin")
        if not os.path.exists(path):
            break
        nstep, t, nx, ny, flds = formats.read_frame(path)
        frames.append((nstep, t, flds))
        k += 1
    return energy, frames


def oracle_frames(case, nsteps, save_every):
    o = orc.Oracle(case.params)
    o.load(case.fields())
    out = []
    energy = [o.energy()]
    done = 0
    while done < nsteps:
        rc, bad = o.step(save_every)
        if rc:
            raise RuntimeError(f"oracle check failed rc={rc} at step {bad}")
        done += save_every
        out.append({k: o.field(k) for k in ("eta", "u", "v", "tracer")})
        energy.append(o.energy())
    return out, energy


def interior(a):
    return np.ascontiguousarray(a[2:-2, 2:-2])


def params_json(p):
    d = {k: getattr(p, k) for k in ("nx", "ny", "sch", "lon0", "lon1", "lat0", "lat1", "t0", "nsteps", "Dt",
                                    "CFL", "Tau", "IteInfo", "SaveEvery", "LoadFrom", "Omega", "rE", "rP",
                                    "gE", "depth", "TracerDis", "polar", "angleSim", "BetaSp", "SigSp")}
    d["hypernu"] = list(p.hypernu)
    d["wind"] = None if p.wind is None else p.wind.tolist()
    return d


def run_reference_crash(name, case, nsteps, workdir):
    """Run a case expected to abort; return the step the reference aborted in."""
    p = case.params
    p.nsteps, p.SaveEvery, p.IteInfo, p.LoadFrom = nsteps, nsteps, 1, 1
    os.makedirs(os.path.join(workdir, "out"), exist_ok=True)
    formats.write_sw(os.path.join(workdir, name + ".sw"), p)
    fr = [np.zeros_like(case.eta) for _ in range(5)]
    for dst, src in zip(fr, (case.eta, case.u, case.v, case.tracer)):
        dst[2:-2, 2:-2] = src[2:-2, 2:-2]
    formats.write_frame(os.path.join(workdir, "out", name + ".0001.bin"), 0, 0.0, p.nx, p.ny, fr)
    env = dict(os.environ, PATH=REF_PATH + os.pathsep + os.environ["PATH"])
    r = subprocess.run([REF_BIN, "1", "1", name, "out"], cwd=workdir, env=env, capture_output=True, text=True)
    out = r.stdout + r.stderr
    if "nonsense value detected" not in out:
        raise RuntimeError(f"{name}: expected the reference to abort on its range check")
    started = [int(ln.split()[4]) for ln in r.stdout.splitlines() if ln.startswith("===SW STARTING TIME STEP")]
    return started[-1]


def check_pin(name, ref_frames, orc_frames):
    for (nstep, t, rf), of in zip(ref_frames, orc_frames):
        for k in ("eta", "u", "v", "tracer"):
            a, b = interior(rf[k]), interior(of[k])
            if not np.array_equal(a, b):
                d = np.max(np.abs(a - b))
                raise AssertionError(f"{name}: oracle differs from reference in {k} at step {nstep}: max|d|={d}")


def main():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "all", "ref"], check=True)
    if not os.path.exists(REF_BIN):
        raise SystemExit("reference not built (sources absent?)")
    only_forcing = "--forcing" in sys.argv  # regenerate the forcing and polar cases only
    # --only NAME: run the reference on that one forcing case and update its entry
    only = sys.argv[sys.argv.index("--only") + 1] if "--only" in sys.argv else None
    manifest = {}
    if only:
        with open(os.path.join(OUT, "manifest.json")) as fh:
            manifest = json.load(fh)
        CRASH_CASES.clear()
        CASES.clear()
        HASH_CASES.clear()
        POLAR_CASES.clear()
        for k in list(FORCING_CASES):
            if k != only:
                del FORCING_CASES[k]
    if only_forcing:
        with open(os.path.join(OUT, "manifest.json")) as fh:
            manifest = {k: v for k, v in json.load(fh).items() if not v.get("forcing") and not v.get("polar")}
        CRASH_CASES.clear()
        CASES.clear()
        HASH_CASES.clear()
    for name, (kw, nsteps) in CRASH_CASES.items():
        case = cases.make_case(**dict(kw, nsteps=nsteps))
        with tempfile.TemporaryDirectory() as wd:
            crash_step = run_reference_crash(name, case, nsteps, wd)
        o = orc.Oracle(case.params)
        o.load(case.fields())
        rc, bad = o.step(nsteps)
        assert rc == 2 and bad + 1 == crash_step, (name, rc, bad, crash_step)
        arrs = {"init_" + k: interior(getattr(case, k)) for k in ("eta", "u", "v", "tracer")}
        np.savez_compressed(os.path.join(OUT, name + ".npz"), **arrs)
        manifest[name] = {"params": params_json(case.params), "nsteps": nsteps, "abort_step": crash_step}
        print(f"{name}: reference and oracle both abort in step {crash_step}")
    for name, (kw, nsteps, every) in list(CASES.items()) + list(HASH_CASES.items()):
        kw = dict(kw)
        kw.setdefault("nsteps", nsteps)
        case = tweak(name, cases.make_case(**kw))
        with tempfile.TemporaryDirectory() as wd:
            energy, ref_frames = run_reference(name, case, nsteps, every, wd)
        orc_fr, orc_en = oracle_frames(case, nsteps, every)
        assert len(ref_frames) == nsteps // every, (name, len(ref_frames))
        check_pin(name, ref_frames, orc_fr)
        # the reference prints ENERGY (with %e, 7 significant digits) after the
        # load, at the first step and every IteInfo steps (core.c:126-136,328-331)
        printed = [energy[0]] + (energy[2:] if every > 1 else energy[1:])
        assert len(printed) == len(orc_en), (name, len(printed), len(orc_en))
        for (t, ke, ape, tot), (oke, oape, _m) in zip(printed, orc_en):
            assert float(f"{oke:e}") == ke and float(f"{oape:e}") == ape, (name, t, ke, oke, ape, oape)
        entry = {"params": params_json(case.params), "nsteps": nsteps, "save_every": every,
                 "energy_printed": energy}
        if name in CASES:
            arrs = {}
            for k in ("eta", "u", "v", "tracer"):
                arrs["init_" + k] = interior(getattr(case, k))
            arrs["windx"] = case.windx
            arrs["windy"] = case.windy
            for fi, (nstep, t, rf) in enumerate(ref_frames):
                for k in ("eta", "u", "v", "tracer"):
                    arrs[f"f{fi}_{k}"] = interior(rf[k])
            np.savez_compressed(os.path.join(OUT, name + ".npz"), **arrs)
        else:
            nstep, t, rf = ref_frames[-1]
            entry["sha256"] = {k: hashlib.sha256(interior(rf[k]).tobytes()).hexdigest() for k in ("eta", "u", "v")}
            entry["init_sha256"] = {k: hashlib.sha256(interior(getattr(case, k)).tobytes()).hexdigest()
                                    for k in ("eta", "u", "v")}
            entry["make_case"] = {k: v for k, v in kw.items()}
        manifest[name] = entry
        print(f"{name}: reference and oracle agree bit for bit over {nsteps} steps")
    for name in POLAR_CASES:
        kw, nsteps, every = POLAR_CASES[name]
        case = polar_case(name)
        with tempfile.TemporaryDirectory() as wd:
            energy, ref_frames = run_reference(name, case, nsteps, every, wd)
        assert len(ref_frames) == nsteps // every, (name, len(ref_frames))
        arrs = {"init_" + k: interior(getattr(case, k)) for k in ("eta", "u", "v", "tracer")}
        arrs["windx"], arrs["windy"] = case.windx, case.windy
        for fi, (nstep, t, rf) in enumerate(ref_frames):
            for k in ("eta", "u", "v", "tracer"):
                arrs[f"f{fi}_{k}"] = interior(rf[k])
        np.savez_compressed(os.path.join(OUT, name + ".npz"), **arrs)
        manifest[name] = {"params": params_json(case.params), "nsteps": nsteps, "save_every": every,
                          "energy_printed": energy, "polar": True}
        print(f"{name}: {len(ref_frames)} reference frames (polar {case.params.polar})")
    for name in FORCING_CASES:
        p = forcing_params(name)
        with tempfile.TemporaryDirectory() as wd:
            energy, frames = run_reference_forcing(name, p, wd)
        nframes = p.nsteps // p.SaveEvery + 1
        assert len(frames) == nframes, (name, len(frames), nframes)
        manifest[name] = {"params": params_json(p), "vortices": p.vortices, "gaussians": p.gaussians,
                          "nsteps": p.nsteps, "save_every": p.SaveEvery, "ite_info": p.IteInfo,
                          "frames": nframes, "energy_printed": energy, "forcing": True}
        if name in HASH_ONLY:
            nstep, t, nx, ny, fl = frames[-1]
            manifest[name]["last_frame"] = {"t": t, "sha256": {
                k: hashlib.sha256(np.ascontiguousarray(fl[k]).tobytes()).hexdigest()
                for k in ("eta", "u", "v", "tracer", "perturbs")}}
        else:
            arrs = {}
            for fi, (nstep, t, nx, ny, fl) in enumerate(frames):
                for k in ("eta", "u", "v", "tracer", "perturbs"):
                    arrs[f"f{fi}_{k}"] = np.ascontiguousarray(fl[k])
                arrs[f"f{fi}_t"] = np.array(t)
            np.savez_compressed(os.path.join(OUT, name + ".npz"), **arrs)
        print(f"{name}: {nframes} reference frames, {len(energy)} ENERGY lines")
    # the reference's only known-answer file: ENERGY lines of its
    # examples/JupiterEnergyTest run (an older version of the code), which
    # f04_jupiter_box mirrors; kept for its first 1e5 s
    kat = os.path.join(REF_DIR, "examples", "JupiterEnergyTest", "enou.txt")
    if os.path.exists(kat) and not only:
        with open(kat) as fh:
            lines = [ln.split(None, 1)[1].strip() for ln in fh if ln.startswith("ENERGY")]
        manifest["kat_enou"] = {"source": "examples/JupiterEnergyTest/enou.txt",
                                "energy_printed": [ln for ln in lines if float(ln.split()[0]) <= 1.0e5],
                                "forcing": True}
    with open(os.path.join(OUT, "manifest.json"), "w") as fh:
        json.dump(manifest, fh, indent=1)


if __name__ == "__main__":
    main()
