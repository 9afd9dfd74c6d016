#!/usr/bin/env python3
"""Throughput of the SW2 shallow-water step on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--config band2048]

A "step" is one model time step of the whole grid. The default workload is
the plain-FP64 drop-in configuration: a 2048x1024 latitude-longitude band
(Jupiter constants, balanced 60cos(6phi) jet plus a seeded Gaussian bump,
minmod limiter, AB3, nabla^4 hyperviscosity), inputs synthetic.

Printed (rank 0, one JSON line): cell-updates/s over the K timed steps (device
time, CUDA events on the library's stream, inputs resident), the same metric
end to end through the C ABI with the state copied host->device and back
every step (pinned host buffers), the roofline of the dominant kernel, the
GPU clocks seen during the timed region, and the CPU oracle timed on the
host cores as the CPU baseline.

With --impl reference the CPU implementation of the step (the oracle
restatement of the reference, all host threads) is timed on the same
workload and metric instead.

Multi-GPU: one process per GPU (torchrun); the step does not shard, so each
rank advances an independent replica (its own seed) and the throughput is the
sum over ranks divided by the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-updates/s and HBM GB/s/roofline: FP64 plain vs FP32 batched at stated h L2 err"
UNIT = "cell-updates/s"

# Algorithmic bytes per interior cell and launch, per kernel of the FP64 step:
# the fields a kernel must read and write at least once (8 B each; winds and
# bottom height are zero in these workloads and are not counted).
KERNEL_BYTES = {
    "mass": 8 * (3 + 1),        # eta u v -> Deta
    "adv_u": 8 * (2 + 1),       # u v -> Du_adv
    "adv_v": 8 * (2 + 1),       # u v -> Dv_adv
    "pres_sum": 8 * (5 + 2),    # eta u v Du_adv Dv_adv -> Du_n Dv_n
    "ab": 8 * (3 + 1),
    "coriolis_u": 8 * (6 + 2),  # from the third step: u v, D_n D_n-1 D_n-2, nu4 L -> D_n u (AB3 fused)
    "coriolis_v": 8 * (6 + 2),
    "eta_ab3": 8 * (6 + 2),     # eta v, D_n D_n-1 D_n-2, nu4 L -> D_n eta (hyper, AB3, geofactor, update)
    "lape_pass1": 8 * (1 + 2),
    "lape_pass2": 8 * (2 + 1),
    "lapv_pass1": 8 * (2 + 2),
    "lapv_pass2": 8 * (2 + 2),
    "hyper_add": 8 * (4 + 1),
    "geofactor": 8 * (3 + 1),
    "add": 8 * (2 + 1),
    "cfl": 8 * 2,
    "range": 8 * 1,
    # FP32 form: FP64 state (8 B), FP32 shadows of the state, histories and
    # intermediates (4 B)
    "f32_lap1": 4 * 2 + 4 * 2,  # u v shadows -> Lu Lv
    # eta u v shadows, Lu Lv, eta, 2 eta hist -> eta + shadow, hist, partial Du Dv
    "f32_main1": 4 * 3 + 4 * 2 + 8 + 4 * 2 + 8 + 4 + 4 + 4 * 2,
    # new eta shadow, u v, their shadows, partials, 4 hist -> u v + shadows, 2 hist
    "f32_main2": 4 + 8 * 2 + 4 * 2 + 4 * 2 + 4 * 4 + 8 * 2 + 4 * 2 + 4 * 2,
    "f32_lap3": 4 * 2 + 4 * 2 + 4 * 2,  # LLu LLv, partials -> partials
    "f32_tracer": 4 * 3 + 8 + 4 * 2 + 8 + 4 + 4,  # tracer u v shadows, tracer, 2 hist -> tracer + shadow, hist
}
# DRAM bytes (read + write) of one launch of the dominant kernels on the
# 2048x1024 workload, from an ncu capture of the same step (third step, one
# launch each, the current kernels). With zero winds the plain bodies read eta
# or u and v only; part of each input is still in L2 from the kernel before,
# and most of the output leaves L2 later, so DRAM bytes are below the
# algorithmic bytes.
NCU_TRAFFIC = {("band2048", "mass"): 52.60e6, ("band2048", "adv_u"): 34.18e6, ("band2048", "adv_v"): 34.26e6}
# FP64 thread instructions (DADD + DMUL + DFMA) per interior cell of the
# dominant kernels on the 2048x1024 workload, from ncu's instruction counters
# of the same capture, and the FP64 unit's busy fraction there; GB300's FP64
# peak per cycle over the whole GPU (ncu's peak for DFMA: 304 = 2 lanes per SM
# x 152 SMs). The FP64 form is bound by this unit.
NCU_FP64_PER_CELL = {("band2048", "mass"): 52.5, ("band2048", "adv_u"): 68.8, ("band2048", "adv_v"): 69.2}
NCU_FP64_PIPE_BUSY = {("band2048", "mass"): 0.827, ("band2048", "adv_u"): 0.838, ("band2048", "adv_v"): 0.838}
FP64_LANES_PER_CYCLE = 304
# The whole step: read eta u v, write eta u v, read two history levels of
# three tendencies, write one (a per-cell count for the step's GB/s figure).
STEP_BYTES = 120


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        # the raw samples: a folder named by SW2G_CLOCKS_DIR, else /tmp
        out = os.environ.get("SW2G_CLOCKS_DIR") or "/tmp"
        self.path = os.path.join(out, f"sw2g_clocks_rank{device}_{os.getpid()}.csv")

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        with open(self.path) as fh:
            for ln in fh:
                p = [x.strip() for x in ln.split(",")]
                if len(p) >= 9 and p[1].isdigit():
                    rows.append(p)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        # samples with the "GPU idle" event bit (0x1) were taken outside kernel work
        busy = [r for r in rows if not (int(r[4], 16) & 0x1)]
        use = busy or rows
        sm = [int(r[1]) for r in use]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in use for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": int(rows[0][2]), "reasons": reasons,
                "samples": len(rows), "samples_under_load": len(busy)}


def make_workload(name: str, seed: int):
    from sw2_gb300 import cases

    case = cases.config_case(name, seed=seed)
    desc = {
        "band2048": "2048x1024 lat-lon band 0-360E x 70S-70N, Jupiter (a=7.1492e7 m, Omega=1.7585e-4, g=10, "
                    "h0=2.5e4 m), balanced jet 60cos(6phi) + 1 Gaussian (0.05 h0, 2000 km), minmod, AB3, "
                    "nabla^4 (grid e-fold 10 dt), dt from CFL 0.3",
        "band256": "256x128 band, same physics as band2048",
        "saturn4096": "4096x2048 band, Saturn, jet 100cos(4phi) + 3 Gaussians, superbee, AB3",
        "band8192": "8192x4096 band, Jupiter, jet 60cos6phi+20cos14phi + 200 Gaussians, minmod, AB3",
    }[name]
    return case, desc


def time_cpu_oracle(case, nsteps: int):
    """Oracle restatement on the host cores: (cell-updates/s, threads, seconds)."""
    from oracle import oracle as orc

    o = orc.Oracle(case.params)
    o.load(case.fields())
    o.step(1)  # first touch
    t0 = time.perf_counter()
    rc, _ = o.step(nsteps)
    dt = time.perf_counter() - t0
    if rc:
        raise RuntimeError(f"oracle aborted (rc={rc})")
    p = case.params
    return p.nx * p.ny * nsteps / dt, orc.threads(), dt


def run_reference_arm(args, ws, rank):
    if rank != 0:
        return
    case, desc = make_workload(args.config, seed=1)
    p = case.params
    from oracle import oracle as orc

    o = orc.Oracle(p)
    o.load(case.fields())
    o.step(args.warmup)
    t0 = time.perf_counter()
    rc, _ = o.step(args.steps)
    dt = time.perf_counter() - t0
    if rc:
        raise RuntimeError(f"oracle aborted (rc={rc})")
    v = p.nx * p.ny * args.steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{args.config}: {desc}", "nx": p.nx, "ny": p.ny, "form": "fp64-exact"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": orc.threads(), "kind": "port",
                         "sample": f"{args.config}, {args.steps} full-grid steps after {args.warmup} warm-up "
                                   f"(C restatement of the reference step, OpenMP over rows; the reference "
                                   f"binary itself cannot be built on the GPU host)"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def measure(lib, case, precision, steps, warmup, local, barrier, flags=0):
    """Timed region of one form: K steps with inputs resident; then a second
    pass with per-kernel timers. Returns a dict of measurements."""
    p = case.params
    cells = p.nx * p.ny
    s = lib.Solver(p, precision=precision, device=local, flags=flags)
    s.upload(*case.fields())
    assert s.step(warmup) == lib.OK
    barrier()
    rc = s.step(steps)
    barrier()
    if rc != lib.OK:
        raise RuntimeError(f"step failed: {lib.status_string(rc)} at step {s.error_step()}")
    ms = s.last_step_ms()
    launches = s.last_launches()
    s.timers(True)
    s.timers_reset()
    assert s.step(steps) == lib.OK
    table = s.timer_table()
    s.timers(False)
    name, (nl, kms) = max(table.items(), key=lambda kv: kv[1][1])
    per_launch = kms / nl
    kb = KERNEL_BYTES.get(name)
    total_k = sum(v[1] for v in table.values())
    gbs = {k: KERNEL_BYTES[k] * cells / (v[1] / v[0] * 1e-3) / 1e9 for k, v in table.items() if k in KERNEL_BYTES}
    return {"solver": s, "ms": ms, "launches": launches, "value": cells * steps / (ms * 1e-3),
            "kernel": name, "per_launch_ms": per_launch, "bytes_per_cell": kb,
            "achieved_gbs": (kb * cells / (per_launch * 1e-3) / 1e9) if kb else None,
            "kernel_share": kms / total_k,
            "kernels_ms_per_step": {k: v[1] / steps for k, v in sorted(table.items(), key=lambda kv: -kv[1][1])},
            "kernels_gbs": dict(sorted(gbs.items(), key=lambda kv: -kv[1]))}


def accuracy(lib, case, nsteps, local):
    """FP32 form against the FP64 reference-exact step after nsteps: relative
    L2 over the interior of h = eta + depth, u, v, and the relative drift of
    mass and energy of each form."""
    d = case.params.depth
    out = {"steps": nsteps}
    res = {}
    for nm, prec in (("fp64", lib.FP64), ("fp32", lib.FP32)):
        s = lib.Solver(case.params, precision=prec, device=local)
        s.upload(*case.fields())
        k0, a0, m0 = s.diag()
        rc = s.step(nsteps)
        if rc != lib.OK:
            return {"steps": nsteps, "error": f"{nm}: {lib.status_string(rc)} at step {s.error_step()}"}
        out[f"value_{nm}"] = case.params.nx * case.params.ny * nsteps / (s.last_step_ms() * 1e-3)
        k1, a1, m1 = s.diag()
        res[nm] = s.download()
        out[f"mass_drift_{nm}"] = (m1 - m0) / m0
        out[f"energy_drift_{nm}"] = ((k1 + a1) - (k0 + a0)) / (k0 + a0)
        s.close()
    a, b = res["fp32"], res["fp64"]
    I = (slice(2, -2), slice(2, -2))
    out["h_rel_l2"] = float(np.linalg.norm((a["eta"] - b["eta"])[I]) / np.linalg.norm((b["eta"] + d)[I]))
    for k in ("u", "v"):
        out[f"{k}_rel_l2"] = float(np.linalg.norm((a[k] - b[k])[I]) / np.linalg.norm(b[k][I]))
    return out


def parity_fp64(lib, case, nsteps, local):
    """The FP64 CUDA step against the oracle (the C restatement of the
    reference step, pinned to the reference's own frames) after nsteps from
    the same state: whether every padded cell of eta, u and v is bit-identical,
    the relative L2 over the interior of h = eta + depth, u and v, and the
    relative mass and energy drift of each."""
    from oracle import oracle as orc

    p = case.params
    s = lib.Solver(p, precision=lib.FP64, device=local)
    s.upload(*case.fields(), mode=lib.UPLOAD_FRAME)
    g0 = s.diag()
    rc = s.step(nsteps)
    if rc != lib.OK:
        return {"steps": nsteps, "error": f"gpu: {lib.status_string(rc)} at step {s.error_step()}"}
    g1 = s.diag()
    got = s.download()
    s.close()
    o = orc.Oracle(p)
    o.load(case.fields())
    r0 = o.energy()
    t0 = time.perf_counter()
    rc, bad = o.step(nsteps)
    secs = time.perf_counter() - t0
    if rc:
        return {"steps": nsteps, "error": f"oracle: rc {rc} at step {bad}"}
    r1 = o.energy()
    ref = {k: o.field(k) for k in ("eta", "u", "v")}
    I = (slice(2, -2), slice(2, -2))
    out = {"steps": nsteps, "bit_identical": all(np.array_equal(got[k], ref[k]) for k in ref),
           "h_rel_l2": float(np.linalg.norm((got["eta"] - ref["eta"])[I]) / np.linalg.norm((ref["eta"] + p.depth)[I]))}
    for k in ("u", "v"):
        out[f"{k}_rel_l2"] = float(np.linalg.norm((got[k] - ref[k])[I]) / np.linalg.norm(ref[k][I]))
    for nm, (a, b) in (("gpu", (g0, g1)), ("oracle", (r0, r1))):
        out[f"mass_drift_{nm}"] = (b[2] - a[2]) / a[2]
        out[f"energy_drift_{nm}"] = ((b[0] + b[1]) - (a[0] + a[1])) / (a[0] + a[1])
    out["oracle_seconds"] = secs
    out["oracle_threads"] = orc.threads()
    return out


def metric_divisors(case):
    """The row metric factors the FP64 step divides by (DXE, DXV, DYN, DYC,
    DXE+DXE, rZ at centres and faces), every row including halos."""
    from sw2_gb300 import cases

    p = case.params
    g = cases.Grid(p)
    dlon = (g.lon1 - g.lon0) / float(p.nx)
    dlat = (g.lat1 - g.lat0) / float(p.ny)
    out = []
    for j in range(-1, p.ny + 3):
        lc, ln, ln1 = g.latc(j), g.latn(j), g.latn(j - 1)
        dxe = dlon * g.rZ(lc)
        out += [dxe, dlon * g.rZ(ln), dlat * g.rM(lc), dlat * g.rM(ln1), dxe + dxe, g.rZ(lc), g.rZ(ln)]
    return np.array(out)


def forcing_leg(nsteps: int = 40):
    """Per-step time of the case-file runner (sw2g-run: case reader, forcing,
    GPU step) on a 1024x512 band with three Gaussians injected in each of its
    40 steps (cases.forcing_band), in its two forcing paths: the host
    evaluates the cells inside the radii with the reference's expressions and
    sends them as lists (bit for bit), or the GPU evaluates the fields, the
    volume and its rescale from the per-step scalars (--device-forcing, within
    rounding). The runner times its own time loop (--timing: every step
    forced, a frame at the first and the last); best of three runs per path.
    The band starts at rest, as the reference's forcing cases do: the cells
    the waves have not reached have zero fluxes, which the FP64 bodies compute
    with the literal per-cell code, so these steps cost more than a step of a
    flowing state."""
    import re
    import tempfile

    from sw2_gb300 import cases, formats, hostlib

    def per_step(flags):
        best = None
        with tempfile.TemporaryDirectory() as wd:
            p = cases.forcing_band(nsteps)
            name = "forced"
            formats.write_sw(os.path.join(wd, name + ".sw"), p)
            os.makedirs(os.path.join(wd, "out"), exist_ok=True)
            for _ in range(3):
                r = subprocess.run([hostlib.RUNNER, "--quiet", "--timing", *flags, "1", "1", name, "out"], cwd=wd,
                                   capture_output=True, text=True, timeout=600)
                m = re.search(r"LOOP (\d+) steps ([0-9.eE+-]+) s", r.stderr)
                if r.returncode != 0 or not m:
                    return {"error": r.stderr[-500:]}
                t = float(m.group(2)) / int(m.group(1))
                best = t if best is None else min(best, t)
        return best

    host = per_step(())
    dev = per_step(("--device-forcing",))
    p = cases.forcing_band(nsteps)
    out = {"workload": f"{p.nx}x{p.ny} band from rest, 3 Gaussians injected in each of {nsteps} steps (ramped "
                       f"static, moving across the seam with tracer, against the wall), minmod, nu4, FP64"}
    for key, v, path in (("host_forcing", host, "host evaluation of the cells inside each radius, sw2g_set_cells + "
                                                  "sw2g_add_cells between sw2g_step_open and sw2g_step_close"),
                         ("device_forcing", dev, "sw2g_add_gaussian: field, volume sum and rescale on the GPU, "
                                                 "between sw2g_step_open and sw2g_step_close")):
        out[key] = v if isinstance(v, dict) else {"ms_per_forced_step": 1e3 * v,
                                                  "cell_updates_per_s": p.nx * p.ny / v, "path": path}
    return out


def ensemble(lib, nsteps, tune_steps, acc_steps, local, seed=7):
    """The 64-member ensemble on uneven grids (16 x 512x256, 24 x 1024x512,
    24 x 2048x1024; Van Leer, FP32 form) stepped as one batch: one launch per
    phase over all members, one-step CUDA graph replays, tile shape and sweep
    schedule chosen by the tuner. Worst-member h error against the FP64 step
    over all members."""
    from sw2_gb300 import cases

    specs = cases.ensemble_members(seed)
    solvers, cs = [], []
    for nx, ny, kw in specs:
        c = cases.make_case(nx, ny, **kw)
        s = lib.Solver(c.params, precision=lib.FP32, device=local, flags=lib.FLAG_VANLEER_SAFE)
        s.upload(*c.fields())
        solvers.append(s)
        cs.append(c)
    cells = sum(c.params.nx * c.params.ny for c in cs)
    b = lib.Batch(solvers)
    assert b.step(3) == lib.OK
    tune = b.tune(tune_steps)
    rc = b.step(nsteps)
    if rc != lib.OK:
        raise RuntimeError(f"ensemble step failed: {lib.status_string(rc)} {b.error()}")
    ms = b.last_step_ms()
    out = {"members": len(cs), "grids": "16 x 512x256, 24 x 1024x512, 24 x 2048x1024",
           "cells_per_step": cells, "steps": nsteps, "value": cells * nsteps / (ms * 1e-3), "unit": UNIT,
           "ms_per_step": ms / nsteps, "launches_per_step": b.last_launches() / nsteps,
           "schedule": f"128x{b.tile_rows()}/{b.schedule()}", "tune_ms_per_step": tune,
           "tune_spread": max(tune.values()) / min(tune.values()), "limiter": "Van Leer (r <= 0 -> 0)"}
    b.close()
    if acc_steps > 0:
        # every member from its initial state, acc_steps steps as one batch,
        # against the FP64 step of the same member run alone
        for s, c in zip(solvers, cs):
            s.upload(*c.fields())
        b = lib.Batch(solvers)
        if b.step(acc_steps) != lib.OK:
            raise RuntimeError(f"ensemble accuracy batch failed: {b.error()}")
        b.close()
        errs = []
        for s, c in zip(solvers, cs):
            e32 = s.download()["eta"][2:-2, 2:-2]
            ref = lib.Solver(c.params, precision=lib.FP64, device=local, flags=lib.FLAG_VANLEER_SAFE)
            ref.upload(*c.fields())
            if ref.step(acc_steps) != lib.OK:
                raise RuntimeError("ensemble FP64 reference run failed")
            e64 = ref.download()["eta"][2:-2, 2:-2]
            ref.close()
            errs.append(float(np.linalg.norm(e32 - e64) / np.linalg.norm(e64 + c.params.depth)))
        w = int(np.argmax(errs))
        out["worst_member_h_rel_l2"] = errs[w]
        out["worst_member"] = {"index": w, "grid": f"{cs[w].params.nx}x{cs[w].params.ny}"}
        out["median_member_h_rel_l2"] = float(np.median(errs))
        out["accuracy_members"] = f"all {len(cs)} (the batched run against each member's FP64 run alone)"
        out["accuracy_steps"] = acc_steps
    for s in solvers:
        s.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="band2048")
    ap.add_argument("--fp32-config", default="saturn4096", help="workload of the FP32-form throughput line")
    ap.add_argument("--accuracy-steps", type=int, default=2000)
    ap.add_argument("--ensemble-steps", type=int, default=1000, help="0 skips the 64-member ensemble leg")
    ap.add_argument("--parity-steps", type=int, default=2000,
                    help="steps of the FP64 step against the oracle on the headline workload (0 skips)")
    ap.add_argument("--large-config", default="band8192", help="workload of the large case run in both forms")
    ap.add_argument("--large-steps", type=int, default=1000, help="steps of the large case (0 skips it)")
    ap.add_argument("--no-forcing", dest="forcing", action="store_false",
                    help="skip the per-step time of the forced 1024x512 case through the case-file runner")
    ap.add_argument("--cpu-steps", type=int, default=None, help="oracle steps for the CPU baseline sample")
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    from sw2_gb300.replicas import aggregate, dist_env

    ws, rank, local = dist_env()
    if args.impl == "reference":
        return run_reference_arm(args, ws, rank)

    import torch

    pg = None
    if ws > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        pg = dist
    from sw2_gb300 import lib

    lib.load()
    case, desc = make_workload(args.config, seed=1 + rank)
    p = case.params
    cells = p.nx * p.ny

    def barrier():
        torch.cuda.synchronize(local)
        if pg:
            pg.barrier()

    # headline: the FP64 reference-exact step on the drop-in configuration
    clk = ClockSampler(local).__enter__()
    m64 = measure(lib, case, lib.FP64, args.steps, args.warmup, local, barrier)
    dev = f"cuda:{local}"
    value, _, secs = aggregate(cells * args.steps, m64["ms"] * 1e-3, dev)
    ms = secs * 1e3
    s = m64["solver"]

    # end to end through the C ABI: every step is one sw2g_step_host call on
    # the state held in pinned host arrays (copied in, stepped once, copied
    # back into the same arrays)
    W, H = p.nx + 4, p.ny + 4
    host = [torch.empty((H, W), dtype=torch.float64, pin_memory=True).numpy() for _ in range(3)]
    d = s.download()
    for h, k in zip(host, ("eta", "u", "v")):
        h[...] = d[k]
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        if s.step_host(host[0], host[1], host[2], 1) != lib.OK:
            raise RuntimeError("e2e step failed")
    barrier()
    e2e, _, _ = aggregate(cells * args.steps, time.perf_counter() - t0, dev)
    bytes_io = 3 * W * H * 8
    # back: the three fields, u's halo columns and wall rows once more (written
    # at the end of the step, after u's interior went out) and the step's checks
    bytes_out = bytes_io + (4 * W + 4 * p.ny) * 8 + 2 * 8 + 4
    s.close()

    # the FP32 precision form, same workload and the larger precision-form workload
    m32 = measure(lib, case, lib.FP32, args.steps, args.warmup, local, barrier)
    m32["solver"].close()
    c32, desc32 = make_workload(args.fp32_config, seed=1 + rank)
    m32b = measure(lib, c32, lib.FP32, args.steps, args.warmup, local, barrier)
    m32b["solver"].close()
    m64b = measure(lib, c32, lib.FP64, args.steps, args.warmup, local, barrier)
    m64b["solver"].close()
    clk.__exit__(None, None, None)
    acc = accuracy(lib, c32, args.accuracy_steps, local) if args.accuracy_steps > 0 else None
    if acc:
        acc["workload"] = args.fp32_config
    ens = ensemble(lib, args.ensemble_steps, 5, min(args.ensemble_steps, 1000), local) if args.ensemble_steps > 0 else None
    # the large case in both forms: per-kernel times and GB/s over a short
    # timed run, then large_steps steps of each form (throughput over the
    # whole run, errors of the FP32 form against the FP64 one)
    large = None
    if args.large_steps > 0:
        cl, descl = make_workload(args.large_config, seed=1 + rank)
        ml64 = measure(lib, cl, lib.FP64, args.steps, args.warmup, local, barrier)
        ml64["solver"].close()
        ml32 = measure(lib, cl, lib.FP32, args.steps, args.warmup, local, barrier)
        ml32["solver"].close()
        accl = accuracy(lib, cl, args.large_steps, local)
        accl["workload"] = args.large_config
        large = (cl.params.nx * cl.params.ny, descl, ml64, ml32, accl)
        del cl
    forced = forcing_leg() if args.forcing and rank == 0 else None
    # the FP64 step's division by row metrics (one Markstein correction)
    # against IEEE division: 1e10 random and near-midpoint numerators over the
    # metric factors of the headline workload, and each factor against the
    # 1024 numerators within 512 ulps below +-2
    divs = metric_divisors(case)
    per = int(1e10) // len(divs) + 1
    div_check = {"divisors": len(divs), "samples": per * len(divs), "grid_pairs": 1024 * len(divs),
                 "mismatches": lib.selfcheck_division(divs, samples=per, seed=2026 + rank, device=local)}
    # the FP64 step against the oracle at the drop-in configuration's length
    par = None
    if args.parity_steps > 0 and rank == 0:
        par = parity_fp64(lib, case, args.parity_steps, local)
        par["workload"] = args.config

    if rank != 0:
        pg.destroy_process_group()
        return

    cpu = None
    if not args.no_cpu:
        n_cpu = args.cpu_steps or max(2, int(round(15.0 / (cells / 30e6))))  # ~15 s at ~30 M cell/s
        v_cpu, thr, secs = time_cpu_oracle(case, n_cpu)
        cpu = {"value": v_cpu, "unit": UNIT, "cores": thr, "kind": "port",
               "sample": f"{args.config}: {n_cpu} full-grid steps ({secs:.1f} s) of the C restatement of the "
                         f"reference step, OpenMP over rows"}

    peak, peak_kind = load_peaks()

    def form_line(m, cfg, nxy):
        return {"config": cfg, "cells": nxy, "value": m["value"], "unit": UNIT,
                "ms_per_step": m["ms"] / args.steps, "gpu_launches": m["launches"],
                "dominant_kernel": m["kernel"], "kernel_per_launch_ms": m["per_launch_ms"],
                "kernel_bytes_per_cell": m["bytes_per_cell"], "kernel_achieved_gbs": m["achieved_gbs"],
                "kernel_frac_of_measured_hbm": (m["achieved_gbs"] / peak) if m["achieved_gbs"] else None,
                "kernels_ms_per_step": m["kernels_ms_per_step"], "kernels_gbs": m["kernels_gbs"]}

    clocks = clk.summary()
    fp64_roof = None
    n64 = NCU_FP64_PER_CELL.get((args.config, m64["kernel"]))
    if n64 and m64["per_launch_ms"] and clocks.get("sm_mhz"):
        ach = n64 * cells / (m64["per_launch_ms"] * 1e-3)
        pk = FP64_LANES_PER_CYCLE * clocks["sm_mhz"] * 1e6
        fp64_roof = {"bound": "fp64", "kernel": m64["kernel"], "achieved": ach, "peak": pk,
                     "unit": "FP64 instr/s", "frac": ach / pk, "instr_per_cell": n64,
                     "pipe_busy_ncu": NCU_FP64_PIPE_BUSY.get((args.config, m64["kernel"])),
                     "peak_kind": "ncu per-cycle FP64 peak x median SM clock under load; frac counts DADD, DMUL "
                                  "and DFMA only, pipe_busy_ncu every instruction on the FP64 unit"}

    forms = {
        "fp64": form_line(m64, args.config, cells),
        "fp32": form_line(m32, args.config, cells),
        "fp32_large": form_line(m32b, f"{args.fp32_config}: {desc32}", c32.params.nx * c32.params.ny),
        "fp64_large": form_line(m64b, f"{args.fp32_config}: {desc32}", c32.params.nx * c32.params.ny),
    }
    if large:
        nl, descl, ml64, ml32, accl = large
        forms["fp64_" + args.large_config] = form_line(ml64, f"{args.large_config}: {descl}", nl)
        forms["fp32_" + args.large_config] = form_line(ml32, f"{args.large_config}: {descl}", nl)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded balanced jet + Gaussian; no dataset)",
        "config": {"workload": f"{args.config}: {desc}", "nx": p.nx, "ny": p.ny, "form": "fp64-exact",
                   "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU",
                   "l2": "no flush: each step streams >0.6 GB of fields, far above L2"},
        "hbm_gbs_step": STEP_BYTES * value / 1e9,
        "roofline": {"bound": "hbm", "kernel": m64["kernel"], "achieved": m64["achieved_gbs"], "peak": peak,
                     "unit": "GB/s", "frac": (m64["achieved_gbs"] / peak) if m64["achieved_gbs"] else None,
                     "traffic": NCU_TRAFFIC.get((args.config, m64["kernel"])), "peak_kind": peak_kind,
                     "bytes_per_cell": m64["bytes_per_cell"],
                     "per_launch_ms": m64["per_launch_ms"], "kernel_share": m64["kernel_share"],
                     "note": "the FP64 form is bound by GB300's FP64 unit (84 % busy in ncu), not by HBM: "
                             "see roofline_fp64"},
        "roofline_fp64": fp64_roof,
        "kernels_ms_per_step": m64["kernels_ms_per_step"],
        "gpu_launches": m64["launches"],
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": bytes_io, "d2h_bytes_per_step": bytes_out},
        "clocks": clocks,
        "cpu_baseline": cpu,
        "forms": forms,
        "large_case_both_forms": large[4] if large else None,
        "fp32_over_fp64": m32["value"] / m64["value"],
        "fp32_over_fp64_large": m32b["value"] / m64b["value"],
        "accuracy_fp32_vs_fp64": acc,
        "parity_fp64_vs_oracle": par,
        "division_selfcheck": div_check,
        "forcing_runner": forced,
        "ensemble_fp32_batched": ens,
        "fp32_batched_over_fp64": (ens["value"] / m64["value"]) if ens else None,
    }
    print(json.dumps(line), flush=True)
    if pg:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
