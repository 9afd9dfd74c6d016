"""Run a synthetic SW2 case on the GPU through the C ABI.

    python -m sw2_gb300.run --config band2048 --precision fp64 --steps 20
    python -m sw2_gb300.run --ensemble --steps 20
    python -m sw2_gb300.run --config band8192 --steps 1000 --compare-fp32

--config names one of the seeded workloads of sw2_gb300.cases (band256,
band2048, saturn4096, band8192); --ensemble runs the 64-member batch of
uneven grids (FP32 form, one launch per phase over all members). Prints one
JSON line: device time per step, cell-updates/s, launches, status, and the
energy/mass diagnostic of the final state (single cases).
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import cases, lib


def run_case(name, precision, steps, warmup, seed, timers):
    case = cases.config_case(name, seed=seed)
    p = case.params
    flags = lib.FLAG_VANLEER_SAFE if p.sch == 3 else 0
    s = lib.Solver(p, precision=precision, flags=flags)
    s.upload(*case.fields())
    if warmup and s.step(warmup) != lib.OK:
        raise RuntimeError(f"warm-up failed at step {s.error_step()}")
    if timers:
        s.timers(True)
    rc = s.step(steps)
    ms = s.last_step_ms()
    out = {"config": name, "nx": p.nx, "ny": p.ny, "precision": "fp64" if precision == lib.FP64 else "fp32",
           "steps": steps, "status": lib.status_string(rc), "ms_per_step": ms / max(steps, 1),
           "cell_updates_per_s": p.nx * p.ny * steps / (ms * 1e-3) if ms > 0 else None,
           "launches": s.last_launches()}
    if rc != lib.OK:
        out["error_step"] = s.error_step()
    else:
        ke, ape, mass = s.diag()
        out.update(ke=ke, ape=ape, mass=mass)
    if timers:
        out["kernels_ms"] = {k: v[1] for k, v in s.timer_table().items()}
    s.close()
    return out


def compare_forms(name, steps, seed):
    """Both forms of the step from the same synthetic case: throughput of each
    (device time of one call of `steps` steps) and, after those steps, the
    relative L2 error of h = eta + depth, u and v of the FP32 form against the
    FP64 form, and the relative mass and energy drift of each."""
    case = cases.config_case(name, seed=seed)
    p = case.params
    flags = lib.FLAG_VANLEER_SAFE if p.sch == 3 else 0
    out = {"config": name, "nx": p.nx, "ny": p.ny, "steps": steps}
    res = {}
    for nm, prec in (("fp64", lib.FP64), ("fp32", lib.FP32)):
        s = lib.Solver(p, precision=prec, flags=flags)
        s.upload(*case.fields())
        k0, a0, m0 = s.diag()
        rc = s.step(steps)
        if rc != lib.OK:
            raise RuntimeError(f"{nm}: {lib.status_string(rc)} at step {s.error_step()}")
        ms = s.last_step_ms()
        k1, a1, m1 = s.diag()
        out[nm] = {"ms_per_step": ms / steps, "cell_updates_per_s": p.nx * p.ny * steps / (ms * 1e-3),
                   "mass_drift": (m1 - m0) / m0, "energy_drift": ((k1 + a1) - (k0 + a0)) / (k0 + a0)}
        res[nm] = s.download()
        s.close()
    a, b = res["fp32"], res["fp64"]
    inner = (slice(2, -2), slice(2, -2))
    out["h_rel_l2"] = float(np.linalg.norm((a["eta"] - b["eta"])[inner]) / np.linalg.norm((b["eta"] + p.depth)[inner]))
    for k in ("u", "v"):
        out[f"{k}_rel_l2"] = float(np.linalg.norm((a[k] - b[k])[inner]) / np.linalg.norm(b[k][inner]))
    out["status"] = lib.status_string(lib.OK)
    return out


def run_ensemble(steps, warmup, seed):
    solvers, cells = [], 0
    for nx, ny, kw in cases.ensemble_members(seed):
        c = cases.make_case(nx, ny, **kw)
        s = lib.Solver(c.params, precision=lib.FP32, flags=lib.FLAG_VANLEER_SAFE)
        s.upload(*c.fields())
        solvers.append(s)
        cells += nx * ny
    b = lib.Batch(solvers)
    if warmup and b.step(warmup) != lib.OK:
        raise RuntimeError(f"warm-up failed: {b.error()}")
    rc = b.step(steps)
    ms = b.last_step_ms()
    out = {"ensemble": len(solvers), "cells_per_step": cells, "steps": steps, "status": lib.status_string(rc),
           "ms_per_step": ms / max(steps, 1),
           "cell_updates_per_s": cells * steps / (ms * 1e-3) if ms > 0 else None,
           "launches": b.last_launches()}
    b.close()
    for s in solvers:
        s.close()
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--config", default="band2048")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32"])
    ap.add_argument("--ensemble", action="store_true")
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--timers", action="store_true", help="per-kernel device timers (direct launches)")
    ap.add_argument("--compare-fp32", action="store_true",
                    help="run both forms from the same case and report the FP32 form's error")
    a = ap.parse_args(argv)
    lib.load()
    if a.compare_fp32:
        out = compare_forms(a.config, a.steps, a.seed)
    elif a.ensemble:
        out = run_ensemble(a.steps, a.warmup, a.seed if a.seed != 1 else 7)
    else:
        prec = lib.FP64 if a.precision == "fp64" else lib.FP32
        out = run_case(a.config, prec, a.steps, a.warmup, a.seed, a.timers)
    print(json.dumps(out), flush=True)
    return 0 if out["status"] == lib.status_string(lib.OK) else 1


if __name__ == "__main__":
    raise SystemExit(main())
