#!/usr/bin/env python3
"""Time the reference's own step (oracle/_ref/SW, built from its sources by
oracle/Makefile) against the C restatement in oracle/ on one host core.

Runs only where the reference sources are present. Both run the same case
from the same initial frame: the reference as `SW 1 1 <case> out` with
LoadFrom 1 and no output until the last step, the restatement through
oracle.Oracle with OMP_NUM_THREADS=1 (set before the library loads). The
reference's wall time includes its start-up (parsing, geometry, one frame
read and one frame write); the restatement's timed region is the steps only,
so the start-up is measured separately with a 1-step reference run and
subtracted.

    python oracle/time_ref_vs_port.py [--case band256] [--steps 100]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

os.environ["OMP_NUM_THREADS"] = "1"
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from oracle import oracle as orc  # noqa: E402
from sw2_gb300 import cases, formats  # noqa: E402

REF_BIN = os.path.join(ROOT, "oracle", "_ref", "SW")
REF_PATH = os.path.join(ROOT, "oracle", "_ref", "bin")


def run_ref(case, nsteps, wd):
    p = case.params
    p.nsteps, p.SaveEvery, p.IteInfo, p.LoadFrom = nsteps, nsteps, nsteps, 1
    os.makedirs(os.path.join(wd, "out"), exist_ok=True)
    formats.write_sw(os.path.join(wd, "t.sw"), p)
    fr = [np.zeros_like(case.eta) for _ in range(5)]
    for dst, src in zip(fr, (case.eta, case.u, case.v, case.tracer)):
        dst[2:-2, 2:-2] = src[2:-2, 2:-2]
    formats.write_frame(os.path.join(wd, "out", "t.0001.bin"), 0, 0.0, p.nx, p.ny, fr)
    env = dict(os.environ, PATH=REF_PATH + os.pathsep + os.environ["PATH"])
    t0 = time.perf_counter()
    r = subprocess.run([REF_BIN, "1", "1", "t", "out"], cwd=wd, env=env, capture_output=True, text=True)
    dt = time.perf_counter() - t0
    if r.returncode != 0 or "CRASH" in r.stdout + r.stderr:
        raise RuntimeError(r.stdout[-2000:] + r.stderr[-2000:])
    return dt


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", default="band256")
    ap.add_argument("--steps", type=int, default=100)
    a = ap.parse_args()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "all", "ref"], check=True)
    if not os.path.exists(REF_BIN):
        raise SystemExit("reference not built (sources absent?)")
    case = cases.config_case(a.case, seed=1)
    p = case.params
    with tempfile.TemporaryDirectory() as wd:
        t_one = run_ref(cases.config_case(a.case, seed=1), 1, wd)
    with tempfile.TemporaryDirectory() as wd:
        t_all = run_ref(case, a.steps + 1, wd)
    ref_s = max(t_all - t_one, 1e-9)
    o = orc.Oracle(cases.config_case(a.case, seed=1).params)
    o.load(case.fields())
    o.step(1)
    t0 = time.perf_counter()
    rc, _ = o.step(a.steps)
    port_s = time.perf_counter() - t0
    if rc:
        raise RuntimeError(f"oracle aborted rc={rc}")
    cells = p.nx * p.ny * a.steps
    print(json.dumps({"case": a.case, "steps": a.steps, "threads": orc.threads(),
                      "reference_cell_updates_per_s": cells / ref_s, "port_cell_updates_per_s": cells / port_s,
                      "port_over_reference": ref_s / port_s}))


if __name__ == "__main__":
    main()
