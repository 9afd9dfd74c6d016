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
    "coriolis_u": 8 * (3 + 1),
    "coriolis_v": 8 * (3 + 1),
    "lape_pass1": 8 * (1 + 2),
    "lape_pass2": 8 * (2 + 1),
    "lapv_pass1": 8 * (2 + 2),
    "lapv_pass2": 8 * (2 + 2),
    "hyper_add": 8 * (4 + 1),
    "geofactor": 8 * (3 + 1),
    "add": 8 * (2 + 1),
    "cfl": 8 * 2,
    "range": 8 * 1,
}
# The whole step: read eta u v, write eta u v, read two history levels of
# three tendencies, write one (SURVEY-style count for the FP64 form).
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
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_rank{device}.csv") if os.path.isdir(
            os.path.join(ROOT, "gpurun_out")) else f"/tmp/sw2g_clocks_{os.getpid()}.csv"

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
        sm = [int(r[1]) for r in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": int(rows[0][2]), "reasons": reasons,
                "samples": len(rows)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="band2048")
    ap.add_argument("--cpu-steps", type=int, default=None, help="oracle steps for the CPU baseline sample")
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

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
    s = lib.Solver(p, device=local)
    s.upload(*case.fields())

    def barrier():
        torch.cuda.synchronize(local)
        if pg:
            pg.barrier()

    # warm-up
    assert s.step(args.warmup) == lib.OK

    # timed region: K steps, device time by CUDA events on the library's stream
    barrier()
    with ClockSampler(local) as clk:
        rc = s.step(args.steps)
        barrier()
    if rc != lib.OK:
        raise RuntimeError(f"step failed: {lib.status_string(rc)} at step {s.error_step()}")
    ms = s.last_step_ms()
    launches = s.last_launches()
    if pg:
        t = torch.tensor([ms], device=f"cuda:{local}")
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        ms = float(t.item())
    value = cells * args.steps * ws / (ms * 1e-3)

    # per-kernel device times (second timed pass, timers on)
    s.timers(True)
    s.timers_reset()
    assert s.step(args.steps) == lib.OK
    table = s.timer_table()
    s.timers(False)
    name, (nl, kms) = max(table.items(), key=lambda kv: kv[1][1])
    per_launch_ms = kms / nl
    kb = KERNEL_BYTES.get(name)
    peak, peak_kind = load_peaks()
    achieved = (kb * cells / (per_launch_ms * 1e-3) / 1e9) if kb else None
    total_kernel_ms = sum(v[1] for v in table.values())

    # end to end through the C ABI: every step uploads the state from pinned
    # host memory, steps once, and downloads it again
    W, H = p.nx + 4, p.ny + 4
    host = [torch.empty((H, W), dtype=torch.float64, pin_memory=True).numpy() for _ in range(3)]
    d = s.download()
    for h, k in zip(host, ("eta", "u", "v")):
        h[...] = d[k]
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        s.upload(host[0], host[1], host[2], mode=lib.UPLOAD_CONTINUE)
        if s.step(1) != lib.OK:
            raise RuntimeError("e2e step failed")
        lib.load().sw2g_download(s.h, *[lib._ptr(h) for h in host], None)
    barrier()
    e2e_s = time.perf_counter() - t0
    if pg:
        t = torch.tensor([e2e_s], device=f"cuda:{local}")
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = cells * args.steps * ws / e2e_s
    bytes_io = 3 * W * H * 8

    if rank != 0:
        pg.destroy_process_group()
        return

    cpu = None
    if not args.no_cpu:
        n_cpu = args.cpu_steps or max(2, int(round(15.0 / (cells / 40e6))))  # ~15 s at ~40 M cell/s
        v_cpu, thr, secs = time_cpu_oracle(case, n_cpu)
        cpu = {"value": v_cpu, "unit": UNIT, "cores": thr, "kind": "port",
               "sample": f"{args.config}: {n_cpu} full-grid steps ({secs:.1f} s) of the C restatement of the "
                         f"reference step, OpenMP over rows"}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded balanced jet + Gaussian; no dataset)",
        "config": {"workload": f"{args.config}: {desc}", "nx": p.nx, "ny": p.ny, "form": "fp64-exact",
                   "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU",
                   "l2": "no flush: the step streams ~38 padded FP64 fields (>0.6 GB) per step, far above L2"},
        "hbm_gbs_step": STEP_BYTES * value / 1e9,
        "roofline": {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": None,
                     "peak_kind": peak_kind, "bytes_per_cell": kb,
                     "per_launch_ms": per_launch_ms, "kernel_share": kms / total_kernel_ms},
        "kernels_ms_per_step": {k: v[1] / args.steps for k, v in sorted(table.items(), key=lambda kv: -kv[1][1])},
        "gpu_launches": launches,
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": bytes_io, "d2h_bytes_per_step": bytes_io},
        "clocks": clk.summary(),
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)
    if pg:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
