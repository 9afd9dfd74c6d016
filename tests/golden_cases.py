"""Loader for the committed golden fixtures (tests/golden/*.npz + manifest.json)."""
from __future__ import annotations

import json
import os

import numpy as np

from sw2_gb300.cases import Case, halo_wrap
from sw2_gb300.formats import CaseParams

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def manifest():
    with open(os.path.join(GOLDEN, "manifest.json")) as fh:
        return json.load(fh)


def params_of(entry) -> CaseParams:
    d = dict(entry["params"])
    nu = d.pop("hypernu")
    wind = d.pop("wind")
    p = CaseParams(**{k: v for k, v in d.items() if k in CaseParams.__dataclass_fields__})
    p.hypernu = tuple(nu)
    p.wind = None if wind is None else np.array(wind)
    return p


def padded(inner):
    ny, nx = inner.shape
    a = np.zeros((ny + 4, nx + 4))
    a[2:-2, 2:-2] = inner
    halo_wrap(a)
    return a


def load_case(name):
    entry = manifest()[name]
    p = params_of(entry)
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    f = {k: padded(z["init_" + k]) for k in ("eta", "u", "v", "tracer")}
    wx = z["windx"] if "windx" in z else np.zeros_like(f["eta"])
    wy = z["windy"] if "windy" in z else np.zeros_like(f["eta"])
    case = Case(p, f["eta"], f["u"], f["v"], f["tracer"], wx, wy, np.zeros_like(f["eta"]), [], 0)
    frames = []
    k = 0
    while f"f{k}_eta" in z:
        frames.append({n: z[f"f{k}_{n}"] for n in ("eta", "u", "v", "tracer")})
        k += 1
    return entry, case, frames


def array_cases():
    return sorted(n for n in manifest() if n.startswith("g"))


def polar_cases():
    """Polar caps run by the reference from an initial frame (no oracle pin)."""
    return sorted(n for n, e in manifest().items() if e.get("polar"))


def forcing_cases():
    """Cases run by the reference from its own initial state, with forcing."""
    return sorted(n for n, e in manifest().items() if e.get("forcing") and n.startswith("f"))


def forcing_params(name) -> CaseParams:
    entry = manifest()[name]
    p = params_of(entry)
    p.vortices = [list(r) for r in entry["vortices"]]
    p.gaussians = [list(r) for r in entry["gaussians"]]
    p.nsteps = entry["nsteps"]
    return p


def forcing_frames(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    frames = []
    k = 0
    while f"f{k}_eta" in z:
        frames.append({n: z[f"f{k}_{n}"] for n in ("eta", "u", "v", "tracer", "perturbs", "t")})
        k += 1
    return frames
