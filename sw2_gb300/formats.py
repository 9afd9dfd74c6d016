"""SW2 file formats: `.sw` case files and MAGICSW2 binary frames.

The case writer emits the tags in the fixed order the reference reader
expects (init.c:48-237); numeric values are written with 17 significant
digits so that the reader's sscanf("%le") recovers the exact doubles.
Frames follow io.c:27-64 and sppde/sppde_binary_files.c:34-60: int magic 28,
int nstep, double t, int nx, int ny, then five records (eta, u, v, tracer,
perturbs), each an int 15 followed by (nx+4)*(ny+4) native doubles.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

import numpy as np

MAGIC_SW1 = 27
MAGIC_SW2 = 28
MAGIC_FIELD = 15


@dataclass
class CaseParams:
    """Parsed content of a (polar 0) `.sw` case, in the reference's units."""

    nx: int
    ny: int
    sch: int = 2
    lon0: float = 0.0          # degrees
    lon1: float = 360.0
    lat0: float = -70.0
    lat1: float = 70.0
    t0: float = 0.0
    nsteps: int = 10
    Dt: float = 100.0
    CFL: float = 0.4
    Tau: float = 1e20          # > 1e10 disables damping (init.c:110-114)
    hypernu: tuple = (0.0, 0.0, 0.0)  # as entered; nu4 positive (init.c:120 negates)
    IteInfo: int = 1
    SaveEvery: int = 1
    LoadFrom: int = 0
    Omega: float = 1.7585e-4
    rE: float = 7.1492e7
    rP: float = 7.1492e7
    gE: float = 10.0
    depth: float = 2.5e4
    TracerDis: float = 0.0
    wind: np.ndarray | None = None  # (n, 2) table: latitude deg, u m/s
    # forcing tables (perturbs.c): rows of 7 vortex values
    # (t0, lon, lat, a, b, Umax, n) and 12 Gaussian values (t0, t1, tau, lon,
    # lat, isdegvel, vel, Q, isdegsize, sigma, radius, inject_tracer)
    vortices: list = field(default_factory=list)
    gaussians: list = field(default_factory=list)
    # polar caps (init.c:66-79, 154-162): polar = +-1 replaces lon0..lat1 by
    # -angleSim..angleSim (degrees) and nx, ny by n; BetaSp (degrees) and SigSp
    # set the sponge
    polar: int = 0
    angleSim: float = 0.0
    BetaSp: float = 0.0
    SigSp: float = 0.0
    extra: dict = field(default_factory=dict)

    @property
    def t1(self) -> float:
        # N = (int)((t1-t0)/Dt) (init.c:109); half a step of slack keeps the cast exact
        return self.t0 + (self.nsteps + 0.5) * self.Dt


def _g(x: float) -> str:
    return repr(float(x))


def write_sw(path: str, p: CaseParams) -> None:
    """Write a fully expanded `.sw` case (no m4 macros needed)."""
    nu = p.hypernu
    if p.polar:
        geo = [f"polar {p.polar}", f"angleSim {_g(p.angleSim)}", f"n {p.nx}"]
    else:
        geo = ["polar 0", f"lon0 {_g(p.lon0)}", f"lon1 {_g(p.lon1)}", f"lat0 {_g(p.lat0)}", f"lat1 {_g(p.lat1)}",
               f"nx {p.nx}", f"ny {p.ny}"]
    lines = [
        f"sch {p.sch}",
        *geo,
        f"t0 {_g(p.t0)}",
        f"t1 {_g(p.t1)}",
        f"Dt {_g(p.Dt)}",
        f"CFL {_g(p.CFL)}",
        f"Tau {_g(p.Tau)}",
        f"Hypernu {_g(nu[0])} {_g(nu[1])} {_g(nu[2])}",
        f"IteInfo {p.IteInfo}",
        f"SaveEvery {p.SaveEvery}",
        f"LoadFrom {p.LoadFrom}",
        "reftype 0",
        f"Omega {_g(p.Omega)}",
        f"rE {_g(p.rE)}",
        f"rP {_g(p.rP)}",
        f"gE {_g(p.gE)}",
        f"depth {_g(p.depth)}",
        *([f"BetaSp {_g(p.BetaSp)}", f"SigSp {_g(p.SigSp)}"] if p.polar else []),
        "geoeq 0",
        str(len(p.vortices)), "7",
        *[" ".join(_g(x) for x in row) for row in p.vortices],
        str(len(p.gaussians)), "12",
        *[" ".join(_g(x) for x in row) for row in p.gaussians],
        f"TracerDis {_g(p.TracerDis)}",
    ]
    # a zero table wide enough for the halo-row latitudes of any band (io.c:201-203)
    w = p.wind if p.wind is not None else np.array([[-180.0, 0.0], [180.0, 0.0]])
    lines += [str(len(w)), "2"] + [f"{_g(a)} {_g(b)}" for a, b in w]
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def write_frame(path: str, nstep: int, t: float, nx: int, ny: int, fields) -> None:
    """Write a MAGICSW2 frame; `fields` = (eta, u, v, tracer, perturbs), each padded."""
    S = (nx + 4) * (ny + 4)
    with open(path, "wb") as fh:
        fh.write(struct.pack("=iidii", MAGIC_SW2, nstep, t, nx, ny))
        for f in fields:
            a = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
            if a.size != S:
                raise ValueError(f"field has {a.size} values, frame needs {S}")
            fh.write(struct.pack("=i", MAGIC_FIELD))
            fh.write(a.tobytes())


def read_frame(path: str):
    """Read a MAGICSW1/MAGICSW2 frame -> (nstep, t, nx, ny, dict of padded (ny+4, nx+4) arrays)."""
    with open(path, "rb") as fh:
        raw = fh.read()
    magic, nstep, t, nx, ny = struct.unpack_from("=iidii", raw, 0)
    if magic not in (MAGIC_SW1, MAGIC_SW2):
        raise ValueError(f"wrong frame magic {magic}")
    names = ["eta", "u", "v", "perturbs"] if magic == MAGIC_SW1 else ["eta", "u", "v", "tracer", "perturbs"]
    S = (nx + 4) * (ny + 4)
    off = struct.calcsize("=iidii")
    out = {}
    for nm in names:
        (fm,) = struct.unpack_from("=i", raw, off)
        if fm != MAGIC_FIELD:
            raise ValueError(f"wrong field magic {fm}")
        off += 4
        out[nm] = np.frombuffer(raw, dtype=np.float64, count=S, offset=off).reshape(ny + 4, nx + 4).copy()
        off += 8 * S
    if magic == MAGIC_SW1:
        out["tracer"] = np.zeros((ny + 4, nx + 4))
    return nstep, t, nx, ny, out
