"""Synthetic cases for the SW2 step: balanced zonal jets plus seeded Gaussian
height perturbations on the latitude-longitude band, in the reference's padded
field layout ((ny+4, nx+4) doubles, halo 2, x fastest; sppde/sppde.h:131-142).

The geometry helpers restate sw.h:16,108-118,170-193 and tools.c:256-273 in
the same operation order, so that values that must agree with the reference
(latitudes, wind-table interpolation) come out bit-identical.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, replace

import numpy as np

from .formats import CaseParams

PI = 4.0 * math.atan(1.0)  # sw.h:16

PLANETS = {
    "jupiter": dict(rE=7.1492e7, rP=7.1492e7, Omega=1.7585e-4, gE=10.0),
    "saturn": dict(rE=6.0268e7, rP=6.0268e7, Omega=1.638e-4, gE=10.0),
}


def deg2rad(a):
    return a * (PI / 180.0)


def rad2deg(b):
    return b * (180.0 / PI)


def linspace_val(i, x0, x1, n):
    return x0 + float(i) * (x1 - x0) / float(n)


class Grid:
    """Per-row geometry of a polar-0 case (coords.c:35-96; init.c:279-297)."""

    def __init__(self, p: CaseParams):
        self.p = p
        self.nx, self.ny = p.nx, p.ny
        self.lon0, self.lon1 = deg2rad(p.lon0), deg2rad(p.lon1)
        self.lat0, self.lat1 = deg2rad(p.lat0), deg2rad(p.lat1)
        self.eps2 = (p.rE / p.rP) * (p.rE / p.rP)

    def latn(self, j):
        return linspace_val(j, self.lat0, self.lat1, self.ny)

    def latc(self, j):
        return (self.latn(j) + self.latn(j - 1)) / 2.0

    def lone(self, i):
        return linspace_val(i, self.lon0, self.lon1, self.nx)

    def lonc(self, i):
        return (self.lone(i) + self.lone(i - 1)) / 2.0

    def rZ(self, lat):
        t = math.tan(lat)
        return self.p.rE / math.sqrt(1.0 + (t * t) / self.eps2)

    def rM(self, lat):
        q = self.rZ(lat) / (self.p.rE * math.cos(lat))
        return self.p.rE / self.eps2 * (q * q * q)

    def g_eff(self, lat):
        pc = math.atan(1.0 / self.eps2 * math.tan(lat))
        a, b = self.p.rE * math.sin(pc), self.p.rP * math.cos(pc)
        r = self.p.rE * self.p.rP / math.sqrt(a * a + b * b)
        Om = self.p.Omega
        g0 = (self.p.gE + Om * Om * self.p.rE) * ((self.p.rE / r) * (self.p.rE / r))
        return g0 - Om * Om * r * math.cos(pc)

    def rows(self):
        """dict of per-row arrays over j = -1..ny+2 (index j+1)."""
        dlon = (self.lon1 - self.lon0) / float(self.nx)
        dlat = (self.lat1 - self.lat0) / float(self.ny)
        js = range(-1, self.ny + 3)
        out = {
            "latc": [self.latc(j) for j in js],
            "latn": [self.latn(j) for j in js],
            "dxe": [dlon * self.rZ(self.latc(j)) for j in js],
            "dxv": [dlon * self.rZ(self.latn(j)) for j in js],
            "dyn": [dlat * self.rM(self.latc(j)) for j in js],
            "dyc": [dlat * self.rM(self.latn(j - 1)) for j in js],
            "ge": [self.g_eff(self.latc(j)) for j in js],
            "gn": [self.g_eff(self.latn(j)) for j in js],
        }
        return {k: np.array(v) for k, v in out.items()}


def halo_wrap(x: np.ndarray) -> None:
    """Single-rank halo update in place (sppde_hupdate.c:274-342)."""
    ny, nx = x.shape[0] - 4, x.shape[1] - 4
    # rows are j+1, columns i+1
    x[0, 2:nx + 2] = x[ny, 2:nx + 2]          # j=-1 <- ny-1
    x[1, 2:nx + 2] = x[ny + 1, 2:nx + 2]      # j=0  <- ny
    x[ny + 2, 2:nx + 2] = x[2, 2:nx + 2]      # j=ny+1 <- 1
    x[ny + 3, 2:nx + 2] = x[3, 2:nx + 2]      # j=ny+2 <- 2
    x[:, 0] = x[:, nx]                        # i=-1 <- nx-1
    x[:, 1] = x[:, nx + 1]                    # i=0 <- nx
    x[:, nx + 2] = x[:, 2]                    # i=nx+1 <- 1
    x[:, nx + 3] = x[:, 3]                    # i=nx+2 <- 2


def linterp(xi, x, y):
    """tools.c:21-74 (linear search from the start, same arithmetic)."""
    n = len(x)
    if x[0] > xi or x[n - 1] < xi:
        raise ValueError("wind table does not cover latitude %r" % xi)
    i = 0
    while i < n - 1 and x[i + 1] <= xi:
        i += 1
    return (y[i + 1] - y[i]) * (xi - x[i]) / (x[i + 1] - x[i]) + y[i]


def wind_fields(p: CaseParams):
    """windx, windy as they stand when the reference's time loop starts:
    read_wind over all cells (io.c:199-206), halo update (init.c:232-235),
    then do_channel on the wall rows (core.c:101; calc.c:600-649)."""
    g = Grid(p)
    nx, ny = p.nx, p.ny
    wx = np.zeros((ny + 4, nx + 4))
    wy = np.zeros((ny + 4, nx + 4))
    if p.wind is not None:
        lat = [float(a) for a in p.wind[:, 0]]
        val = [float(b) for b in p.wind[:, 1]]
        for j in range(-1, ny + 3):
            wx[j + 1, :] = linterp(rad2deg(g.latc(j)), lat, val)
    halo_wrap(wx)
    halo_wrap(wy)
    I = slice(2, nx + 2)
    wy[1, I] = 0.0; wy[0, I] = 0.0
    wx[1, I] = wx[2, I]; wx[0, I] = wx[1, I]
    wy[ny + 1, I] = 0.0; wy[ny + 2, I] = 0.0; wy[ny + 3, I] = 0.0
    wx[ny + 2, I] = wx[ny + 1, I]; wx[ny + 3, I] = wx[ny + 2, I]
    return wx, wy


class SplitMix64:
    """Seeded generator for case parameters (SplitMix64, 53-bit uniform doubles)."""

    M = (1 << 64) - 1

    def __init__(self, seed: int):
        self.s = seed & self.M

    def next(self) -> int:
        self.s = (self.s + 0x9E3779B97F4A7C15) & self.M
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & self.M
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & self.M
        return z ^ (z >> 31)

    def uniform(self, lo=0.0, hi=1.0) -> float:
        return lo + (hi - lo) * ((self.next() >> 11) * (1.0 / (1 << 53)))


@dataclass
class Bump:
    lon: float  # degrees
    lat: float
    amp: float  # metres
    sigma: float  # metres


@dataclass
class Case:
    params: CaseParams
    eta: np.ndarray
    u: np.ndarray
    v: np.ndarray
    tracer: np.ndarray
    windx: np.ndarray
    windy: np.ndarray
    hB: np.ndarray
    bumps: list
    seed: int

    def fields(self):
        return self.eta, self.u, self.v, self.tracer, self.windx, self.windy, self.hB


def jet_profile(kind: str):
    if kind == "cos6":
        return lambda phi: 60.0 * np.cos(6.0 * phi)
    if kind == "cos4x100":
        return lambda phi: 100.0 * np.cos(4.0 * phi)
    if kind == "cos6+cos14":
        return lambda phi: 60.0 * np.cos(6.0 * phi) + 20.0 * np.cos(14.0 * phi)
    if kind == "none":
        return lambda phi: 0.0 * phi
    raise ValueError(kind)


def make_case(nx, ny, *, planet="jupiter", jet="cos6", sch=2, nsteps=500, seed=1,
              bumps=1, amp=(0.05, 0.05), sigma_km=(2000.0, 2000.0), lat_lim=50.0,
              h0=2.5e4, lat0=-70.0, lat1=70.0, lon0=0.0, lon1=360.0, cfl=0.3,
              efold_steps=10.0, hyper=True, Dt=None, tracer=False, wind=None,
              Tau=1e20, TracerDis=0.0) -> Case:
    """Balanced jet u(phi) at east faces, v = 0, height from geostrophic balance
    dh/dphi = -(a/g)(f u + u^2 tan(phi)/a) integrated in FP64 (trapezoid) at cell
    centres, mean height h0 (area weighted), plus seeded Gaussian bumps
    A exp(-r^2 / 2 sigma^2) with r the great-circle distance (the form of
    tools.c:104-120 and perturbs.c:377-380). Dt from CFL `cfl` on gravity-wave
    plus advective speed, summed over the two directions; nu4 so that the
    grid-scale e-folding time is `efold_steps` * Dt.

    The default CFL is 0.3: with the reference scheme (AB3, forward-backward
    pressure, semi-implicit Coriolis) a CFL of 0.4 grows a grid-scale zonal
    mode within ~100 steps on these jets, with or without hyperviscosity."""
    pl = PLANETS[planet]
    p = CaseParams(nx=nx, ny=ny, sch=sch, lon0=lon0, lon1=lon1, lat0=lat0, lat1=lat1,
                   nsteps=nsteps, depth=h0, Tau=Tau, TracerDis=TracerDis, wind=wind, **pl)
    g = Grid(p)
    rows = g.rows()
    a = pl["rE"]
    jc = np.array([g.latc(j) for j in range(1, ny + 1)])
    ujet = jet_profile(jet)(jc)
    f = 2.0 * pl["Omega"] * np.sin(jc)
    gc = rows["ge"][2:ny + 2]
    dhdphi = -(a / gc) * (f * ujet + ujet * ujet * np.tan(jc) / a)
    h = np.zeros(ny)
    dphi = np.diff(jc)
    h[1:] = np.cumsum(0.5 * (dhdphi[1:] + dhdphi[:-1]) * dphi)
    w = np.cos(jc)
    h = h - np.sum(h * w) / np.sum(w) + h0

    rng = SplitMix64(seed)
    blist = []
    for _ in range(bumps):
        lon = rng.uniform(lon0, lon1)
        lat = rng.uniform(-lat_lim, lat_lim)
        A = rng.uniform(amp[0], amp[1]) * h0
        sg = rng.uniform(sigma_km[0], sigma_km[1]) * 1e3
        blist.append(Bump(lon, lat, A, sg))

    lonc = np.array([g.lonc(i) for i in range(1, nx + 1)])
    H = np.repeat(h[:, None], nx, axis=1)
    sl, cl = np.sin(jc)[:, None], np.cos(jc)[:, None]
    for b in blist:
        l0, p0 = deg2rad(b.lon), deg2rad(b.lat)
        # exp(-x) is exactly 0.0 for x > 746, so beyond rc = sqrt(2*746) sigma
        # (with a margin for rounding) the bump adds exactly 0: only the rows
        # and cells that can be reached are evaluated, with the same result
        rc = np.sqrt(2.0 * 746.0) * b.sigma * 1.001
        rows_in = np.nonzero(np.abs(jc - p0) * a <= rc)[0]
        if rows_in.size == 0:
            continue
        j0, j1 = rows_in[0], rows_in[-1] + 1
        cosang = np.sin(p0) * sl[j0:j1] + np.cos(p0) * cl[j0:j1] * np.cos(lonc[None, :] - l0)
        near = cosang >= np.cos(min(rc / a, np.pi))
        r = a * np.arccos(np.clip(cosang[near], -1.0, 1.0))
        block = H[j0:j1]
        block[near] = block[near] + b.amp * np.exp(-(r * r) / (2.0 * b.sigma * b.sigma))
    if np.min(H) <= 0:
        raise ValueError("non-positive layer depth in synthetic case")

    eta = np.zeros((ny + 4, nx + 4))
    u = np.zeros_like(eta)
    v = np.zeros_like(eta)
    tr = np.zeros_like(eta)
    eta[2:ny + 2, 2:nx + 2] = H - h0
    u[2:ny + 2, 2:nx + 2] = ujet[:, None]
    if tracer:
        tr[2:ny + 2, 2:nx + 2] = np.exp(-((jc[:, None] - jc.mean()) / 0.2) ** 2) * (1 + 0.1 * np.cos(3 * lonc[None, :]))
    for x in (eta, u, v, tr):
        halo_wrap(x)
    wx, wy = wind_fields(p)
    hB = np.zeros_like(eta)

    if Dt is None:
        ge = rows["ge"][2:ny + 2][:, None]
        c = np.sqrt(ge * H)
        uw = np.abs(u[2:ny + 2, 2:nx + 2] + wx[2:ny + 2, 2:nx + 2])
        dxe = rows["dxe"][2:ny + 2][:, None]
        dyn = rows["dyn"][2:ny + 2][:, None]
        Dt = cfl / float(np.max((uw + c) / dxe + c / dyn))
    p.Dt = float(Dt)
    if hyper:
        dxmin = float(np.min(rows["dxe"][2:ny + 2]))
        dy = float(np.min(rows["dyn"][2:ny + 2]))
        nu4 = 1.0 / (efold_steps * p.Dt * (4.0 / dxmin ** 2 + 4.0 / dy ** 2) ** 2)
        p.hypernu = (0.0, nu4, 0.0)
    return Case(p, eta, u, v, tr, wx, wy, hB, blist, seed)


def channel_walls(wx, wy, nx, ny):
    """do_channel's changes to the winds of a band (calc.c:600-649), which the
    reference applies before its time loop (core.c:101); on a polar cap its
    wall loops run over no cells (sppde_core.c:589)."""
    I = slice(2, nx + 2)
    wy[1, I] = 0.0
    wy[0, I] = 0.0
    wx[1, I] = wx[2, I]
    wx[0, I] = wx[1, I]
    wy[ny + 1, I] = 0.0
    wy[ny + 2, I] = 0.0
    wy[ny + 3, I] = 0.0
    wx[ny + 2, I] = wx[ny + 1, I]
    wx[ny + 3, I] = wx[ny + 2, I]


def make_polar_case(n, polar, *, angle_sim=20.0, planet="jupiter", sch=2, nsteps=60, seed=1, h0=2.5e4,
                    amp=0.05, sigma_km=2500.0, beta_sp=15.0, sig_sp=1e-5, wind=None, hyper=True, tracer=False,
                    cfl=0.25, Tau=1e20, TracerDis=0.0) -> Case:
    """A polar cap (polar = 1 north, -1 south): the square -angle_sim..angle_sim
    degrees around the pole, n x n cells, at rest with a seeded Gaussian
    height bump; winds from the table (turned around the pole, damped in the
    sponge beyond beta_sp degrees) as the reference's reader builds them,
    computed by the C restatement (sw2_gb300.hostlib). Dt from CFL `cfl` on
    the gravity-wave speed plus the largest wind."""
    import os
    import tempfile

    from . import formats, hostlib

    pl = PLANETS[planet]
    p = CaseParams(nx=n, ny=n, sch=sch, nsteps=nsteps, depth=h0, Tau=Tau, TracerDis=TracerDis, wind=wind, **pl)
    p.polar, p.angleSim, p.BetaSp, p.SigSp = polar, angle_sim, beta_sp, sig_sp
    p.lon0 = p.lat0 = -angle_sim
    p.lon1 = p.lat1 = angle_sim
    rng = SplitMix64(seed)
    b = Bump(rng.uniform(-angle_sim / 2, angle_sim / 2), rng.uniform(-angle_sim / 2, angle_sim / 2), amp * h0,
             sigma_km * 1e3)
    d = deg2rad(2.0 * angle_sim) / n
    lc = np.array([deg2rad(-angle_sim) + (k - 0.5) * d for k in range(1, n + 1)])
    R = pl["rE"] * pl["rE"] / pl["rP"]
    cosang = (np.sin(deg2rad(b.lat)) * np.sin(lc)[:, None] +
              np.cos(deg2rad(b.lat)) * np.cos(lc)[:, None] * np.cos(lc[None, :] - deg2rad(b.lon)))
    r = R * np.arccos(np.clip(cosang, -1.0, 1.0))
    eta = np.zeros((n + 4, n + 4))
    eta[2:-2, 2:-2] = b.amp * np.exp(-(r * r) / (2.0 * b.sigma * b.sigma))
    u, v, tr = np.zeros_like(eta), np.zeros_like(eta), np.zeros_like(eta)
    if tracer:
        tr[2:-2, 2:-2] = np.exp(-(r * r) / (2.0 * (3 * b.sigma) ** 2))
    for x in (eta, u, v, tr):
        halo_wrap(x)
    p.Dt = 100.0
    with tempfile.TemporaryDirectory() as wd:
        path = os.path.join(wd, "c.sw")
        formats.write_sw(path, p)
        wx, wy = hostlib.Case(path).winds(beta_sp)
    g = float(pl["gE"]) * 1.2
    dx = R * d * np.cos(deg2rad(angle_sim) * 1.5)
    c = np.sqrt(g * h0 * (1 + amp)) + float(np.max(np.abs(wx)) + np.max(np.abs(wy)))
    p.Dt = float(cfl * dx / (2 * c))
    if hyper:
        nu4 = 1.0 / (10.0 * p.Dt * (8.0 / dx ** 2) ** 2)
        p.hypernu = (0.0, nu4, 0.0)
    return Case(p, eta, u, v, tr, wx, wy, np.zeros_like(eta), [b], seed)


def config_case(name: str, seed: int = 1, **over) -> Case:
    """The benchmark configurations by name (sizes, physics and step counts)."""
    if name == "band256":      # plain FP64, CPU-runnable
        kw = dict(nx=256, ny=128, planet="jupiter", jet="cos6", sch=2, nsteps=500, bumps=1,
                  amp=(0.05, 0.05), sigma_km=(2000.0, 2000.0))
    elif name == "band2048":   # plain FP64 drop-in size
        kw = dict(nx=2048, ny=1024, planet="jupiter", jet="cos6", sch=2, nsteps=2000, bumps=1,
                  amp=(0.05, 0.05), sigma_km=(2000.0, 2000.0))
    elif name == "saturn4096":  # precision form
        kw = dict(nx=4096, ny=2048, planet="saturn", jet="cos4x100", sch=1, nsteps=2000, bumps=3,
                  amp=(0.03, 0.03), sigma_km=(1500.0, 1500.0))
    elif name == "band8192":
        kw = dict(nx=8192, ny=4096, planet="jupiter", jet="cos6+cos14", sch=2, nsteps=1000, bumps=200,
                  amp=(0.005, 0.02), sigma_km=(500.0, 1500.0))
    else:
        raise ValueError(name)
    kw.update(over)
    return make_case(seed=seed, **kw)


def ensemble_members(seed: int = 7):
    """64-member uneven ensemble: 16 x 512x256, 24 x 1024x512, 24 x 2048x1024,
    Van Leer limiter, amplitude U[0.01,0.08] h0, sigma U[1000,3000] km."""
    out = []
    sizes = [(512, 256)] * 16 + [(1024, 512)] * 24 + [(2048, 1024)] * 24
    for m, (nx, ny) in enumerate(sizes):
        out.append((nx, ny, dict(planet="jupiter", jet="cos6", sch=3, nsteps=1000, bumps=1,
                                 amp=(0.01, 0.08), sigma_km=(1000.0, 3000.0), seed=seed * 1000 + m)))
    return out


def forcing_band(nsteps: int = 30, nx: int = 1024, ny: int = 512) -> CaseParams:
    """A band with Gaussian mass injections in every step (add_Gaussians,
    perturbs.c:22-195), run from the reference's own initial state (LoadFrom
    0: zero fields, forcing at t0): a ramped static injection, a moving one
    across the periodic seam that injects tracer, and one against the northern
    wall moving in degrees per second; sizes in degrees. Table rows are the
    reference's 12 Gaussian columns (t0, t1, tau, lon, lat, isdegvel, vel, Q,
    isdegsize, sigma, radius, inject_tracer)."""
    p = make_case(nx, ny, sch=2, seed=36, jet="none", bumps=0, lat0=-60.0, lat1=60.0, nsteps=nsteps).params
    p.nsteps, p.SaveEvery, p.IteInfo, p.LoadFrom = nsteps, nsteps, nsteps, 0
    p.gaussians = [[0.0, 40 * p.Dt, 2 * p.Dt, 100.0, 10.0, 0, 0.0, 2.0e13 / p.Dt, 1, 2.0, 6.0, 0.0],
                   [0.0, 40 * p.Dt, 0.0, 2.0, -20.0, 0, -60.0, 1.5e13 / p.Dt, 1, 1.5, 5.0, 1.0],
                   [0.0, 40 * p.Dt, 3 * p.Dt, 250.0, 50.0, 1, 0.01, 1.0e13 / p.Dt, 1, 3.0, 9.0, 0.5]]
    return p
