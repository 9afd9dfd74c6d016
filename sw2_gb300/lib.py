"""ctypes binding of libsw2g.so (the C ABI in include/sw2g.h).

There is no fallback: if the library is missing or no GPU is present, every
call raises. `Solver` mirrors the reference's step interface: create from the
parsed case, upload the fields in the reference's padded layout, step, read
back, and query the energy diagnostic.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .formats import CaseParams

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsw2g.so")

OK, ERR_BAD_ARG, ERR_CFL, ERR_NONFINITE, ERR_TIMEOUT, ERR_CUDA, ERR_NOMEM, ERR_STATE, ERR_FORCING = range(9)
FP64, FP32 = 0, 1
FLAG_VANLEER_SAFE = 0x1
FLAG_RADIANS = 0x2
FLAG_SIGMA = 0x4
FLAG_LAPE_ETA = 0x8
UPLOAD_RAW, UPLOAD_FRAME, UPLOAD_CONTINUE = 0, 1, 2
BATCH_MAX = 96

SYMBOLS = [
    "sw2g_status_string", "sw2g_create", "sw2g_upload", "sw2g_step", "sw2g_error_step", "sw2g_download",
    "sw2g_diag", "sw2g_reset_ab", "sw2g_steps_done", "sw2g_device_field", "sw2g_stream", "sw2g_last_launches",
    "sw2g_destroy", "sw2g_last_step_ms", "sw2g_timers_enable", "sw2g_timers_reset", "sw2g_timers_count",
    "sw2g_timer_read", "sw2g_selfcheck_division", "sw2g_add_field", "sw2g_set_field_where",
    "sw2g_apply_channel", "sw2g_step_open", "sw2g_step_close", "sw2g_checkpoint_doubles",
    "sw2g_checkpoint_save", "sw2g_checkpoint_load", "sw2g_test_tile_timeout", "sw2g_step_host",
    "sw2g_selfcheck_add",
]


class Case(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("sch", ctypes.c_int),
                ("lon0", ctypes.c_double), ("lon1", ctypes.c_double),
                ("lat0", ctypes.c_double), ("lat1", ctypes.c_double),
                ("Omega", ctypes.c_double), ("rE", ctypes.c_double), ("rP", ctypes.c_double),
                ("gE", ctypes.c_double), ("depth", ctypes.c_double),
                ("Dt", ctypes.c_double), ("courant", ctypes.c_double),
                ("tau", ctypes.c_double), ("tracer_dis", ctypes.c_double),
                ("hypernu", ctypes.c_double * 3), ("flags", ctypes.c_uint),
                ("polar", ctypes.c_int), ("beta_sponge", ctypes.c_double), ("sigma_sponge", ctypes.c_double)]


class Gaussian(ctypes.Structure):
    """sw2g_gaussian: one injection evaluated on the device (sw2g_add_gaussian)."""
    _fields_ = [("lon", ctypes.c_double), ("lat", ctypes.c_double), ("amp", ctypes.c_double),
                ("sigma", ctypes.c_double), ("radius", ctypes.c_double), ("inject", ctypes.c_double),
                ("volume", ctypes.c_double), ("images", ctypes.c_int)]


class SW2GError(RuntimeError):
    def __init__(self, code, what, step=-1):
        super().__init__(f"{what}: {status_string(code)} (status {code}, step {step})")
        self.code = code
        self.step = step


_lib = None


def load():
    """Load the library (no rebuild, no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} not built: run `python -m sw2_gb300.build`")
        L = ctypes.CDLL(LIB_PATH)
        vp, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)
        L.sw2g_status_string.restype = ctypes.c_char_p
        L.sw2g_status_string.argtypes = [ctypes.c_int]
        L.sw2g_create.argtypes = [ctypes.POINTER(Case), ctypes.c_int, ctypes.c_int, ctypes.POINTER(vp)]
        L.sw2g_upload.argtypes = [vp, dp, dp, dp, dp, dp, dp, dp, ctypes.c_int]
        L.sw2g_step.argtypes = [vp, ctypes.c_int]
        L.sw2g_step_host.argtypes = [vp, dp, dp, dp, ctypes.c_int]
        L.sw2g_error_step.argtypes = [vp]
        L.sw2g_download.argtypes = [vp, dp, dp, dp, dp]
        L.sw2g_diag.argtypes = [vp, dp, dp, dp]
        L.sw2g_reset_ab.argtypes = [vp]
        L.sw2g_steps_done.restype = ctypes.c_longlong
        L.sw2g_steps_done.argtypes = [vp]
        L.sw2g_device_field.restype = vp
        L.sw2g_device_field.argtypes = [vp, ctypes.c_int]
        L.sw2g_stream.restype = vp
        L.sw2g_stream.argtypes = [vp]
        L.sw2g_last_launches.restype = ctypes.c_longlong
        L.sw2g_last_launches.argtypes = [vp]
        L.sw2g_destroy.argtypes = [vp]
        L.sw2g_last_step_ms.restype = ctypes.c_double
        L.sw2g_last_step_ms.argtypes = [vp]
        L.sw2g_timers_enable.argtypes = [vp, ctypes.c_int]
        L.sw2g_timers_reset.argtypes = [vp]
        L.sw2g_timers_reset.restype = None
        L.sw2g_timers_count.argtypes = [vp]
        L.sw2g_timer_read.argtypes = [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_char_p),
                                      ctypes.POINTER(ctypes.c_longlong), dp]
        _lib = L
    return _lib


def selfcheck_division(divisors, samples: int, seed: int = 1, device: int = 0) -> int:
    """Mismatches of the step's metric division against IEEE division."""
    L = load()
    L.sw2g_selfcheck_division.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.c_longlong,
                                          ctypes.c_ulonglong, ctypes.c_int, ctypes.POINTER(ctypes.c_longlong)]
    d = np.ascontiguousarray(divisors, dtype=np.float64)
    out = ctypes.c_longlong()
    rc = L.sw2g_selfcheck_division(_ptr(d), len(d), int(samples), int(seed), int(device), ctypes.byref(out))
    if rc != OK:
        raise SW2GError(rc, "sw2g_selfcheck_division")
    return out.value


def selfcheck_add(samples: int, seed: int = 1, device: int = 0) -> int:
    """Mismatches of the step's integer-pipe additions against the FP64 unit."""
    L = load()
    L.sw2g_selfcheck_add.argtypes = [ctypes.c_longlong, ctypes.c_ulonglong, ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_longlong)]
    out = ctypes.c_longlong()
    rc = L.sw2g_selfcheck_add(int(samples), int(seed), int(device), ctypes.byref(out))
    if rc != OK:
        raise SW2GError(rc, "sw2g_selfcheck_add")
    return out.value


def status_string(code: int) -> str:
    return load().sw2g_status_string(int(code)).decode()


def case_struct(p: CaseParams, flags: int = 0) -> Case:
    c = Case()
    c.nx, c.ny, c.sch = p.nx, p.ny, p.sch
    c.lon0, c.lon1, c.lat0, c.lat1 = p.lon0, p.lon1, p.lat0, p.lat1
    if getattr(p, "polar", 0):  # init.c:66-74: the square -angleSim..angleSim around the pole
        c.lon0 = c.lat0 = -p.angleSim
        c.lon1 = c.lat1 = p.angleSim
    c.Omega, c.rE, c.rP, c.gE, c.depth = p.Omega, p.rE, p.rP, p.gE, p.depth
    c.Dt, c.courant, c.tau, c.tracer_dis = p.Dt, p.CFL, p.Tau, p.TracerDis
    for k in range(3):
        c.hypernu[k] = p.hypernu[k]
    c.flags = flags
    c.polar = getattr(p, "polar", 0)
    c.beta_sponge = getattr(p, "BetaSp", 0.0)
    c.sigma_sponge = getattr(p, "SigSp", 0.0)
    return c


def _ptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Solver:
    """One GPU run of a case (a sw2g context)."""

    def __init__(self, params: CaseParams, precision: int = FP64, device: int = 0, flags: int = 0):
        self.params = params
        self.nx, self.ny = params.nx, params.ny
        self._c = case_struct(params, flags)
        h = ctypes.c_void_p()
        rc = load().sw2g_create(ctypes.byref(self._c), precision, device, ctypes.byref(h))
        if rc != OK:
            raise SW2GError(rc, "sw2g_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            load().sw2g_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _check(self, rc, what):
        if rc != OK:
            raise SW2GError(rc, what, load().sw2g_error_step(self.h))

    def _arr(self, a):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=np.float64)
        if a.shape != (self.ny + 4, self.nx + 4):
            raise ValueError(f"field shape {a.shape} != {(self.ny + 4, self.nx + 4)}")
        return a

    def upload(self, eta, u, v, tracer=None, windx=None, windy=None, hB=None, mode=UPLOAD_FRAME):
        arrs = [self._arr(a) for a in (eta, u, v, tracer, windx, windy, hB)]
        self._keep = arrs
        self._check(load().sw2g_upload(self.h, *[_ptr(a) for a in arrs], mode), "sw2g_upload")

    def step(self, n: int):
        """Advance n steps; returns the status code (raises only on CUDA/argument errors)."""
        rc = load().sw2g_step(self.h, int(n))
        if rc in (OK, ERR_CFL, ERR_NONFINITE):
            return rc
        self._check(rc, "sw2g_step")

    def step_host(self, eta, u, v, n: int = 1):
        """sw2g_step_host: n steps of the state held in the caller's padded
        float64 arrays (C order, writable), which receive the new state in
        place; returns the status code as step() does."""
        for a in (eta, u, v):
            if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous
                    and a.flags.writeable and a.shape == (self.ny + 4, self.nx + 4)):
                raise ValueError("step_host takes writable C-contiguous float64 arrays of the padded shape")
        rc = load().sw2g_step_host(self.h, _ptr(eta), _ptr(u), _ptr(v), int(n))
        if rc in (OK, ERR_CFL, ERR_NONFINITE):
            return rc
        self._check(rc, "sw2g_step_host")

    def error_step(self) -> int:
        return load().sw2g_error_step(self.h)

    def steps_done(self) -> int:
        return load().sw2g_steps_done(self.h)

    def last_launches(self) -> int:
        return load().sw2g_last_launches(self.h)

    def download(self):
        out = [np.empty((self.ny + 4, self.nx + 4)) for _ in range(4)]
        self._check(load().sw2g_download(self.h, *[_ptr(a) for a in out]), "sw2g_download")
        return dict(zip(("eta", "u", "v", "tracer"), out))

    def diag(self):
        k, a, m = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self._check(load().sw2g_diag(self.h, ctypes.byref(k), ctypes.byref(a), ctypes.byref(m)), "sw2g_diag")
        return k.value, a.value, m.value

    def reset_ab(self):
        self._check(load().sw2g_reset_ab(self.h), "sw2g_reset_ab")

    def checkpoint(self) -> np.ndarray:
        """Exact-restart checkpoint (FP64 contexts): header, seven padded
        fields, the Adams-Bashforth histories."""
        L = load()
        L.sw2g_checkpoint_doubles.restype = ctypes.c_size_t
        L.sw2g_checkpoint_doubles.argtypes = [ctypes.c_void_p]
        L.sw2g_checkpoint_save.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_size_t]
        n = L.sw2g_checkpoint_doubles(self.h)
        if n == 0:
            raise ValueError("checkpoints are for FP64 contexts")
        buf = np.empty(n, dtype=np.float64)
        self._check(L.sw2g_checkpoint_save(self.h, _ptr(buf), n), "sw2g_checkpoint_save")
        return buf

    def test_tile_timeout(self, waits: int):
        """FP32 contexts: make the following steps' tile loads also wait for a
        barrier phase that never completes (waits > 0 tries each), or restore (0)."""
        L = load()
        L.sw2g_test_tile_timeout.argtypes = [ctypes.c_void_p, ctypes.c_int]
        self._check(L.sw2g_test_tile_timeout(self.h, int(waits)), "sw2g_test_tile_timeout")

    def restore(self, buf):
        L = load()
        L.sw2g_checkpoint_load.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_size_t]
        b = np.ascontiguousarray(buf, dtype=np.float64)
        self._check(L.sw2g_checkpoint_load(self.h, _ptr(b), b.size), "sw2g_checkpoint_load")

    def last_step_ms(self) -> float:
        return load().sw2g_last_step_ms(self.h)

    def timers(self, on: bool = True):
        self._check(load().sw2g_timers_enable(self.h, 1 if on else 0), "sw2g_timers_enable")

    def timers_reset(self):
        load().sw2g_timers_reset(self.h)

    def timer_table(self):
        """{kernel name: (launches, total ms)} accumulated while timers were on."""
        out = {}
        for i in range(load().sw2g_timers_count(self.h)):
            nm, n, ms = ctypes.c_char_p(), ctypes.c_longlong(), ctypes.c_double()
            self._check(load().sw2g_timer_read(self.h, i, ctypes.byref(nm), ctypes.byref(n), ctypes.byref(ms)),
                        "sw2g_timer_read")
            out[nm.value.decode()] = (n.value, ms.value)
        return out

    def add_field(self, which: int, delta, scale: float = 1.0):
        L = load()
        L.sw2g_add_field.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.c_double]
        d = self._arr(delta)
        self._check(L.sw2g_add_field(self.h, int(which), _ptr(d), float(scale)), "sw2g_add_field")

    def set_field_where(self, which: int, value, mask):
        L = load()
        L.sw2g_set_field_where.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                           ctypes.POINTER(ctypes.c_ubyte)]
        v = self._arr(value)
        m = np.ascontiguousarray(mask, dtype=np.uint8)
        if m.shape != v.shape:
            raise ValueError("mask shape")
        self._check(L.sw2g_set_field_where(self.h, int(which), _ptr(v), m.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte))),
                    "sw2g_set_field_where")

    def add_cells(self, which: int, cells, values, scale: float = 1.0):
        """sw2g_add_cells: field += scale * value on listed interior cells
        (increasing padded indices), += scale * 0 elsewhere."""
        L = load()
        L.sw2g_add_cells.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                     ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.c_double]
        c = np.ascontiguousarray(cells, dtype=np.int32)
        v = np.ascontiguousarray(values, dtype=np.float64)
        return L.sw2g_add_cells(self.h, int(which), c.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _ptr(v),
                                int(c.size), float(scale))

    def set_cells(self, which: int, cells, values):
        """sw2g_set_cells: field = value on listed interior cells."""
        L = load()
        L.sw2g_set_cells.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                     ctypes.POINTER(ctypes.c_double), ctypes.c_int]
        c = np.ascontiguousarray(cells, dtype=np.int32)
        v = np.ascontiguousarray(values, dtype=np.float64)
        return L.sw2g_set_cells(self.h, int(which), c.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _ptr(v),
                                int(c.size))

    def add_gaussian(self, g: "Gaussian") -> int:
        """sw2g_add_gaussian: the injection evaluated on the device; returns the status."""
        L = load()
        L.sw2g_add_gaussian.argtypes = [ctypes.c_void_p, ctypes.POINTER(Gaussian)]
        return L.sw2g_add_gaussian(self.h, ctypes.byref(g))

    def apply_channel(self):
        L = load()
        L.sw2g_apply_channel.argtypes = [ctypes.c_void_p]
        self._check(L.sw2g_apply_channel(self.h), "sw2g_apply_channel")

    def device_field(self, which: int) -> int:
        return load().sw2g_device_field(self.h, which)

    def stream(self) -> int:
        return load().sw2g_stream(self.h)


class Batch:
    """Several SW2G_FP32 solvers stepped together (sw2g_batch_*): one launch
    per phase over all members' strips, time loop replayed as a CUDA graph."""

    SCHEDULES = ("rows", "columns", "interleaved", "bands")
    TILE_ROWS = (16, 32, 64)  # strip shapes: 128 cells wide, this many rows high

    def __init__(self, solvers):
        L = load()
        vp = ctypes.c_void_p
        L.sw2g_batch_create.argtypes = [ctypes.POINTER(vp), ctypes.c_int, ctypes.POINTER(vp)]
        L.sw2g_batch_step.argtypes = [vp, ctypes.c_int]
        L.sw2g_batch_error_member.argtypes = [vp]
        L.sw2g_batch_error_step.argtypes = [vp]
        L.sw2g_batch_last_step_ms.restype = ctypes.c_double
        L.sw2g_batch_last_step_ms.argtypes = [vp]
        L.sw2g_batch_last_launches.restype = ctypes.c_longlong
        L.sw2g_batch_last_launches.argtypes = [vp]
        L.sw2g_batch_tune.argtypes = [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        L.sw2g_batch_schedule.argtypes = [vp]
        L.sw2g_batch_destroy.argtypes = [vp]
        self.solvers = list(solvers)
        arr = (vp * len(self.solvers))(*[s.h.value for s in self.solvers])
        h = vp()
        rc = L.sw2g_batch_create(arr, len(self.solvers), ctypes.byref(h))
        if rc != OK:
            raise SW2GError(rc, "sw2g_batch_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            load().sw2g_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def step(self, n: int) -> int:
        rc = load().sw2g_batch_step(self.h, int(n))
        if rc in (OK, ERR_CFL, ERR_NONFINITE):
            return rc
        raise SW2GError(rc, "sw2g_batch_step")

    def error(self):
        return load().sw2g_batch_error_member(self.h), load().sw2g_batch_error_step(self.h)

    def last_step_ms(self) -> float:
        return load().sw2g_batch_last_step_ms(self.h)

    def last_launches(self) -> int:
        return load().sw2g_batch_last_launches(self.h)

    def tune(self, steps_per_candidate: int):
        """Times every (strip shape, schedule) pair and keeps the fastest;
        returns {"128xTH/schedule": ms per step}."""
        nc = len(self.TILE_ROWS) * len(self.SCHEDULES)
        ms = (ctypes.c_double * nc)()
        rc = load().sw2g_batch_tune(self.h, int(steps_per_candidate), ms)
        if rc != OK:
            raise SW2GError(rc, "sw2g_batch_tune")
        ns = len(self.SCHEDULES)
        return {f"128x{th}/{self.SCHEDULES[k]}": ms[i * ns + k] for i, th in enumerate(self.TILE_ROWS)
                for k in range(ns)}

    def set_schedule(self, tile_rows: int, schedule: str):
        L = load()
        L.sw2g_batch_set_schedule.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        rc = L.sw2g_batch_set_schedule(self.h, int(tile_rows), self.SCHEDULES.index(schedule))
        if rc != OK:
            raise SW2GError(rc, "sw2g_batch_set_schedule")

    def schedule(self) -> str:
        return self.SCHEDULES[load().sw2g_batch_schedule(self.h)]

    def tile_rows(self) -> int:
        L = load()
        L.sw2g_batch_tile_rows.argtypes = [ctypes.c_void_p]
        return L.sw2g_batch_tile_rows(self.h)
