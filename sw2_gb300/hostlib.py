"""ctypes binding of libsw2host.so: the SW2 case reader and the host
restatement of the reference's forcing (sw2_gb300/host/). Plain C, no GPU:
the tests use it to check the reader and the forcing fields on the CPU."""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsw2host.so")
RUNNER = os.path.join(HERE, "_build", "sw2g-run")

_D = ctypes.c_double
_P = ctypes.POINTER(ctypes.c_double)


class SwCase(ctypes.Structure):
    _fields_ = [("sch", ctypes.c_int), ("polar", ctypes.c_int),
                ("lon0", _D), ("lon1", _D), ("lat0", _D), ("lat1", _D),
                ("nx", ctypes.c_int), ("ny", ctypes.c_int),
                ("t0", _D), ("t1", _D), ("Dt", _D), ("CFL", _D), ("N", ctypes.c_int),
                ("tau", _D), ("sigma_dis", _D), ("nu2", _D), ("nu4", _D), ("nu6", _D),
                ("IteInfo", ctypes.c_int), ("saveEvery", ctypes.c_int), ("loadFrom", ctypes.c_int),
                ("reftype", ctypes.c_int),
                ("Omega", _D), ("rE", _D), ("rP", _D), ("gE", _D), ("depth", _D), ("epsilon2", _D),
                ("geoeq", ctypes.c_int),
                ("num_vortices", ctypes.c_int), ("vortices", _P),
                ("num_gaussians", ctypes.c_int), ("gaussians", _P),
                ("tracer_dis", _D),
                ("wind_rows", ctypes.c_int), ("wind", _P),
                ("beta_sponge", _D), ("sigma_sponge", _D)]


class SwForce(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("pert", _P), ("tracer", _P),
                ("mask", ctypes.POINTER(ctypes.c_ubyte)), ("perturbs", _P), ("deta", _P), ("du", _P), ("dv", _P),
                ("cells", ctypes.POINTER(ctypes.c_int)), ("ncells", ctypes.c_int),
                ("cell_pert", _P), ("cell_tracer", _P),
                ("row_pl", _P), ("row_sin", _P), ("row_cos", _P), ("row_surf", _P), ("col_lonc", _P),
                ("tables_ready", ctypes.c_int)]


_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} not built: run `python -m sw2_gb300.build`")
        L = ctypes.CDLL(LIB_PATH)
        L.swcase_read.argtypes = [ctypes.c_char_p, ctypes.POINTER(SwCase), ctypes.c_char_p, ctypes.c_size_t]
        L.swcase_free.argtypes = [ctypes.POINTER(SwCase)]
        L.swcase_m4.restype = ctypes.c_void_p
        L.swcase_m4.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_size_t]
        L.swcase_eval.argtypes = [ctypes.c_char_p, ctypes.POINTER(_D)]
        L.swforce_init.argtypes = [ctypes.POINTER(SwForce), ctypes.c_int, ctypes.c_int]
        L.swforce_free.argtypes = [ctypes.POINTER(SwForce)]
        L.swforce_gaussian.argtypes = [ctypes.POINTER(SwCase), ctypes.c_int, _D, _D, ctypes.POINTER(SwForce),
                                       ctypes.POINTER(_D), ctypes.c_char_p, ctypes.c_size_t]
        L.swforce_vortex.argtypes = [ctypes.POINTER(SwCase), ctypes.c_int, ctypes.POINTER(SwForce)]
        L.swforce_windx.argtypes = [ctypes.POINTER(SwCase), _P, ctypes.c_char_p, ctypes.c_size_t]
        L.swforce_winds.argtypes = [ctypes.POINTER(SwCase), _D, _P, _P, ctypes.c_char_p, ctypes.c_size_t]
        libc = ctypes.CDLL(None)
        libc.free.argtypes = [ctypes.c_void_p]
        L._free = libc.free
        _lib = L
    return _lib


def evaluate(expr: str) -> float:
    v = _D()
    if load().swcase_eval(expr.encode(), ctypes.byref(v)) != 0:
        raise ValueError(f"cannot evaluate {expr!r}")
    return v.value


def m4(path: str) -> str:
    err = ctypes.create_string_buffer(512)
    p = load().swcase_m4(path.encode(), err, 512)
    if not p:
        raise ValueError(err.value.decode())
    s = ctypes.string_at(p).decode()
    load()._free(p)
    return s


class Case:
    """A parsed case file (the fields of the reference's sw struct after initialize())."""

    def __init__(self, path: str):
        self.c = SwCase()
        err = ctypes.create_string_buffer(512)
        if load().swcase_read(path.encode(), ctypes.byref(self.c), err, 512) != 0:
            raise ValueError(err.value.decode())

    def __getattr__(self, name):
        return getattr(self.__dict__["c"], name)

    def table(self, which: str) -> np.ndarray:
        c = self.c
        if which == "gaussians":
            return np.ctypeslib.as_array(c.gaussians, (c.num_gaussians, 12)).copy() if c.num_gaussians else np.zeros((0, 12))
        if which == "vortices":
            return np.ctypeslib.as_array(c.vortices, (c.num_vortices, 7)).copy() if c.num_vortices else np.zeros((0, 7))
        w = np.ctypeslib.as_array(c.wind, (2 * c.wind_rows,)).copy()
        return np.stack([w[:c.wind_rows], w[c.wind_rows:]], axis=1)

    def windx(self) -> np.ndarray:
        c = self.c
        out = np.zeros((c.ny + 4, c.nx + 4))
        err = ctypes.create_string_buffer(512)
        if load().swforce_windx(ctypes.byref(c), out.ctypes.data_as(_P), err, 512) != 0:
            raise ValueError(err.value.decode())
        return out

    def winds(self, beta_sponge_deg: float = 0.0):
        """(windx, windy) over all padded cells as read_wind leaves them (io.c:199-240)."""
        c = self.c
        wx = np.zeros((c.ny + 4, c.nx + 4))
        wy = np.zeros_like(wx)
        err = ctypes.create_string_buffer(512)
        if load().swforce_winds(ctypes.byref(c), beta_sponge_deg, wx.ctypes.data_as(_P), wy.ctypes.data_as(_P),
                                err, 512) != 0:
            raise ValueError(err.value.decode())
        return wx, wy

    def close(self):
        if getattr(self, "c", None) is not None:
            load().swcase_free(ctypes.byref(self.c))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Forcing:
    """Host forcing fields of one case (swforce.c)."""

    def __init__(self, case: Case):
        self.case = case
        self.w = SwForce()
        if load().swforce_init(ctypes.byref(self.w), case.c.nx, case.c.ny) != 0:
            raise MemoryError("swforce_init")
        self.shape = (case.c.ny + 4, case.c.nx + 4)

    def _arr(self, p):
        return np.ctypeslib.as_array(p, (self.shape[0] * self.shape[1],)).reshape(self.shape).copy()

    def gaussian(self, row: int, Dt: float, t: float):
        """(status, rescale factor, field, tracer values, mask, perturbs)."""
        rf = _D()
        err = ctypes.create_string_buffer(512)
        rc = load().swforce_gaussian(ctypes.byref(self.case.c), row, Dt, t, ctypes.byref(self.w), ctypes.byref(rf),
                                     err, 512)
        if rc < 0:
            raise ValueError(err.value.decode())
        return (rc, rf.value, self._arr(self.w.pert), self._arr(self.w.tracer),
                np.ctypeslib.as_array(self.w.mask, (self.shape[0] * self.shape[1],)).reshape(self.shape).copy(),
                self._arr(self.w.perturbs))

    def cells(self):
        """The last injection's cell list: (padded indices, Gaussian values, tracer values)."""
        n = self.w.ncells
        if n == 0:
            return np.zeros(0, np.int32), np.zeros(0), np.zeros(0)
        return (np.ctypeslib.as_array(self.w.cells, (n,)).copy(), np.ctypeslib.as_array(self.w.cell_pert, (n,)).copy(),
                np.ctypeslib.as_array(self.w.cell_tracer, (n,)).copy())

    def vortex(self, row: int):
        load().swforce_vortex(ctypes.byref(self.case.c), row, ctypes.byref(self.w))
        return self._arr(self.w.deta), self._arr(self.w.du), self._arr(self.w.dv)

    def __del__(self):
        try:
            load().swforce_free(ctypes.byref(self.w))
        except Exception:
            pass
