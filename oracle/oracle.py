"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg to
check or time the CUDA implementation; the product never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libsw2oracle.so")


class Params(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("sch", ctypes.c_int),
                ("lon0", ctypes.c_double), ("lon1", ctypes.c_double),
                ("lat0", ctypes.c_double), ("lat1", ctypes.c_double),
                ("Omega", ctypes.c_double), ("rE", ctypes.c_double), ("rP", ctypes.c_double),
                ("gE", ctypes.c_double), ("depth", ctypes.c_double),
                ("Dt", ctypes.c_double), ("courant", ctypes.c_double),
                ("tau", ctypes.c_double), ("tracer_dis", ctypes.c_double),
                ("hypernu", ctypes.c_double * 3), ("lape_eta", ctypes.c_int)]


_lib = None


def build():
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        L.sw2o_create.restype = ctypes.c_void_p
        L.sw2o_create.argtypes = [ctypes.POINTER(Params)]
        L.sw2o_destroy.argtypes = [ctypes.c_void_p]
        L.sw2o_padded_size.argtypes = [ctypes.c_void_p]
        L.sw2o_field.restype = dp
        L.sw2o_field.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.sw2o_load.argtypes = [ctypes.c_void_p] + [dp] * 7
        L.sw2o_load_raw.argtypes = [ctypes.c_void_p] + [dp] * 7
        L.sw2o_step.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        L.sw2o_reset_ab.argtypes = [ctypes.c_void_p]
        L.sw2o_energy.argtypes = [ctypes.c_void_p, dp, dp, dp]
        L.sw2o_row_table.restype = dp
        L.sw2o_row_table.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.sw2o_halo_update.argtypes = [ctypes.c_int, ctypes.c_int, dp]
        L.sw2o_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def params_from_case(p, lape_eta=False) -> Params:
    q = Params()
    q.lape_eta = int(bool(lape_eta))
    q.nx, q.ny, q.sch = p.nx, p.ny, p.sch
    q.lon0, q.lon1, q.lat0, q.lat1 = p.lon0, p.lon1, p.lat0, p.lat1
    q.Omega, q.rE, q.rP, q.gE, q.depth = p.Omega, p.rE, p.rP, p.gE, p.depth
    q.Dt, q.courant, q.tau, q.tracer_dis = p.Dt, p.CFL, p.Tau, p.TracerDis
    for k in range(3):
        q.hypernu[k] = p.hypernu[k]
    return q


def _ptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


FIELDS = ("eta", "u", "v", "tracer", "windx", "windy", "hB")


class Oracle:
    """One oracle run of a case; fields are (ny+4, nx+4) padded arrays."""

    def __init__(self, params, lape_eta=False):
        self._p = params_from_case(params, lape_eta)
        self.nx, self.ny = params.nx, params.ny
        self.h = lib().sw2o_create(ctypes.byref(self._p))
        if not self.h:
            raise ValueError("oracle rejected the case parameters")

    def close(self):
        if self.h:
            lib().sw2o_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def load(self, fields, raw=False):
        arrs = [np.ascontiguousarray(f, dtype=np.float64) for f in fields]
        fn = lib().sw2o_load_raw if raw else lib().sw2o_load
        fn(self.h, *[_ptr(a) for a in arrs])

    def step(self, n):
        bad = ctypes.c_int(-1)
        rc = lib().sw2o_step(self.h, int(n), ctypes.byref(bad))
        return rc, bad.value

    def reset_ab(self):
        lib().sw2o_reset_ab(self.h)

    def field(self, name):
        k = FIELDS.index(name)
        S = (self.nx + 4) * (self.ny + 4)
        p = lib().sw2o_field(self.h, k)
        return np.ctypeslib.as_array(p, shape=(S,)).reshape(self.ny + 4, self.nx + 4).copy()

    def energy(self):
        k, a, m = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        lib().sw2o_energy(self.h, ctypes.byref(k), ctypes.byref(a), ctypes.byref(m))
        return k.value, a.value, m.value

    def row_table(self, which):
        p = lib().sw2o_row_table(self.h, which)
        return np.ctypeslib.as_array(p, shape=(self.ny + 4,)).copy()


def threads() -> int:
    return lib().sw2o_threads()
