"""The case reader's expression evaluator against the reference's own.

The reference evaluates every <...> expression of a case file with its
vendored expression library (sppde/sppde_parser.c:111 calls te_interp of
sppde/sppde_tinyexpr.c). `oracle/Makefile` (target `ref`) compiles that one
file, from the reference's sources where they lie, into
oracle/_ref/libtinyexpr.so; this test evaluates a corpus of expressions with
both and requires the same verdict (error or not) and the same double, bit for
bit (any NaN matches any NaN). The corpus covers operator precedence (unary
signs bind tighter than '^', '^' is left-associative), '%', the functions and
constants, and the integer arithmetic of fac, ncr and npr at and beyond 64-bit
overflow. Skipped where the reference's sources are absent.
"""
import ctypes
import math
import os
import struct
import subprocess

import pytest

from sw2_gb300 import hostlib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TE = os.path.join(ROOT, "oracle", "_ref", "libtinyexpr.so")

CORPUS = [
    # numbers and precedence
    "1", ".5", "1e-3", "1.5e+3*2", "7.1492e7", "2*pi*7.1492e7/360",
    "1+2*3", "(1+2)*3", "2^3^2", "-2^2", "-2^-2", "2^-1", "--3", "+-+3", "2*-3", "-(2)^2",
    "10%3", "-7%3", "7%-3", "7.5%2", "1/3", "3/0", "-3/0", "0/0", "1-2-3", "2/4/8",
    "(1,2,3)", "1,2", "(1,2)*3",
    # functions and constants
    "pi", "pi()", "e", "e()", "sin pi", "sin(pi/6)^2", "cos(0)", "tan(1)", "asin(0.5)", "acos(0.5)",
    "atan(1)", "atan2(1,2)", "atan2(-1,-2)", "pow(2,0.5)", "pow(-8,1/3)", "sqrt 16", "sqrt(2)",
    "exp(1)", "ln(e)", "log(100)", "log10(1000)", "abs(-3)", "ceil(2.5)", "floor(-2.5)",
    "cosh(1)", "sinh(1)", "tanh(0.5)", "-fac(3)", "fac 3", "2^sqrt 4",
    # integer arithmetic of fac / ncr / npr
    *[f"fac({k})" for k in range(0, 26)],
    "fac(20.7)", "fac(-1)", "fac(170)", "fac(171)", "fac(4294967295)", "fac(4294967296)",
    "ncr(10,3)", "ncr(60,30)", "ncr(62,31)", "ncr(66,33)", "ncr(67,33)", "ncr(68,34)", "ncr(100,50)",
    "ncr(5.5,2.5)", "ncr(5.5,5.2)", "ncr(3,4)", "ncr(-1,0)", "ncr(4294967296,1)", "ncr(7,0)", "ncr(7,7)",
    "npr(20,5)", "npr(25,20)", "npr(25,21)", "npr(30,2)", "npr(5,6)",
    # errors
    "2+", "(1", "foo", "1 2", "", "sin", "atan2(1)", "pow(1,2,3)", "1)",
]


def _te():
    if not os.path.exists(TE):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=False,
                       capture_output=True)
    if not os.path.exists(TE):
        pytest.skip("the reference's sources are not present: its evaluator cannot be built")
    L = ctypes.CDLL(TE)
    L.te_interp.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int)]
    L.te_interp.restype = ctypes.c_double
    return L


def _bits(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


@pytest.mark.parametrize("expr", CORPUS)
def test_expression_matches_reference(expr):
    L = _te()
    err = ctypes.c_int(0)
    ref = L.te_interp(expr.encode(), ctypes.byref(err))
    try:
        got = hostlib.evaluate(expr)
        ok = True
    except ValueError:
        ok = False
    assert ok == (err.value == 0), (expr, ref, err.value)
    if not ok:
        return
    if math.isnan(ref):
        assert math.isnan(got), (expr, got)
    else:
        assert _bits(got) == _bits(ref), (expr, got, ref)
