"""The red-exact mode's exp and pow (red.cuda_gb300/csrc/crmath.cuh) against
exact values (Python's decimal module at 80 digits) and against the C
library's exp and pow, which red's CPU code and its host-side step controller
call.

crmath's functions must return the double nearest to the exact result on
every sampled input.  The C library's agree with them except in its rare
misrounded cases (its documented error bound is about 0.52 ulp): at least
99.5 % of the samples must be bit-identical.  The header is compiled here for
the host by g++ without FMA contraction, the same source nvcc compiles for
the device with explicit round-to-nearest intrinsics.
"""
import ctypes as C
import math
import os
import subprocess
from decimal import Decimal, getcontext

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "red.cuda_gb300", "csrc")

SHIM = r'''
#include "crmath.cuh"
extern "C" double shim_pow(double x, double y) { return crmath::cr_pow(x, y); }
extern "C" double shim_exp(double x) { return crmath::cr_exp(x); }
'''


@pytest.fixture(scope="module")
def cr(tmp_path_factory):
    d = tmp_path_factory.mktemp("crmath")
    src = d / "shim.cpp"
    src.write_text(SHIM)
    so = d / "shim.so"
    subprocess.check_call(["g++", "-O2", "-ffp-contract=off", "-shared", "-fPIC", "-I", CSRC, "-o", str(so),
                           str(src)])
    L = C.CDLL(str(so))
    L.shim_pow.restype = C.c_double
    L.shim_pow.argtypes = [C.c_double, C.c_double]
    L.shim_exp.restype = C.c_double
    L.shim_exp.argtypes = [C.c_double]
    return L


def nearest(exact, got):
    """got is the double nearest to the Decimal exact (ties either way)."""
    d = abs(Decimal(got) - exact)
    up = abs(Decimal(math.nextafter(got, math.inf)) - exact)
    dn = abs(Decimal(math.nextafter(got, -math.inf)) - exact)
    return d <= up and d <= dn


def samples(rng, n):
    """The inputs the path meets: the step-size factor (tol/err)^(1/7) and
    ^(1/4) (RKF7(8), RK4) over 18 decades, the gas-disk powers r^p at
    0.05-6 AU, and the density profile's and reduction factor's exp."""
    pw = [(float(10 ** rng.uniform(-4, 14)), 1.0 / 7.0) for _ in range(n)]
    pw += [(float(10 ** rng.uniform(-4, 14)), 1.0 / 4.0) for _ in range(n)]
    pw += [(float(rng.uniform(0.05, 6.0)), float(rng.choice([-2.75, -2.5, -1.5, 1.0, 0.25, -3.5, 0.5, -6.5])))
           for _ in range(n)]
    ex = [float(-rng.uniform(0.0, 60.0)) for _ in range(n)] + [float(rng.uniform(-700.0, 700.0)) for _ in range(n)]
    return pw, ex


def test_correctly_rounded(cr):
    getcontext().prec = 80
    pw, ex = samples(np.random.default_rng(3), 1500)
    for x, y in pw:
        got = cr.shim_pow(x, y)
        assert nearest((Decimal(x).ln() * Decimal(y)).exp(), got), (x, y)
    for x in ex:
        assert nearest(Decimal(x).exp(), cr.shim_exp(x)), x


def test_agrees_with_the_c_library(cr):
    pw, ex = samples(np.random.default_rng(4), 20000)
    same = sum(cr.shim_pow(x, y) == math.pow(x, y) for x, y in pw) + sum(cr.shim_exp(x) == math.exp(x) for x in ex)
    assert same >= 0.995 * (len(pw) + len(ex)), same / (len(pw) + len(ex))


def test_special_cases(cr):
    assert cr.shim_pow(2.0, 0.0) == 1.0 and cr.shim_pow(1.0, 7.5) == 1.0 and cr.shim_pow(3.25, 1.0) == 3.25
    assert cr.shim_pow(4.0, 0.5) == 2.0 and cr.shim_pow(0.25, -0.5) == 2.0
    assert math.isinf(cr.shim_pow(0.0, -2.5)) and cr.shim_pow(0.0, 2.5) == 0.0
    assert math.isnan(cr.shim_pow(-1.0, 0.5))
    assert cr.shim_exp(0.0) == 1.0 and cr.shim_exp(-800.0) == math.exp(-800.0)
    assert math.isinf(cr.shim_exp(800.0))
