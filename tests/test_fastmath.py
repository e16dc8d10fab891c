"""The device exponential and logarithm (mpart_gb300/csrc/mpgb_fastmath.cuh),
built for the host with g++, against 40-digit decimal references: at most
1.5 units in the last place over the arguments the rectifiers and Hermite
functions give them, the IEEE special values, and the tables equal to what
their generator writes."""
import ctypes
import math
import os
import subprocess
import sys
from decimal import Decimal, getcontext

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "mpart_gb300", "csrc")


@pytest.fixture(scope="module")
def fm(tmp_path_factory):
    out = tmp_path_factory.mktemp("fm") / "fm.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-o", str(out),
                    os.path.join(HERE, "fastmath_harness.cpp")], check=True)
    lib = ctypes.CDLL(str(out))

    def call(name, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        getattr(lib, name)(x.ctypes.data_as(ctypes.c_void_p), y.ctypes.data_as(ctypes.c_void_p),
                           ctypes.c_long(x.size))
        return y

    return call


def _max_ulps(y, ref):
    worst = 0.0
    for a, r in zip(y, ref):
        u = Decimal(math.ulp(float(r)))
        worst = max(worst, float(abs(Decimal(float(a)) - r) / u))
    return worst


@pytest.mark.parametrize("lo,hi", [(-1.0, 0.0), (-40.0, 0.0), (-700.0, 700.0), (-745.1, -708.0), (700.0, 709.7)])
def test_exp_within_1_5_ulp(fm, lo, hi):
    getcontext().prec = 40
    x = np.random.default_rng(int(abs(lo) + hi)).uniform(lo, hi, 3000)
    ref = [Decimal(float(v)).exp() for v in x]
    assert _max_ulps(fm("fm_exp", x), ref) <= 1.5


@pytest.mark.parametrize("lo,hi", [(1.0, 1.0 + 1e-12), (1.0, 1.01), (1.0, 2.0), (1.99, 2.0)])
def test_log_within_1_5_ulp(fm, lo, hi):
    getcontext().prec = 40
    x = np.random.default_rng(int(hi * 100)).uniform(lo, hi, 3000)
    ref = [Decimal(float(v)).ln() for v in x]
    assert _max_ulps(fm("fm_log1to2", x), ref) <= 1.5


def test_special_values(fm):
    x = np.array([np.nan, np.inf, -np.inf, 710.0, -746.0, 0.0, -0.0, 1e300, -1e300, -745.0])
    y = fm("fm_exp", x)
    assert np.isnan(y[0])
    assert y[1] == np.inf and y[3] == np.inf and y[7] == np.inf
    assert y[2] == 0.0 and y[4] == 0.0 and y[8] == 0.0
    assert y[5] == 1.0 and y[6] == 1.0
    assert y[9] == 5e-324  # gradual underflow down to the last subnormal
    lg = fm("fm_log1to2", np.array([1.0, 2.0, np.nan, np.nextafter(1.0, 2.0)]))
    assert lg[0] == 0.0 and lg[1] == math.log(2.0) and np.isnan(lg[2])
    assert lg[3] == math.log(np.nextafter(1.0, 2.0))  # log(1 + u) = u - u^2 / 2 to the last bit


def test_tables_match_their_generator():
    out = subprocess.run([sys.executable, os.path.join(CSRC, "gen_fastmath_tables.py")], check=True,
                         capture_output=True, text=True).stdout
    with open(os.path.join(CSRC, "mpgb_fastmath_tables.h")) as f:
        assert f.read() == out
