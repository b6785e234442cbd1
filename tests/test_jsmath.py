"""JavaScript math semantics used by the voxeliser.

* The device routines (pixels_gb300/csrc/jsmath.cuh, compiled for the host by
  the build) are correctly rounded: checked against 300-bit mpmath.
* The oracle's independent routines agree with them bit for bit.
* Math.round / Math.hypot edge cases.
"""
import ctypes
import math
import os
import random

import pytest

from pixels_gb300 import build
from pixels_gb300.jsmath import js_hypot, js_round, mulberry32

mpmath = pytest.importorskip("mpmath")


@pytest.fixture(scope="module")
def jsm():
    build.build()
    L = ctypes.CDLL(build.JSM_OUT)
    for f in ("px_host_sin", "px_host_atan2", "px_host_hypot2", "px_host_round"):
        getattr(L, f).restype = ctypes.c_double
    L.px_host_sin.argtypes = [ctypes.c_double]
    L.px_host_round.argtypes = [ctypes.c_double]
    L.px_host_atan2.argtypes = [ctypes.c_double, ctypes.c_double]
    L.px_host_hypot2.argtypes = [ctypes.c_double, ctypes.c_double]
    return L


def test_sin_correctly_rounded(jsm):
    mpmath.mp.prec = 300
    rnd = random.Random(11)
    for i in range(3000):
        x = rnd.uniform(-200, 200) if i % 3 else rnd.uniform(-4, 4) * 2.0 ** rnd.randint(-30, 0)
        assert jsm.px_host_sin(x) == float(mpmath.sin(mpmath.mpf(x))), x


def test_atan2_correctly_rounded_and_special_cases(jsm):
    mpmath.mp.prec = 300
    rnd = random.Random(12)
    for i in range(3000):
        y = rnd.uniform(-1, 1) * 2.0 ** rnd.randint(-20, 5)
        x = y if i % 7 == 0 else rnd.uniform(-1, 1) * 2.0 ** rnd.randint(-20, 5)
        assert jsm.px_host_atan2(y, x) == float(mpmath.atan2(mpmath.mpf(y), mpmath.mpf(x))), (y, x)
    for y, x in [(0.0, 1.0), (-0.0, 1.0), (0.0, -1.0), (-0.0, -1.0), (0.0, -0.0), (-0.0, -0.0),
                 (1.0, 0.0), (-1.0, 0.0), (math.inf, math.inf), (-math.inf, -math.inf), (1.0, -math.inf)]:
        a, b = jsm.px_host_atan2(y, x), math.atan2(y, x)
        assert a == b and math.copysign(1, a) == math.copysign(1, b), (y, x)


def test_oracle_routines_agree_with_device_routines(jsm, tmp_path):
    src = tmp_path / "r.cpp"
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src.write_text('#include "%s/oracle/jsmath_ref.h"\nextern "C" { double rs(double x){return ref::ref_sin(x);}'
                   ' double ra(double y,double x){return ref::ref_atan2(y,x);} }\n' % root)
    so = tmp_path / "r.so"
    import subprocess
    subprocess.run(["g++", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-o", str(so), str(src)], check=True)
    R = ctypes.CDLL(str(so))
    R.rs.restype = R.ra.restype = ctypes.c_double
    R.rs.argtypes = [ctypes.c_double]
    R.ra.argtypes = [ctypes.c_double, ctypes.c_double]
    rnd = random.Random(13)
    for _ in range(20000):
        x = rnd.uniform(-300, 300)
        assert R.rs(x) == jsm.px_host_sin(x)
        y, z = rnd.uniform(-2, 2), rnd.uniform(-2, 2)
        assert R.ra(y, z) == jsm.px_host_atan2(y, z)


def test_round_half_up(jsm):
    for x, r in [(0.5, 1.0), (-0.5, -0.0), (1.5, 2.0), (-1.5, -1.0), (2.4999999999999996, 2.0),
                 (0.49999999999999994, 0.0), (-2.5, -2.0), (1e16 + 1, 1e16 + 1)]:
        assert js_round(x) == r and jsm.px_host_round(x) == r, x


def test_hypot_engine_method(jsm):
    rnd = random.Random(14)
    for _ in range(5000):
        a, b = rnd.uniform(-3, 3), rnd.uniform(-3, 3)
        assert js_hypot(a, b) == jsm.px_host_hypot2(a, b)
    assert js_hypot(0.0, 0.0) == 0.0 and js_hypot(3.0, 4.0) == 5.0


def test_mulberry32_known_answers():
    # independent restatement with explicit 32-bit arithmetic
    def ref(seed, n):
        a = seed & 0xFFFFFFFF
        out = []
        for _ in range(n):
            a = (a + 0x6D2B79F5) & 0xFFFFFFFF
            t = a
            t = ((t ^ (t >> 15)) * (t | 1)) & 0xFFFFFFFF
            t ^= (t + (((t ^ (t >> 7)) * (t | 61)) & 0xFFFFFFFF)) & 0xFFFFFFFF
            out.append(((t ^ (t >> 14)) & 0xFFFFFFFF) / 4294967296)
        return out
    r = mulberry32(1337)
    assert [r() for _ in range(50)] == ref(1337, 50)
    assert all(0 <= v < 1 for v in ref(5, 100))
