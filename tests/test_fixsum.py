"""Fixed-point summation of the CG grid reductions (csrc/sa_fixsum.cuh) on the host.

The GPU reductions align every value to the largest exponent of its set and
add 128-bit integers, then round once.  Checked here through a host shim:
- the result is the correctly rounded exact sum (math.fsum) whenever the
  values lie within 2^60 of the largest one (random sets, mixed signs, zeros,
  subnormals, up to 1200 values);
- it does not depend on the order of the values;
- FP32 inputs are summed exactly as their FP64 values;
- overflow gives +-Inf, an Inf or NaN in the set gives NaN, values more than
  2^112 below the largest are dropped (documented truncation).
"""
import ctypes as C
import math
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def fx(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("fx") / "libfx.so")
    subprocess.run(["g++", "-O2", "-shared", "-fPIC", "-o", out, os.path.join(HERE, "fixsum_shim.cpp")], check=True)
    lib = C.CDLL(out)
    lib.fx_sum_f64.restype = C.c_double
    lib.fx_sum_f64.argtypes = [C.c_void_p, C.c_int]
    lib.fx_sum_f32.restype = C.c_double
    lib.fx_sum_f32.argtypes = [C.c_void_p, C.c_int]

    def f64(v):
        a = np.ascontiguousarray(v, dtype=np.float64)
        return lib.fx_sum_f64(a.ctypes.data, a.size)

    def f32(v):
        a = np.ascontiguousarray(v, dtype=np.float32)
        return lib.fx_sum_f32(a.ctypes.data, a.size)
    return f64, f32


def test_correctly_rounded_exact_sum(fx):
    f64, _ = fx
    rng = np.random.default_rng(5)
    for trial in range(4000):
        n = int(rng.integers(1, 1200))
        spread = int(rng.integers(0, 58))
        base = int(rng.integers(-1070, 1015 - spread))
        v = rng.uniform(0.5, 1.0, n) * np.exp2((base + rng.integers(0, spread + 1, n)).astype(float))
        v *= rng.choice([-1.0, 1.0], n)
        if trial % 5 == 0:
            v[rng.integers(0, n, n // 3)] = 0.0
        try:
            want = math.fsum(v.tolist())
        except OverflowError:
            continue
        assert f64(v) == want, (trial, n, spread, base)


def test_order_independent(fx):
    f64, _ = fx
    rng = np.random.default_rng(6)
    v = rng.standard_normal(608) * np.exp2(rng.integers(-40, 40, 608).astype(float))
    s = f64(v)
    for _ in range(20):
        assert f64(rng.permutation(v)) == s


def test_float_inputs_are_exact(fx):
    f64, f32 = fx
    rng = np.random.default_rng(7)
    for _ in range(1000):
        n = int(rng.integers(1, 700))
        v = (rng.standard_normal(n) * np.exp2(rng.integers(-30, 30, n).astype(float))).astype(np.float32)
        want = math.fsum(v.astype(np.float64).tolist())
        assert f32(v) == want
        assert f64(v.astype(np.float64)) == want
    tiny = np.array([1e-45, 1e-45, -3e-45], dtype=np.float32)          # FP32 subnormals
    assert f32(tiny) == math.fsum(tiny.astype(np.float64).tolist())


def test_special_values(fx):
    f64, f32 = fx
    assert f64([5e-324, 5e-324]) == 1e-323
    assert f64([2.2250738585072014e-308, -5e-324]) == 2.225073858507201e-308
    assert f64([1e308, 1e308]) == math.inf and f64([-1e308, -1e308]) == -math.inf
    assert math.isnan(f64([math.inf, 1.0])) and math.isnan(f64([math.nan, 0.0]))
    assert math.isnan(f32(np.array([np.inf, 1.0], dtype=np.float32)))
    assert f64([0.0]) == 0.0 and f64([1.0, -1.0]) == 0.0
    assert f64([0.1] * 1000) == math.fsum([0.1] * 1000)
    assert f64([1e308, -1e308, 1.0]) == 0.0                            # 1.0 lies below the 2^-112 window
