"""Accuracy of the FP64 exponential and square root of the varifold pair sums.

The pair kernels evaluate e^x with Tang's table-driven method (64-entry
table of 2^(j/64), degree-5 Taylor polynomial; csrc/sa_varifold.cu exp_tab)
and the Matern kernel's distance sqrt(d^2) by two Newton (Heron) steps from
the FP32 reciprocal square root (sqrt_nr).  Both are checked here against
CUDA's exp() / sqrt() and against the host libm on the ranges the kernels
use (x <= 0 down to -40; squared distances of shapes of extent ~1), the
whole fast range, every table index, and the values passed on to CUDA's
functions (|x| >= 700, squared distances outside [2^-95, 2^96), zero,
infinities, NaN)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ulps(a, b):
    """Distance in units in the last place between finite non-negative doubles."""
    return np.abs(a.view(np.int64) - b.view(np.int64))       # integer difference of the bit patterns


def _run(fn, x):
    from shape_atrophy_gb300 import api
    ctx = api.context(0)
    dp = C.POINTER(C.c_double)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y, yref = np.empty_like(x), np.empty_like(x)
    rc = ctx.lib.sa_selftest_math(ctx.h, fn, x.size, x.ctypes.data_as(dp), y.ctypes.data_as(dp),
                                  yref.ctypes.data_as(dp))
    assert rc == 0, ctx.lib.sa_error_message(ctx.h)
    return y, yref


def test_exp_tab_within_two_ulps_of_cuda_and_libm():
    rng = np.random.default_rng(5)
    ln2_64 = np.log(2.0) / 64
    x = np.concatenate([
        -rng.uniform(0.0, 40.0, 2_000_000),                       # the pair kernels' range
        rng.uniform(-700.0, 700.0, 1_000_000),
        -rng.exponential(1e-3, 200_000), rng.exponential(1e-3, 200_000),
        np.arange(-64 * 30, 64 * 30) * ln2_64,                     # every table index, exact multiples
        np.arange(-64 * 30, 64 * 30) * ln2_64 + ln2_64 / 2,        # half-way points (largest |r|)
        [0.0, -0.0, 5e-324, -5e-324, 1e-300, -1e-300, 699.999999, -699.999999],
    ])
    y, yref = _run(0, x)
    assert np.all(np.isfinite(y)) and np.all(y > 0)
    u_cuda = _ulps(y, yref)
    u_libm = _ulps(y, np.exp(x))
    assert u_cuda.max() <= 2, f"max {u_cuda.max()} ulps from exp() at x = {x[np.argmax(u_cuda)]!r}"
    assert u_libm.max() <= 2, f"max {u_libm.max()} ulps from libm at x = {x[np.argmax(u_libm)]!r}"
    assert np.mean(u_cuda) < 0.5 and np.mean(u_libm) < 0.5          # most values are the same double


def test_exp_tab_passes_outside_values_to_exp():
    x = np.array([700.0, -700.0, 709.7, -745.0, -746.0, -1e4, 1e4, np.inf, -np.inf, np.nan])
    y, yref = _run(0, x)
    np.testing.assert_array_equal(np.isnan(y), np.isnan(yref))
    ok = ~np.isnan(yref)
    np.testing.assert_array_equal(y[ok], yref[ok])


def test_sqrt_nr_within_one_ulp_of_correctly_rounded():
    rng = np.random.default_rng(6)
    k = np.arange(1, 200_000, dtype=np.float64)
    x = np.concatenate([
        rng.uniform(0.0, 4.0, 2_000_000),                         # squared distances on a unit shape
        10.0 ** rng.uniform(-28.0, 28.0, 1_000_000),              # the whole fast range
        k * k, (k * k) * (1 + 2.0 ** -52), (k * k) * (1 - 2.0 ** -53),   # exact squares and neighbours
        2.0 ** np.arange(-95, 96, dtype=np.float64),               # the fast range's ends
        np.nextafter(2.0 ** 96, 0.0) * np.ones(1),
    ])
    y, yref = _run(1, x)
    u_cuda = _ulps(y, yref)                                        # CUDA's sqrt() is correctly rounded
    u_libm = _ulps(y, np.sqrt(x))
    assert u_cuda.max() <= 1, f"max {u_cuda.max()} ulps from sqrt() at x = {x[np.argmax(u_cuda)]!r}"
    assert u_libm.max() <= 1
    assert np.mean(u_cuda) < 0.01                                  # nearly always the same double
    np.testing.assert_array_equal(y[: 2_000_000][x[: 2_000_000] == 0.0], 0.0)


def test_sqrt_nr_passes_outside_values_to_sqrt():
    x = np.array([0.0, -0.0, 5e-324, 1e-300, 2.0 ** -96, 2.0 ** 96, 1e300, np.inf, np.nan, -1.0])
    y, yref = _run(1, x)
    np.testing.assert_array_equal(np.isnan(y), np.isnan(yref))
    ok = ~np.isnan(yref)
    np.testing.assert_array_equal(y[ok].view(np.int64), yref[ok].view(np.int64))
