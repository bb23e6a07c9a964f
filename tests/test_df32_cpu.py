"""Double-float routines of the far-field tiles, checked on the host.

The harness compiles bem_gmsh_gb300/csrc/df32.cuh with contraction off, which
makes its results bit-identical to the device build; references are long
double (64- or 113-bit mantissa).
"""
import ctypes
import os
import subprocess
import tempfile

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def h():
    d = tempfile.mkdtemp(prefix="df32_")
    so = os.path.join(d, "libdf32.so")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC",
                           os.path.join(HERE, "native", "df32_harness.cpp"), "-o", so])
    L = ctypes.CDLL(so)
    P = ctypes.POINTER(ctypes.c_double)
    F = ctypes.POINTER(ctypes.c_float)
    for nm in ("df_log_batch",):
        getattr(L, nm).argtypes = [P, ctypes.c_int, P]
    for nm in ("df_div_batch", "df_mul_batch", "df_diff_batch"):
        getattr(L, nm).argtypes = [P, P, ctypes.c_int, P]
    L.df_to_double_batch.argtypes = [F, F, ctypes.c_int, P]
    L.df_scale_to_f32_batch.argtypes = [P, ctypes.POINTER(ctypes.c_int), ctypes.c_int, F]
    return L


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _df(x):
    """Value of the double-float split of x, in long double."""
    hi = x.astype(np.float32)
    lo = (x - hi.astype(np.float64)).astype(np.float32)
    return hi.astype(np.longdouble) + lo.astype(np.longdouble)


def test_log_accuracy(h):
    rng = np.random.default_rng(0)
    x = np.exp(rng.uniform(np.log(1e-12), np.log(1e8), 200000))
    x = np.concatenate([x, [1.0, 2.0, 0.5, 1.0 + 2.0 ** -20, 1.99999, 1.00390625, 1.0 - 1e-7]])
    out = np.empty_like(x)
    h.df_log_batch(_p(x), x.size, _p(out))
    ref = np.log(_df(x))  # log of the DF input the routine sees
    err = np.abs(out.astype(np.longdouble) - ref)
    bound = 2.0 ** -46 * np.maximum(np.abs(ref), 1.0)
    assert np.all(err <= bound), float(np.max(err / bound))


def test_div_mul_accuracy(h):
    rng = np.random.default_rng(1)
    a = rng.standard_normal(100000) * np.exp(rng.uniform(-10, 10, 100000))
    b = rng.standard_normal(100000) * np.exp(rng.uniform(-10, 10, 100000))
    out = np.empty_like(a)
    h.df_div_batch(_p(a), _p(b), a.size, _p(out))
    ref = _df(a) / _df(b)
    # measured worst case 6.4 units of 2^-48 (double-float precision is ~2^-48)
    assert np.max(np.abs((out - ref) / ref)) < 2.0 ** -45
    h.df_mul_batch(_p(a), _p(b), a.size, _p(out))
    ref = _df(a) * _df(b)
    # measured worst case 3.1 units of 2^-48
    assert np.max(np.abs((out - ref) / ref)) < 2.0 ** -46


def test_difference_exact_under_cancellation(h):
    """xn - xs for nearby coordinates keeps ~48 bits of the difference."""
    rng = np.random.default_rng(2)
    xs = rng.uniform(-3, 3, 100000)
    d = rng.standard_normal(100000) * np.exp(rng.uniform(np.log(1e-9), 0, 100000))
    xn = xs + d
    out = np.empty_like(xs)
    h.df_diff_batch(_p(xn), _p(xs), xs.size, _p(out))
    ref = xn.astype(np.longdouble) - xs.astype(np.longdouble)
    assert np.max(np.abs((out - ref) / ref)) < 2.0 ** -47


def test_to_double_rounding(h):
    rng = np.random.default_rng(3)
    x = rng.standard_normal(100000) * np.exp(rng.uniform(-30, 30, 100000))
    # include exact powers of two with low parts of both signs
    p2 = np.ldexp(1.0, rng.integers(-40, 40, 2000)) * rng.choice([-1.0, 1.0], 2000)
    x = np.concatenate([x, p2])
    hi = x.astype(np.float32)
    lo = (x - hi.astype(np.float64)).astype(np.float32)
    lo[-2000:] = (np.float32(2.0) ** -30 * rng.standard_normal(2000).astype(np.float32)) * hi[-2000:]
    out = np.empty(x.size)
    h.df_to_double_batch(hi.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                         lo.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), x.size, _p(out))
    exact = hi.astype(np.longdouble) + lo.astype(np.longdouble)
    # zero and non-finite leading parts
    z = np.zeros(4, np.float32)
    hz = np.array([0.0, -0.0, np.inf, -np.inf], np.float32)
    oz = np.empty(4)
    h.df_to_double_batch(hz.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                         z.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), 4, _p(oz))
    assert oz[0] == 0.0 and oz[1] == 0.0 and np.signbit(oz[1]) and oz[2] == np.inf and oz[3] == -np.inf
    # within one double ulp of the exact sum (round half away at the last bit)
    ulp = np.spacing(np.abs(out))
    assert np.all(np.abs(out.astype(np.longdouble) - exact) <= ulp.astype(np.longdouble))


def test_scale_to_f32_matches_scaled_conversion(h):
    """The equilibration's integer conversion equals (float)(v * 2^s) bit for
    bit: random magnitudes, exact ties (even and odd), zeros, values whose
    result leaves the FP32 range."""
    rng = np.random.default_rng(11)
    n = 200000
    v = rng.standard_normal(n) * 10.0 ** rng.uniform(-12, 12, n)
    s = rng.integers(-60, 60, n).astype(np.int32)
    # ties: 24 significant bits then exactly half an FP32 ulp
    m = rng.integers(1 << 23, 1 << 24, 4000).astype(np.float64)
    ties = (m + 0.5) * 2.0 ** rng.integers(-30, 30, 4000)
    v = np.concatenate([v, ties, -ties, [0.0, -0.0, 1e-300, -1e300, 3.4e38, 1e-45]])
    s = np.concatenate([s, np.zeros(8000, np.int32), np.array([0, 0, 900, -900, 1, 0], np.int32)])
    out = np.empty(len(v), np.float32)
    h.df_scale_to_f32_batch(_p(v), s.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(v),
                            out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    with np.errstate(over="ignore"):  # the 1e300 case overflows to -inf on purpose
        ref = (v * np.ldexp(1.0, s)).astype(np.float32)
    assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))
