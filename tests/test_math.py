"""The project's deterministic elementary functions: accuracy against float64 numpy on the host
and bit equality between the device and the host."""
import ctypes as C

import numpy as np
import pytest

OPS = {
    "exp": (0, lambda a, b: np.exp(a.astype(np.float64)), lambda r: r.uniform(-104, 89, 200000)),
    "log": (1, lambda a, b: np.log(a.astype(np.float64)), lambda r: np.exp(r.uniform(-100, 88, 200000))),
    "sin": (2, lambda a, b: np.sin(a.astype(np.float64)), lambda r: r.uniform(-50, 50, 200000)),
    "cos": (3, lambda a, b: np.cos(a.astype(np.float64)), lambda r: r.uniform(-50, 50, 200000)),
    "atan2": (4, lambda a, b: np.arctan2(a.astype(np.float64), b.astype(np.float64)), lambda r: r.uniform(-5, 5, 200000)),
    "acos": (5, lambda a, b: np.arccos(a.astype(np.float64)), lambda r: r.uniform(-1, 1, 200000)),
    "pow": (6, lambda a, b: np.power(a.astype(np.float64), b.astype(np.float64)), lambda r: r.uniform(0.01, 4, 200000)),
}
MAX_ULP = {"exp": 2, "log": 2, "sin": 2, "cos": 2, "atan2": 3, "acos": 3, "pow": 16}


def _inputs(name, seed=0):
    r = np.random.default_rng(seed)
    a = OPS[name][2](r).astype(np.float32)
    b = r.uniform(-5, 5, a.size).astype(np.float32) if name == "atan2" else (
        r.uniform(-3, 3, a.size).astype(np.float32) if name == "pow" else None)
    return a, b


def _ulp_err(got, ref):
    ref32 = ref.astype(np.float32)
    spacing = np.spacing(np.abs(ref32)).astype(np.float64)
    spacing = np.maximum(spacing, np.float64(np.finfo(np.float32).smallest_subnormal))
    return np.abs(got.astype(np.float64) - ref) / spacing


@pytest.mark.parametrize("name", list(OPS))
def test_host_accuracy(name):
    from oracle import oracle
    a, b = _inputs(name)
    got = oracle.math_op(OPS[name][0], a, b)
    ref = OPS[name][1](a, b)
    ok = np.isfinite(ref) & (np.abs(ref) < 3e38)
    assert np.all(np.isfinite(got[ok]))
    err = _ulp_err(got[ok], ref[ok])
    assert err.max() <= MAX_ULP[name], f"{name}: max {err.max():.2f} ulp"


def test_special_values():
    from oracle import oracle
    inf, nan = np.float32(np.inf), np.float32(np.nan)
    e = oracle.math_op(0, np.array([0, -0.0, 100, -200, inf, -inf, nan], np.float32))
    assert e[0] == 1 and e[1] == 1 and np.isinf(e[2]) and e[3] == 0 and np.isinf(e[4]) and e[5] == 0 and np.isnan(e[6])
    l = oracle.math_op(1, np.array([1, 0, -1, inf, nan, 1e-45], np.float32))
    assert l[0] == 0 and l[1] == -np.inf and np.isnan(l[2]) and l[3] == np.inf and np.isnan(l[4])
    assert abs(l[5] - np.log(1.401298464e-45)) < 1e-4
    a = oracle.math_op(5, np.array([1, -1, 0, 2], np.float32))
    assert a[0] == 0 and abs(a[1] - np.pi) < 1e-6 and abs(a[2] - np.pi / 2) < 1e-6 and np.isnan(a[3])


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(OPS))
def test_device_equals_host(name, vlib, cuda):
    from oracle import oracle
    a, b = _inputs(name, seed=1)
    host = oracle.math_op(OPS[name][0], a, b)
    dev = np.zeros_like(a)
    fp = lambda x: x.ctypes.data_as(C.POINTER(C.c_float)) if x is not None else None
    assert vlib.vr_selftest_math(OPS[name][0], fp(a), fp(b), fp(dev), a.size) == 0
    assert np.array_equal(dev.view(np.uint32), host.view(np.uint32)), f"{name}: device and host differ"
