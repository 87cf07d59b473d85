"""The tcgen05 tensor-core building block (BF16 x BF16 -> FP32 in TMEM) against a CPU product."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bf16(x):
    u = np.asarray(x, np.float32).view(np.uint32)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    return r, (r.astype(np.uint32) << 16).view(np.float32)


def test_umma_128x64x64(vlib, cuda):
    rng = np.random.default_rng(5)
    a16, a = _bf16(rng.standard_normal((128, 64)))
    b16, b = _bf16(rng.standard_normal((64, 64)))
    ref = a.astype(np.float64) @ b.astype(np.float64).T
    out = np.zeros((128, 64), np.float32)
    p16 = lambda x: np.ascontiguousarray(x).ctypes.data_as(C.POINTER(C.c_uint16))
    r = vlib.vr_selftest_umma(p16(a16), p16(b16), out.ctypes.data_as(C.POINTER(C.c_float)), 0)
    assert r == 0
    assert np.abs(out - ref).max() < 1e-3 * np.abs(ref).max()
