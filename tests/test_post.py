"""Post-process passes: frame accumulation (AccumulatePass) and error measurement
(ErrorMeasurePass) on the GPU.

Bars: every accumulation mode equals the same per-pixel arithmetic in numpy bit for bit (double
sums with the mean rounded to float; float sums; Kahan-compensated float sums), over frames
with values far apart in magnitude; the error modes equal numpy's FP64 evaluation of the
same per-pixel terms to 1e-12 relative (the per-pixel terms bit for bit); the relative MSE
is the metric the benchmark computes on the host; bad arguments are refused.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _frames(n, H, W, seed=4):
    rng = np.random.default_rng(seed)
    out = []
    for f in range(n):
        scale = 10.0 ** rng.integers(-3, 4)
        out.append((rng.random((H, W, 4)) * scale).astype(np.float32))
    return out


@pytest.mark.parametrize("precision", [0, 1, 2], ids=["double", "single", "kahan"])
def test_accumulation_modes(vlib, cuda, precision):
    H, W = 37, 53
    frames = _frames(9, H, W)
    acc = C.c_void_p()
    assert vlib.vr_accumulator_create(W, H, precision, C.byref(acc)) == 0
    try:
        out = cuda.empty((H, W, 4), device="cuda", dtype=cuda.float32)
        for rep in range(2):                     # a reset restarts the sums
            if rep:
                vlib.vr_accumulator_reset(acc)
            s64 = np.zeros((H, W, 4), np.float64)
            s32 = np.zeros((H, W, 4), np.float32)
            c32 = np.zeros((H, W, 4), np.float32)
            for i, fr in enumerate(frames):
                src = cuda.from_numpy(fr).cuda()
                assert vlib.vr_accumulate(acc, C.c_void_p(src.data_ptr()), C.c_void_p(out.data_ptr()), None) == 0
                cuda.cuda.synchronize()
                got = out.cpu().numpy()
                if precision == 0:
                    s64 += fr.astype(np.float64)
                    ref = (s64 / np.float64(i + 1)).astype(np.float32)
                elif precision == 1:
                    s32 = (s32 + fr).astype(np.float32)
                    ref = (s32 / np.float32(i + 1)).astype(np.float32)
                else:
                    y = (fr - c32).astype(np.float32)
                    t = (s32 + y).astype(np.float32)
                    c32 = ((t - s32).astype(np.float32) - y).astype(np.float32)
                    s32 = t
                    ref = (s32 / np.float32(i + 1)).astype(np.float32)
                assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), (rep, i)
            assert vlib.vr_accumulator_count(acc) == len(frames)
    finally:
        vlib.vr_accumulator_destroy(acc)


@pytest.mark.parametrize("mode", [0, 2, 4, 6, 1, 8, 12], ids=["abs", "sqr", "abs_avg", "sqr_avg", "abs_nobg", "relmse", "relmse_avg"])
def test_error_measure(vlib, cuda, mode):
    H, W = 61, 47
    rng = np.random.default_rng(mode)
    src = rng.random((H, W, 4)).astype(np.float32)
    ref = (rng.random((H, W, 4)) * 2).astype(np.float32)
    wpos = rng.random((H, W, 4)).astype(np.float32)
    wpos[rng.random((H, W)) < 0.3, 3] = 0.0
    eps = 0.01
    ds, dr, dw = (cuda.from_numpy(a).cuda() for a in (src, ref, wpos))
    diff = cuda.empty((H, W, 4), device="cuda", dtype=cuda.float32)
    err = (C.c_double * 3)()
    assert vlib.vr_error_measure(C.c_void_p(ds.data_ptr()), C.c_void_p(dr.data_ptr()), C.c_void_p(dw.data_ptr()), W, H, mode, eps, err,
                                 C.c_void_p(diff.data_ptr()), None) == 0
    # the same per-pixel terms in float32 arithmetic
    d = np.abs(src[..., :3] - ref[..., :3]).astype(np.float32)
    if mode & 8:
        d = ((d * d).astype(np.float32) / (ref[..., :3] * ref[..., :3] + np.float32(eps)).astype(np.float32)).astype(np.float32)
    elif mode & 2:
        d = (d * d).astype(np.float32)
    if mode & 4:
        m = (((d[..., 0] + d[..., 1]).astype(np.float32) + d[..., 2]).astype(np.float32) / np.float32(3)).astype(np.float32)
        d = np.stack([m, m, m], -1)
    if mode & 1:
        d[wpos[..., 3] == 0] = 0
    got = diff.cpu().numpy()[..., :3]
    assert np.array_equal(got.view(np.uint32), d.view(np.uint32))
    e = d.astype(np.float64).reshape(-1, 3).sum(0) / (H * W)
    assert np.allclose(np.array(err[:]), e, rtol=1e-12, atol=0)


def test_relmse_matches_the_benchmark_metric(vlib, cuda):
    import bench
    H, W = 33, 29
    rng = np.random.default_rng(9)
    img = (rng.random((H, W, 4)) * 3).astype(np.float32)
    ref = rng.random((H, W, 3))
    ref4 = np.concatenate([ref, np.zeros((H, W, 1))], -1).astype(np.float32)
    di, dr = cuda.from_numpy(img).cuda(), cuda.from_numpy(ref4).cuda()
    err = (C.c_double * 3)()
    assert vlib.vr_error_measure(C.c_void_p(di.data_ptr()), C.c_void_p(dr.data_ptr()), None, W, H, 8, 0.01, err, None, None) == 0
    host = bench._relmse(img, ref4[..., :3].astype(np.float64))
    assert abs(np.mean(err[:]) - host) <= 1e-5 * host


def test_bad_arguments(vlib, cuda):
    acc = C.c_void_p()
    assert vlib.vr_accumulator_create(0, 4, 0, C.byref(acc)) != 0
    assert vlib.vr_accumulator_create(4, 4, 7, C.byref(acc)) != 0
    err = (C.c_double * 3)()
    x = cuda.zeros((4, 4, 4), device="cuda", dtype=cuda.float32)
    p = C.c_void_p(x.data_ptr())
    assert vlib.vr_error_measure(p, p, None, 4, 4, 64, 0.0, err, None, None) != 0
    assert vlib.vr_error_measure(p, p, None, 4, 4, 8, -1.0, err, None, None) != 0
