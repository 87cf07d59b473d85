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


def test_frame_hook_chain(vlib, cuda):
    """vr_set_frame_hook in the slot of the reference graph's post chain (VolumetricReSTIR ->
    AccumulatePass -> OptixDenoiser): a hook that accumulates each frame in place makes every
    output, on the device and through the pipelined host path, the FP64 running mean of the
    frames rendered without it, bit for bit; the hook sees the caller's motion-vector buffer and
    the frame's stream, and removing it restores the plain output."""
    from volumetricrestirrelease_gb300 import capi, scenes
    from volumetricrestirrelease_gb300.restir import Volume, VolumetricReSTIR
    sc = scenes.small(width=64, height=48)
    W, H = sc.width, sc.height
    vol = Volume.procedural(sc.volume, lib=vlib)
    opts = capi.default_options(vlib)
    for k, v in sc.options.items():
        setattr(opts, k, v)

    def ctx():
        r = VolumetricReSTIR(W, H, opts.as_dict(), lib=vlib)
        r.setScene(vol, sc.medium, sc.lights, sc.env_rgb, sc.env_scale)
        return r
    out = cuda.empty((H, W, 4), device="cuda", dtype=cuda.float32)
    mvec = cuda.empty((H, W, 2), device="cuda", dtype=cuda.float32)
    plain = ctx()
    frames = []
    for f in range(4):
        plain.execute(sc.camera(f), out.data_ptr())
        cuda.cuda.synchronize()
        frames.append(out.cpu().numpy().astype(np.float64))
    want = [(np.sum(frames[:k + 1], 0) / (k + 1)).astype(np.float32) for k in range(4)]

    stream = cuda.cuda.current_stream().cuda_stream
    for path in ("device", "host"):
        acc = C.c_void_p()
        assert vlib.vr_accumulator_create(W, H, 0, C.byref(acc)) == 0
        calls = []

        def hook(rgba, mv, w, h, st):
            calls.append((rgba, mv, w, h, st))
            assert vlib.vr_accumulate(acc, C.c_void_p(rgba), C.c_void_p(rgba), C.c_void_p(st)) == 0
        r = ctx()
        r.set_frame_hook(hook)
        try:
            if path == "device":
                for f in range(3):
                    r.execute(sc.camera(f), out.data_ptr(), mvec.data_ptr(), stream=stream)
                    cuda.cuda.synchronize()
                    got = out.cpu().numpy()
                    assert np.array_equal(got.view(np.uint32), want[f].view(np.uint32)), f
                assert all(c[0] == out.data_ptr() and c[1] == mvec.data_ptr() and c[2:4] == (W, H) and c[4] == stream for c in calls)
            else:
                hosts = [np.zeros((H, W, 4), np.float32) for _ in range(3)]
                for f in range(3):
                    assert vlib.vr_render_frame_host_async(r._h, C.byref(sc.camera(f)), hosts[f].ctypes.data_as(C.POINTER(C.c_float)),
                                                           C.c_void_p(stream)) == 0
                assert vlib.vr_host_frames_wait(r._h) == 0
                for f in range(3):
                    assert np.array_equal(hosts[f].view(np.uint32), want[f].view(np.uint32)), f
                assert len(calls) == 3 and all(c[1] == 0 for c in calls)
            # without the hook the next frame is the plain one
            r.set_frame_hook(None)
            r.execute(sc.camera(3), out.data_ptr(), stream=stream)
            cuda.cuda.synchronize()
            assert np.array_equal(out.cpu().numpy().view(np.uint32), frames[3].astype(np.float32).view(np.uint32))
            assert len(calls) == 3
        finally:
            vlib.vr_accumulator_destroy(acc)
