"""Failure handling, injected on the host (no GPU fault): every device allocation of a context
can be made to fail as an out-of-memory would (vr_debug_fail_allocation).  For every allocation
point of a setup + frames sequence in turn, the failing call must return VR_ERR_OOM and leave the
context usable: retried once the injection is off, the sequence must produce images
bit-identical to a run without injection."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sequence(vlib, cuda, sc, opts, vols, inject_at, frames=3):
    from volumetricrestirrelease_gb300 import capi
    from volumetricrestirrelease_gb300.restir import env_struct
    W, H = sc.width, sc.height
    state = {"oom": 0}
    vlib.vr_debug_fail_allocation(inject_at)

    def call(fn):
        r = fn()
        if r == capi.VR_ERR_OOM:
            state["oom"] += 1
            vlib.vr_debug_fail_allocation(-1)
            r = fn()
        assert r == capi.VR_OK, r

    err = C.c_int32()
    ctx = vlib.vr_create(C.byref(opts), W, H, C.byref(err))
    if not ctx:
        assert err.value == capi.VR_ERR_OOM
        state["oom"] += 1
        vlib.vr_debug_fail_allocation(-1)
        ctx = vlib.vr_create(C.byref(opts), W, H, C.byref(err))
    assert ctx
    imgs = []
    try:
        call(lambda: vlib.vr_set_volume(ctx, vols[0]._h, C.byref(sc.medium)))
        lights = (capi.PointLight * len(sc.lights))(*sc.lights)
        env, keep = env_struct(sc.env_rgb, sc.env_scale)
        call(lambda: vlib.vr_set_lights(ctx, lights, len(sc.lights), C.byref(env)))
        if vols[1] is not None:
            call(lambda: vlib.vr_set_emission(ctx, vols[1]._h, *sc.fire[2:], None))
        out = cuda.empty((H, W, 4), device="cuda", dtype=cuda.float32)
        for f in range(frames - 1):
            cam = sc.camera(f)
            call(lambda: vlib.vr_render_frame(ctx, C.byref(cam), C.c_void_p(out.data_ptr()), None, None))
            cuda.cuda.synchronize()
            imgs.append(out.cpu().numpy().copy())
        host = np.zeros((H, W, 4), np.float32)
        cam = sc.camera(frames - 1)
        call(lambda: vlib.vr_render_frame_host_async(ctx, C.byref(cam), host.ctypes.data_as(C.POINTER(C.c_float)), None))
        call(lambda: vlib.vr_host_frames_wait(ctx))
        imgs.append(host)
    finally:
        vlib.vr_debug_fail_allocation(-1)
        vlib.vr_destroy(ctx)
    return imgs, state["oom"]


@pytest.mark.parametrize("kind", ["plain", "learned", "fire"])
def test_every_allocation_failure_is_recoverable(vlib, cuda, kind):
    from volumetricrestirrelease_gb300 import capi, scenes
    if kind == "fire":
        sc = scenes.fire(width=32, height=24, res=64)
    else:
        sc = scenes.small(width=32, height=24)
    vols = scenes.make_volumes(sc, vlib)
    opts = capi.default_options(vlib)
    for k, v in sc.options.items():
        setattr(opts, k, v)
    if kind == "learned":
        opts.mUseLearnedPHat, opts.mLearnedTrainSamples, opts.mLearnedBatch = 1, 256, 128
    ref, n0 = _sequence(vlib, cuda, sc, opts, vols, -1)
    assert n0 == 0
    points = 0
    for at in range(0, 400):
        imgs, ooms = _sequence(vlib, cuda, sc, opts, vols, at)
        if ooms == 0:                    # past the last allocation of the sequence
            break
        points += 1
        assert ooms == 1
        for f, (a, b) in enumerate(zip(imgs, ref)):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (at, f)
    else:
        pytest.fail("more than 400 allocations")
    assert points > 20
