"""The allocation-free frame entry point (vr_render_frame_noalloc) against vr_render_frame.

vr_render_frame_noalloc serves callers that may not allocate GPU memory while rendering: a host
that hands out a fixed device budget at start-up and forbids later allocations, or a real-time
loop where a cudaMalloc (which can synchronise the whole device) would stall a frame.  It keeps
its per-pixel intermediates in a static device array that every call reuses.  Two calls in a
row, with different cameras, must each give exactly the image vr_render_frame gives on a context
at the same frame count, which shows the second call is not affected by what the first left in
the array.  This file is named so pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

W, H = 64, 64


def _scene_and_opts(vlib, max_bounces=2, spatial=1):
    from volumetricrestirrelease_gb300 import capi, scenes
    from volumetricrestirrelease_gb300.restir import Volume
    sc = scenes.small(width=W, height=H)
    vol = Volume.procedural(sc.volume, lib=vlib)
    opts = capi.default_options(vlib)
    for k, v in sc.options.items():
        setattr(opts, k, v)
    opts.mEnableTemporalReuse = 0
    opts.mMaxBounces = max_bounces
    opts.mEnableSpatialReuse = spatial
    return sc, vol, opts


def _context(vlib, sc, vol, opts, w=W, h=H):
    from volumetricrestirrelease_gb300.restir import VolumetricReSTIR
    r = VolumetricReSTIR(w, h, opts.as_dict(), lib=vlib)
    r.setScene(vol, sc.medium, sc.lights, sc.env_rgb, sc.env_scale)
    return r


def _camera(sc, deg):
    sc.orbit_deg_per_frame = deg
    return sc.camera(1)


def _reference_image(vlib, cuda, sc, vol, opts, cam, frame_index):
    """vr_render_frame's image at frame count `frame_index` (temporal reuse is off, so the earlier
    frames only advance the counter that seeds the RNG and picks the neighbour offsets)."""
    ref_ctx = _context(vlib, sc, vol, opts)
    ref = cuda.empty((H, W, 4), device="cuda", dtype=cuda.float32)
    for _ in range(frame_index + 1):
        ref_ctx.execute(cam, ref.data_ptr())
    cuda.cuda.synchronize()
    return ref.cpu().numpy()


@pytest.mark.parametrize("max_bounces,spatial,frame_index", [(2, 1, 0), (2, 1, 3), (1, 1, 0), (2, 0, 0), (1, 0, 2)])
def test_noalloc_matches_existing_entry_point_twice(vlib, cuda, max_bounces, spatial, frame_index):
    sc, vol, opts = _scene_and_opts(vlib, max_bounces, spatial)
    static_ctx = _context(vlib, sc, vol, opts)
    for call, deg in enumerate((0.0, 7.5)):
        cam = _camera(sc, deg)
        b = _reference_image(vlib, cuda, sc, vol, opts, cam, frame_index)
        out = cuda.full((H, W, 4), float("nan"), device="cuda", dtype=cuda.float32)
        r = vlib.vr_render_frame_noalloc(static_ctx._h, C.byref(cam), frame_index, C.c_void_p(out.data_ptr()), None)
        assert r == 0, vlib.vr_last_error(static_ctx._h)
        cuda.cuda.synchronize()
        a = out.cpu().numpy()
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), f"call {call}: images differ"
        assert a[..., :3].mean() > 0.05
    # the entry point left the context untouched
    assert static_ctx.frame_count == 0


def test_noalloc_rejects_requests_beyond_its_scratch(vlib, cuda):
    sc, vol, opts = _scene_and_opts(vlib)
    big = _context(vlib, sc, vol, opts, w=320, h=240)
    out = cuda.empty((240, 320, 4), device="cuda", dtype=cuda.float32)
    r = vlib.vr_render_frame_noalloc(big._h, C.byref(sc.camera(0)), 0, C.c_void_p(out.data_ptr()), None)
    assert r == 1 and b"65536" in vlib.vr_last_error(big._h)
    # the learned target keeps records the static array has no room for: refused, not ignored
    opts.mUseLearnedPHat = 1
    learned = _context(vlib, sc, vol, opts)
    small = cuda.empty((H, W, 4), device="cuda", dtype=cuda.float32)
    r = vlib.vr_render_frame_noalloc(learned._h, C.byref(sc.camera(0)), 0, C.c_void_p(small.data_ptr()), None)
    assert r == 1 and b"mUseLearnedPHat" in vlib.vr_last_error(learned._h)
