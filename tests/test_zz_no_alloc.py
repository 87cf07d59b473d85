"""The allocation-free frame entry point (vr_render_frame_noalloc) against vr_render_frame.

vr_render_frame_noalloc serves callers that may not allocate GPU memory while rendering
(fixed-budget hosts, real-time loops, code under stream capture): it keeps its per-pixel
intermediates in a static device array that every call reuses.  Two calls in a row, with
different cameras, must each give exactly the image vr_render_frame gives on a fresh context,
which shows the second call is not affected by what the first left in the array.  This file is
named so pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

W, H = 64, 64


def _scene_and_opts(vlib):
    from volumetricrestirrelease_gb300 import capi, scenes
    from volumetricrestirrelease_gb300.restir import Volume
    sc = scenes.small(width=W, height=H)
    vol = Volume.procedural(sc.volume, lib=vlib)
    opts = capi.default_options(vlib)
    for k, v in sc.options.items():
        setattr(opts, k, v)
    opts.mEnableTemporalReuse = 0
    return sc, vol, opts


def _context(vlib, sc, vol, opts, w=W, h=H):
    from volumetricrestirrelease_gb300.restir import VolumetricReSTIR
    r = VolumetricReSTIR(w, h, opts.as_dict(), lib=vlib)
    r.setScene(vol, sc.medium, sc.lights, sc.env_rgb, sc.env_scale)
    return r


def _camera(sc, deg):
    s = sc
    s.orbit_deg_per_frame = deg
    return s.camera(1)


def test_noalloc_matches_existing_entry_point_twice(vlib, cuda):
    sc, vol, opts = _scene_and_opts(vlib)
    static_ctx = _context(vlib, sc, vol, opts)
    for call, deg in enumerate((0.0, 7.5)):
        cam = _camera(sc, deg)
        ref_ctx = _context(vlib, sc, vol, opts)            # fresh context: frame 0
        ref = cuda.empty((H, W, 4), device="cuda", dtype=cuda.float32)
        ref_ctx.execute(cam, ref.data_ptr())
        out = cuda.full((H, W, 4), float("nan"), device="cuda", dtype=cuda.float32)
        r = vlib.vr_render_frame_noalloc(static_ctx._h, C.byref(cam), 0, C.c_void_p(out.data_ptr()), None)
        assert r == 0, vlib.vr_last_error(static_ctx._h)
        cuda.cuda.synchronize()
        a, b = out.cpu().numpy(), ref.cpu().numpy()
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), f"call {call}: images differ"
        assert a[..., :3].mean() > 0.05
    # the entry point left the context untouched
    assert static_ctx.frame_count == 0


def test_noalloc_rejects_sizes_beyond_its_scratch(vlib, cuda):
    sc, vol, opts = _scene_and_opts(vlib)
    big = _context(vlib, sc, vol, opts, w=320, h=240)
    out = cuda.empty((240, 320, 4), device="cuda", dtype=cuda.float32)
    r = vlib.vr_render_frame_noalloc(big._h, C.byref(sc.camera(0)), 0, C.c_void_p(out.data_ptr()), None)
    assert r == 1 and b"65536" in vlib.vr_last_error(big._h)
