"""Host-output frames: the pipelined entry point (two device staging images, copies on a copy
stream overlapping the next frame) delivers exactly the images of the synchronous one."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("learned", [False, True], ids=["plain", "learned"])
def test_async_host_frames_match_sync(vlib, cuda, learned):
    from volumetricrestirrelease_gb300 import capi, scenes
    from volumetricrestirrelease_gb300.restir import VolumetricReSTIR, Volume
    sc = scenes.small(width=96, height=64)
    vol = Volume.procedural(sc.volume, lib=vlib)
    opts = capi.default_options(vlib)
    for k, v in sc.options.items():
        setattr(opts, k, v)
    if learned:
        opts.mUseLearnedPHat, opts.mLearnedTrainSamples, opts.mLearnedBatch = 1, 2048, 512
    a = VolumetricReSTIR(sc.width, sc.height, opts.as_dict(), lib=vlib)
    b = VolumetricReSTIR(sc.width, sc.height, opts.as_dict(), lib=vlib)
    for r in (a, b):
        r.setScene(vol, sc.medium, sc.lights, sc.env_rgb, sc.env_scale)
    n = 5
    bufs = [np.zeros((sc.height, sc.width, 4), np.float32) for _ in range(n)]
    for f in range(n):
        ptr = bufs[f].ctypes.data_as(C.POINTER(C.c_float))
        assert vlib.vr_render_frame_host_async(a._h, C.byref(sc.camera(f)), ptr, None) == 0
    assert vlib.vr_host_frames_wait(a._h) == 0
    for f in range(n):
        ref = b.execute_host(sc.camera(f))
        assert np.array_equal(bufs[f].view(np.uint32), ref.view(np.uint32)), f
    assert np.isfinite(bufs[-1]).all() and bufs[-1][..., :3].mean() > 0
