"""Vertex reuse (the reference's VERTEX_REUSE define, mVertexReuse / mVertexReuseStartBounce):
from indirect vertex mVertexReuseStartBounce on a path's suffix is stored as vertex positions,
spatial reuse reconnects the shifted prefix to the same suffix vertex and reuses the suffix's
share of p_hat (p_partial) instead of re-marching it (ReSTIRHelper.slang:91-420,
ComputeInitialSample.slang:88-127, 322-330, Reservoir.slang:46-48, 76-78).

CPU: the oracle's form against its own plain form (different, finite, p_partial kept).  GPU:
frames, reservoirs (with p_partial), suffixes and features bit-exact against the oracle, for
start bounces 1 and 2, path lengths 2 and 3, and an emissive fire plume; the refusals.
"""
import numpy as np
import pytest


def _oracle_frames(vr, start=1, mb=3, frames=2, W=40, H=32):
    from oracle import oracle as O
    from volumetricrestirrelease_gb300 import scenes
    sc = scenes.small(width=W, height=H)
    vol = O.OracleVolume(sc.volume)
    opts = O.default_options(**dict(sc.options, mMaxBounces=mb, mVertexReuse=int(vr), mVertexReuseStartBounce=start))
    ora = O.Oracle(W, H, opts)
    ora.set_volume(vol, sc.medium)
    ora.set_lights(sc.lights, sc.env_rgb, sc.env_scale)
    imgs = [ora.render_frame(sc.camera(f)) for f in range(frames)]
    return imgs, ora.export_reservoirs(0), ora.export_extra(0)


def test_oracle_vertex_reuse_changes_the_estimator():
    plain, rp, _ = _oracle_frames(False)
    reuse, rv, ev = _oracle_frames(True)
    assert all(np.isfinite(x).all() for x in reuse)
    assert not np.array_equal(plain[-1], reuse[-1])
    assert (rv["p_partial"] > 0).any()
    assert np.all(rp["p_partial"] == 0)
    # the same scene, so the image means agree to within the noise of two frames
    assert abs(plain[-1][..., :3].mean() - reuse[-1][..., :3].mean()) < 0.25 * plain[-1][..., :3].mean()


@pytest.mark.gpu
@pytest.mark.parametrize("overrides", [dict(mMaxBounces=3, mVertexReuse=1, mVertexReuseStartBounce=1),
                                       dict(mMaxBounces=3, mVertexReuse=1, mVertexReuseStartBounce=2),
                                       dict(mMaxBounces=2, mVertexReuse=1, mVertexReuseStartBounce=1),
                                       dict(mMaxBounces=3, mVertexReuse=1, mEnableTemporalReuse=0)],
                         ids=["mb3-start1", "mb3-start2", "mb2", "mb3-spatial-only"])
def test_vertex_reuse_bit_exact(vlib, cuda, overrides):
    from tests.test_parity_gpu import _run
    from volumetricrestirrelease_gb300 import scenes
    imgs = _run(vlib, cuda, scenes.small, 64, 48, 3, overrides)
    assert imgs[-1][..., :3].mean() > 0.05


@pytest.mark.gpu
def test_vertex_reuse_fire_bit_exact(vlib, cuda):
    from tests.test_emission import _setup_fire
    from tests.test_parity_gpu import _compare_frame
    sc, vols, opts, gpu, ora = _setup_fire(vlib, 56, 40, dict(mVertexReuse=1, mVertexReuseStartBounce=1))
    for f in range(3):
        img = _compare_frame(gpu, ora, opts, cuda, sc.camera(f), f)
    assert img[..., :3].max() > 0


@pytest.mark.gpu
def test_vertex_reuse_refusals(vlib, cuda):
    import ctypes as C
    from volumetricrestirrelease_gb300 import capi
    o = capi.default_options(vlib)
    o.mMaxBounces = 3
    o.mVertexReuse = 1
    o.mUseLearnedPHat = 1
    err = C.c_int32()
    assert not vlib.vr_create(C.byref(o), 32, 32, C.byref(err)) and err.value == capi.VR_ERR_INVALID_ARG
    o.mUseLearnedPHat = 0
    o.mVertexReuseStartBounce = 0
    assert not vlib.vr_create(C.byref(o), 32, 32, C.byref(err)) and err.value == capi.VR_ERR_INVALID_ARG
