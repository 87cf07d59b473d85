"""GPU frame loop against the CPU oracle, through the C ABI.

Bar: bit-exact images, reservoirs (selection, M, weights, depths, light ids), extra-bounce
suffixes and features, frame after frame, for the option surface of the pass
(VolumetricReSTIR.h:130-207).  Sizes are small enough for the oracle to finish in seconds.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("runningSum", "M", "depth", "p_y", "lightUV", "lightID", "sampledPixel")


def _setup(vlib, scene_fn, W, H, overrides=None):
    from oracle.oracle import Oracle
    from volumetricrestirrelease_gb300 import capi
    from volumetricrestirrelease_gb300.restir import Volume, VolumetricReSTIR
    sc = scene_fn(width=W, height=H)
    vol = Volume.procedural(sc.volume, lib=vlib)
    opts = capi.default_options(vlib)
    for k, v in {**sc.options, **(overrides or {})}.items():
        setattr(opts, k, v)
    gpu = VolumetricReSTIR(W, H, opts.as_dict(), lib=vlib)
    gpu.setScene(vol, sc.medium, sc.lights, sc.env_rgb, sc.env_scale)
    ora = Oracle(W, H, opts)
    ora.set_volume(vol, sc.medium)
    ora.set_lights(sc.lights, sc.env_rgb, sc.env_scale)
    return sc, vol, opts, gpu, ora


def _same(a, b):
    return np.array_equal(np.asarray(a).view(np.uint32), np.asarray(b).view(np.uint32))


def _compare_frame(gpu, ora, opts, cuda, cam, f, check_buffers=True):
    from volumetricrestirrelease_gb300.restir import as_reservoirs
    out = cuda.empty((gpu.height, gpu.width, 4), device="cuda", dtype=cuda.float32)
    gpu.execute(cam, out.data_ptr(), stream=cuda.cuda.current_stream().cuda_stream)
    cuda.cuda.synchronize()
    img = out.cpu().numpy()
    ref = ora.render_frame(cam)
    nbad = int((img.view(np.uint32) != ref.view(np.uint32)).any(-1).sum())
    assert nbad == 0, f"frame {f}: {nbad} pixels differ from the oracle"
    if not check_buffers or opts.mUseReference:
        return img
    vr = bool(opts.mVertexReuse) and opts.mMaxBounces > 1
    for which in (0, 1) if opts.mEnableTemporalReuse else (0,):
        rg = as_reservoirs(gpu.export_reservoirs(which), opts.mMaxBounces, vr)
        ro = ora.export_reservoirs(which)
        for k in FIELDS + (("p_partial",) if vr else ()):
            assert _same(rg[k], ro[k]), f"frame {f} buffer {which}: reservoir field {k} differs"
        if opts.mMaxBounces > 1:
            # extra-bounce records are compared where a reservoir references them
            eg = gpu.export_extra(which).reshape(-1, opts.mMaxBounces - 1, 3)
            eo = ora.export_extra(which).reshape(-1, opts.mMaxBounces - 1, 3)
            nb = (ro["sampledPixel"] >> 20)
            for b in range(opts.mMaxBounces - 1):
                m = nb > b
                assert _same(eg[m, b], eo[m, b]), f"frame {f} buffer {which}: extra bounce {b} differs"
    fg = gpu.export_features().reshape(-1, 2)
    fo = ora.export_features().reshape(-1, 2)
    assert np.array_equal(fg, fo), f"frame {f}: features differ"
    return img


def _run(vlib, cuda, scene_fn, W, H, frames, overrides=None):
    sc, vol, opts, gpu, ora = _setup(vlib, scene_fn, W, H, overrides)
    imgs = []
    for f in range(frames):
        imgs.append(_compare_frame(gpu, ora, opts, cuda, sc.camera(f), f))
    return imgs


def test_small_scene_bit_exact(vlib, cuda):
    from volumetricrestirrelease_gb300 import scenes
    imgs = _run(vlib, cuda, scenes.small, 128, 128, 5)
    assert imgs[-1][..., :3].mean() > 0.05


def test_full_scene_reduced_resolution(vlib, cuda):
    from volumetricrestirrelease_gb300 import scenes
    _run(vlib, cuda, scenes.full, 160, 90, 4)


def test_fp16_bricks(vlib, cuda):
    from volumetricrestirrelease_gb300 import scenes
    _run(vlib, cuda, lambda **k: scenes.small(fp16=True, **k), 96, 96, 3)


@pytest.mark.parametrize("overrides", [
    dict(mMaxBounces=1, mInitialM=4),
    dict(mMaxBounces=3, mInitialM=16),
    dict(mMaxBounces=4, mInitialM=5),
    dict(mEnableSpatialReuse=0),
    dict(mEnableTemporalReuse=0),
    dict(mEnableSpatialReuse=0, mEnableTemporalReuse=0),
    dict(mSpatialReuseRounds=2, mSpatialSampleCount=6, mSampleRadius=6.0),
    dict(mRandomSamplerType=0),
    dict(mTemporalMISMethod=0, mSpatialMISMethod=0),
    dict(mInitialVisibilityUseLinearSampler=1),
    dict(mSpatialVisibilityTrackingMethod=1, mSpatialLightingTrackingMethod=3),
    dict(mInitialLightingTrackingMethod=0, mFinalVisibilityTrackingMethod=2, mFinalLightTrackingMethod=4),
    dict(mTemporalReprojectionMode=2),
    dict(mTemporalReprojectionMode=1),
    dict(mUseAnalyticLights=0),
    dict(mUseEnvironmentLights=0),
    dict(mVisualizeTotalTransmittance=1),
    dict(mUseReference=1, mBaselineSamplePerPixel=2),
], ids=lambda d: ",".join(f"{k}={v}" for k, v in d.items()))
def test_option_surface(vlib, cuda, overrides):
    from volumetricrestirrelease_gb300 import scenes
    _run(vlib, cuda, scenes.small, 64, 64, 3, overrides)


def test_orbiting_camera_reprojection(vlib, cuda):
    from volumetricrestirrelease_gb300 import scenes

    def orbit(**k):
        s = scenes.small(**k)
        s.orbit_deg_per_frame = 2.0
        return s
    _run(vlib, cuda, orbit, 96, 64, 4)


def test_options_change_resets_history(vlib, cuda):
    from volumetricrestirrelease_gb300 import scenes
    sc, vol, opts, gpu, ora = _setup(vlib, scenes.small, 64, 64)
    for f in range(2):
        _compare_frame(gpu, ora, opts, cuda, sc.camera(f), f)
    opts.mInitialM = 6
    gpu.setParams(mInitialM=6)
    ora.set_options(opts)
    for f in range(2, 4):
        _compare_frame(gpu, ora, opts, cuda, sc.camera(f), f)
    assert gpu.frame_count == 2 and ora.frame_count == 2


def test_reference_path_tracer_fp64(vlib, cuda):
    from volumetricrestirrelease_gb300 import scenes
    sc, vol, opts, gpu, ora = _setup(vlib, scenes.small, 48, 48, dict(mBaselineSamplePerPixel=1))
    acc = cuda.zeros((48, 48, 3), device="cuda", dtype=cuda.float64)
    cam = sc.camera(0)
    gpu.render_reference(cam, acc.data_ptr(), 0, 20)
    gpu.render_reference(cam, acc.data_ptr(), 20, 12)
    cuda.cuda.synchronize()
    ref = ora.render_reference(cam, 0, 32)
    assert np.array_equal(acc.cpu().numpy().view(np.uint64), ref.view(np.uint64))


def test_checkpoint_resume_bit_identical(vlib, cuda):
    from volumetricrestirrelease_gb300 import scenes
    from volumetricrestirrelease_gb300.restir import VolumetricReSTIR
    sc, vol, opts, gpu, ora = _setup(vlib, scenes.small, 64, 64)
    out = cuda.empty((64, 64, 4), device="cuda", dtype=cuda.float32)
    for f in range(3):
        gpu.execute(sc.camera(f), out.data_ptr())
    state = gpu.export_state()
    gpu.execute(sc.camera(3), out.data_ptr())
    cuda.cuda.synchronize()
    a = out.cpu().numpy()
    other = VolumetricReSTIR(64, 64, opts.as_dict(), lib=vlib)
    other.setScene(vol, sc.medium, sc.lights, sc.env_rgb, sc.env_scale)
    other.import_state(state)
    out2 = cuda.empty((64, 64, 4), device="cuda", dtype=cuda.float32)
    other.execute(sc.camera(3), out2.data_ptr())
    cuda.cuda.synchronize()
    assert _same(a, out2.cpu().numpy())
    assert other.frame_count == 4


def test_host_entry_point_matches_device(vlib, cuda):
    from volumetricrestirrelease_gb300 import scenes
    sc, vol, opts, gpu, ora = _setup(vlib, scenes.small, 64, 64)
    img = gpu.execute_host(sc.camera(0))
    ref = ora.render_frame(sc.camera(0))
    assert _same(img, ref)


def test_motion_vectors(vlib, cuda):
    from volumetricrestirrelease_gb300 import scenes

    def orbit(**k):
        s = scenes.small(**k)
        s.orbit_deg_per_frame = 3.0
        return s
    sc, vol, opts, gpu, ora = _setup(vlib, orbit, 64, 64)
    out = cuda.empty((64, 64, 4), device="cuda", dtype=cuda.float32)
    mv = cuda.zeros((64, 64, 2), device="cuda", dtype=cuda.float32)
    for f in range(3):
        gpu.execute(sc.camera(f), out.data_ptr(), mv.data_ptr())
        _, mref = ora.render_frame(sc.camera(f), mvec=True)
    cuda.cuda.synchronize()
    assert _same(mv.cpu().numpy(), mref)


def test_invalid_arguments(vlib, cuda):
    import ctypes as C
    from volumetricrestirrelease_gb300 import capi
    o = capi.default_options(vlib)
    o.mMaxBounces = 9
    err = C.c_int32()
    assert not vlib.vr_create(C.byref(o), 64, 64, C.byref(err)) and err.value == capi.VR_ERR_INVALID_ARG
    o = capi.default_options(vlib)
    h = vlib.vr_create(C.byref(o), 64, 64, C.byref(err))
    assert h
    cam = capi.Camera()
    buf = cuda.empty((64, 64, 4), device="cuda", dtype=cuda.float32)
    # no volume bound yet
    assert vlib.vr_render_frame(h, C.byref(cam), C.c_void_p(buf.data_ptr()), None, None) == capi.VR_ERR_STATE
    assert b"volume" in vlib.vr_last_error(h)
    vlib.vr_destroy(h)
