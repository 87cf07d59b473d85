"""Animated volume sequences: the per-frame advance of the sequence, the previous frame's grids in
the temporal tap's MIS weight (usePrevGridForReproj, ReSTIRHelper.slang:95-96, 450-452) and the
velocity reprojection (TemporalReuse.cs.slang:161-166).

Bars: the oracle renders a sequence of identical frames bit-identically to the static volume
(the plumbing changes nothing when nothing moves); on a drifting cloud the previous-frame grids
and the velocity grid each change the temporal pass, and only from the second frame on; GPU
frames of drifting sequences (plain, FP16 bricks, fire plumes with per-frame temperature, the
learned target) are bit-exact against the oracle through more than one cycle, with the motion
vectors; the API rejects inconsistent sequences.
"""
import ctypes as C

import numpy as np
import pytest


def _oracle(vlib, sc, opts, frames=None, temps=None, vels=None, scale=1.0):
    from oracle.oracle import Oracle
    from volumetricrestirrelease_gb300.restir import Volume
    ora = Oracle(sc.width, sc.height, opts)
    base = Volume.procedural(sc.volume, lib=vlib)
    ora.set_volume(base, sc.medium)
    ora.set_lights(sc.lights, sc.env_rgb, sc.env_scale)
    if sc.fire:
        ora.set_emission(temps[0], *sc.fire[2:])
    if frames is not None:
        ora.set_animation(frames, temps, vels, scale)
    return ora, base


def _opts(vlib, sc, overrides=None):
    from volumetricrestirrelease_gb300 import capi
    o = capi.default_options(vlib)
    for k, v in {**sc.options, **(overrides or {})}.items():
        setattr(o, k, v)
    return o


def test_static_sequence_matches_static_volume(vlib):
    from volumetricrestirrelease_gb300 import scenes
    from volumetricrestirrelease_gb300.restir import Volume
    sc = scenes.animated(width=48, height=40, frames=3)
    opts = _opts(vlib, sc)
    same = [Volume.procedural(sc.volume, lib=vlib) for _ in range(3)]
    ora_a, _ = _oracle(vlib, sc, opts, same)
    ora_s, _ = _oracle(vlib, sc, opts)
    for f in range(4):
        a, s = ora_a.render_frame(sc.camera(f)), ora_s.render_frame(sc.camera(f))
        assert np.array_equal(a.view(np.uint32), s.view(np.uint32)), f"frame {f}"


def test_previous_grid_and_velocity_change_the_temporal_pass(vlib):
    from volumetricrestirrelease_gb300 import scenes
    sc = scenes.animated(width=48, height=40, frames=3)
    frames, temps, vels = scenes.make_animation(sc, vlib)
    runs = {}
    for name, over, v in [("prev+vel", {}, vels), ("cur+vel", dict(mUsePrevVolumeForReproj=0), vels),
                          ("prev", {}, None)]:
        ora, _ = _oracle(vlib, sc, _opts(vlib, sc, over), frames, temps, v)
        runs[name] = [ora.render_frame(sc.camera(f), mvec=True) for f in range(3)]
    for name in ("cur+vel", "prev"):
        a0, m0 = runs[name][0]
        b0, n0 = runs["prev+vel"][0]
        assert np.array_equal(a0.view(np.uint32), b0.view(np.uint32)), f"{name}: frame 0 has no temporal pass"
        assert not np.array_equal(runs[name][1][0], runs["prev+vel"][1][0]), f"{name}: frame 1 unchanged"
    # the velocity moves the reprojection: motion vectors differ where samples sit in the volume
    assert not np.array_equal(runs["prev"][1][1], runs["prev+vel"][1][1])
    assert np.array_equal(runs["cur+vel"][1][1], runs["prev+vel"][1][1])


def _gpu_setup(vlib, sc, opts):
    from volumetricrestirrelease_gb300 import scenes
    from volumetricrestirrelease_gb300.restir import VolumetricReSTIR, Volume
    frames, temps, vels = scenes.make_animation(sc, vlib)
    base = Volume.procedural(sc.volume, lib=vlib)
    gpu = VolumetricReSTIR(sc.width, sc.height, opts.as_dict(), lib=vlib)
    gpu.setScene(base, sc.medium, sc.lights, sc.env_rgb, sc.env_scale)
    if sc.fire:
        gpu.setEmission(temps[0], *sc.fire[2:])
    gpu.set_animation(frames, temps, vels, 1.0)
    ora, _ = _oracle(vlib, sc, opts, frames, temps, vels, 1.0)
    return gpu, ora, (frames, temps, vels, base)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["plain", "fp16", "fire", "learned"])
def test_animated_frames_match_oracle(vlib, cuda, kind):
    from tests.test_parity_gpu import _compare_frame
    from volumetricrestirrelease_gb300 import scenes
    sc = scenes.animated(width=64, height=48, frames=3, fp16=kind == "fp16", fire=kind == "fire")
    over = dict(mUseLearnedPHat=1, mLearnedTrainSamples=1024, mLearnedBatch=512) if kind == "learned" else {}
    opts = _opts(vlib, sc, over)
    gpu, ora, keep = _gpu_setup(vlib, sc, opts)
    mv = cuda.empty((sc.height, sc.width, 2), device="cuda", dtype=cuda.float32)
    for f in range(7):                          # more than two cycles of the 3-frame sequence
        cam = sc.camera(f)
        if kind == "learned":
            out = cuda.empty((sc.height, sc.width, 4), device="cuda", dtype=cuda.float32)
            gpu.execute(cam, out.data_ptr(), mv.data_ptr())
            cuda.cuda.synchronize()
            ora.set_lp_T(gpu.export_learned(0))
            ref, mref = ora.render_frame(cam, mvec=True)
            assert np.array_equal(out.cpu().numpy().view(np.uint32), ref.view(np.uint32)), f"frame {f}"
        else:
            out = cuda.empty((sc.height, sc.width, 4), device="cuda", dtype=cuda.float32)
            gpu.execute(cam, out.data_ptr(), mv.data_ptr())
            cuda.cuda.synchronize()
            ref, mref = ora.render_frame(cam, mvec=True)
            nbad = int((out.cpu().numpy().view(np.uint32) != ref.view(np.uint32)).any(-1).sum())
            assert nbad == 0, f"frame {f}: {nbad} pixels differ"
        if f > 0:
            assert np.array_equal(mv.cpu().numpy(), mref), f"frame {f}: motion vectors differ"
        assert gpu.animation_frame() == f % 3
    assert np.isfinite(out.cpu().numpy()).all()


@pytest.mark.gpu
def test_animation_reset_and_validation(vlib, cuda):
    from tests.test_parity_gpu import _compare_frame
    from volumetricrestirrelease_gb300 import capi, scenes
    from volumetricrestirrelease_gb300.restir import Batch, Volume
    sc = scenes.animated(width=32, height=24, frames=2)
    opts = _opts(vlib, sc)
    gpu, ora, (frames, temps, vels, base) = _gpu_setup(vlib, sc, opts)
    assert gpu.animation_frame() == -1
    # inconsistent sequences are refused
    other = scenes.animated(width=32, height=24, frames=2, res=32)
    wrong = Volume.procedural(other.volume, lib=vlib)
    with pytest.raises(RuntimeError):
        gpu.set_animation([frames[0], wrong])
    with pytest.raises(ValueError):
        gpu.set_animation(frames, None, vels[:3])
    fa = (C.c_void_p * 2)(frames[0]._h, frames[1]._h)
    va = (C.c_void_p * 6)(*([v._h for v in vels[:5]] + [None]))
    assert vlib.vr_set_animation(gpu._h, fa, 2, None, va, 1.0) == capi.VR_ERR_INVALID_ARG
    assert vlib.vr_set_animation(gpu._h, fa, 2, None, None, float("nan")) == capi.VR_ERR_INVALID_ARG
    # batches and the allocation-free frame do not play sequences
    gpu.set_animation(frames, None, vels)
    with pytest.raises(RuntimeError):
        Batch([gpu])
    cam = sc.camera(0)
    out = cuda.empty((sc.height, sc.width, 4), device="cuda", dtype=cuda.float32)
    history_free = _opts(vlib, sc, dict(mEnableTemporalReuse=0))
    assert vlib.vr_set_options(gpu._h, C.byref(history_free)) == capi.VR_OK
    assert vlib.vr_render_frame_noalloc(gpu._h, C.byref(cam), 0, C.c_void_p(out.data_ptr()), None) == capi.VR_ERR_INVALID_ARG
    assert vlib.vr_set_options(gpu._h, C.byref(opts)) == capi.VR_OK
    # option validation
    bad = _opts(vlib, sc, dict(mUsePrevVolumeForReproj=2))
    assert vlib.vr_set_options(gpu._h, C.byref(bad)) == capi.VR_ERR_INVALID_ARG
    # an empty sequence returns to the static volume
    gpu.set_animation([])
    ora.set_animation([])
    assert gpu.animation_frame() == -1
    for f in range(2):
        _compare_frame(gpu, ora, opts, cuda, sc.camera(f), f)
