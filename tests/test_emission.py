"""Volume emission (fire plumes): blackbody table, temperature lookup and the frame loop with
emissive media against the oracle.

Bars: the table is the project's own Planck/CIE integration (checked for its physics: the
Wien shift of the colour, the Stefan-Boltzmann growth of the luminance, white near 6400 K);
GPU frames of an emissive plume bit-exact against the oracle, in the ReSTIR passes and in the
FP64 path-traced reference.
"""
import numpy as np
import pytest


def test_blackbody_table_physics(vlib):
    from volumetricrestirrelease_gb300.restir import blackbody_lut
    L = blackbody_lut(vlib).astype(np.float64)
    T = 50.0 + 50.0 * np.arange(128)
    Y = L @ np.array([0.2126, 0.7152, 0.0722])
    assert np.all(L >= 0) and abs(Y[-1] - 1.0) < 1e-3
    hot = T >= 1000
    assert np.all(np.diff(Y[hot]) > 0)                      # brighter with temperature
    # luminance grows much faster than T^4 in the visible band at low T and slower near 6400 K
    assert Y[np.searchsorted(T, 3000)] / Y[np.searchsorted(T, 1500)] > (2.0 ** 4)
    # colour: red-dominated at 1500 K, balanced at 6400 K (D65 white point is 6504 K)
    i1500 = np.searchsorted(T, 1500)
    assert L[i1500, 0] > 5 * L[i1500, 1] > 0 and L[i1500, 2] < L[i1500, 1]
    assert np.all(np.abs(L[-1] / L[-1].mean() - 1) < 0.1)
    # blue fraction rises monotonically with temperature
    frac = L[hot, 2] / L[hot].sum(1)
    assert np.all(np.diff(frac) >= -1e-6)


def test_fire_volumes(vlib):
    from volumetricrestirrelease_gb300 import scenes
    sc = scenes.fire(width=32, height=32, res=64)
    d, t = scenes.make_volumes(sc, vlib)
    di, ti = d.info(), t.info()
    assert di.res == ti.res == 64 and ti.num_mips == 1 and di.num_mips == 3
    tv = t.slot(0)
    n = tv.num_bricks
    vals = np.ctypeslib.as_array(tv.brick_f32, shape=(n * 1000,))
    pos = vals[vals > 0]
    assert pos.min() >= 500.0 - 1e-3 and pos.max() <= 3000.0 + 1e-3


def _setup_fire(vlib, W, H, overrides=None, res=64, gpu=True):
    from oracle.oracle import Oracle
    from volumetricrestirrelease_gb300 import capi, scenes
    from volumetricrestirrelease_gb300.restir import VolumetricReSTIR
    sc = scenes.fire(width=W, height=H, res=res)
    vol, temp = scenes.make_volumes(sc, vlib)
    opts = capi.default_options(vlib)
    for k, v in {**sc.options, **(overrides or {})}.items():
        setattr(opts, k, v)
    tmin, tmax, le, cut, scale = sc.fire
    if gpu:
        gpu = VolumetricReSTIR(W, H, opts.as_dict(), lib=vlib)
        gpu.setScene(vol, sc.medium, sc.lights, sc.env_rgb, sc.env_scale)
        gpu.setEmission(temp, le, cut, scale)
    ora = Oracle(W, H, opts)
    ora.set_volume(vol, sc.medium)
    ora.set_lights(sc.lights, sc.env_rgb, sc.env_scale)
    ora.set_emission(temp, le, cut, scale)
    return sc, (vol, temp), opts, gpu, ora


@pytest.mark.gpu
@pytest.mark.parametrize("overrides", [dict(), dict(mMaxBounces=2, mInitialM=8), dict(mUseLearnedPHat=1, mLearnedTrainSamples=1024,
                                                                                        mLearnedBatch=512)],
                         ids=["plain", "mb2", "learned"])
def test_fire_frames_bit_exact(vlib, cuda, overrides):
    from tests.test_parity_gpu import _compare_frame
    sc, vols, opts, gpu, ora = _setup_fire(vlib, 64, 48, overrides)
    img = None
    for f in range(3):
        if opts.mUseLearnedPHat:
            out = cuda.empty((48, 64, 4), device="cuda", dtype=cuda.float32)
            gpu.execute(sc.camera(f), out.data_ptr())
            cuda.cuda.synchronize()
            ora.set_lp_T(gpu.export_learned(0))
            ref = ora.render_frame(sc.camera(f))
            img = out.cpu().numpy()
            assert np.array_equal(img.view(np.uint32), ref.view(np.uint32)), f"frame {f}"
        else:
            img = _compare_frame(gpu, ora, opts, cuda, sc.camera(f), f)
    assert img[..., :3].max() > 0


@pytest.mark.gpu
def test_fire_reference_fp64(vlib, cuda):
    sc, vols, opts, gpu, ora = _setup_fire(vlib, 40, 32, dict(mBaselineSamplePerPixel=1))
    acc = cuda.zeros((32, 40, 3), device="cuda", dtype=cuda.float64)
    gpu.render_reference(sc.camera(0), acc.data_ptr(), 0, 8)
    cuda.cuda.synchronize()
    ref = ora.render_reference(sc.camera(0), 0, 8)
    assert np.array_equal(acc.cpu().numpy().view(np.uint64), ref.view(np.uint64))


def test_emission_oracle_changes_image(vlib):
    """Emission on vs off on the CPU oracle: the plume glows (more light, warmer)."""
    sc, vols, opts, _, ora = _setup_fire(vlib, 24, 18, dict(mInitialM=4), gpu=False)
    on = ora.render_frame(sc.camera(0))
    from oracle.oracle import Oracle
    off = Oracle(24, 18, opts)
    off.set_volume(vols[0], sc.medium)
    off.set_lights(sc.lights, sc.env_rgb, sc.env_scale)
    img_off = off.render_frame(sc.camera(0))
    assert on[..., 0].sum() > img_off[..., 0].sum()
    assert (on[..., 0] - img_off[..., 0]).sum() > (on[..., 2] - img_off[..., 2]).sum()
