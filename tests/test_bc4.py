"""BC4 brick form (the reference's default texture form for its coarse and conservative mips,
Scene.cpp:3161-3181 with ATLAS_COMPRESSION 2; block layout BCHelper.h:9-69).

CPU: the oracle's block decoder against palettes computed by hand from the format definition;
the library's encoder through the C ABI against an independent numpy decoder (nearest palette
entry per texel, endpoints covering the block, exact 0 and 1 kept, no nonzero voxel of a
conservative mip decoded to zero, bounds of the decoded values), and the library's decoder
against the oracle's (the recomputed bounds).  GPU: frames on a BC4 volume bit-exact against
the oracle.
"""
import ctypes as C

import numpy as np
import pytest


def _block(r0, r1, idx):
    w = r0 | (r1 << 8)
    for t, i in enumerate(idx):
        w |= i << (16 + 3 * t)
    return w


def _oracle_decode(oracle_lib, w):
    out = (C.c_float * 16)()
    oracle_lib.vro_bc4_decode_block(C.c_uint64(w), out)
    return np.array(out[:], np.float64)


def test_oracle_decoder_known_blocks(oracle_lib):
    # eight-value palette (red_0 > red_1): red_0, red_1, then (6 r0 + r1) / 7 ... (r0 + 6 r1) / 7
    r0, r1 = 200, 60
    pal8 = [r0, r1] + [((7 - k) * r0 + k * r1) / 7 for k in range(1, 7)]
    idx = [t % 8 for t in range(16)]
    got = _oracle_decode(oracle_lib, _block(r0, r1, idx))
    assert np.allclose(got, [pal8[i] / 255 for i in idx], rtol=0, atol=2e-7)
    # six-value palette (red_0 <= red_1): red_0, red_1, (4 r0 + r1) / 5 ... (r0 + 4 r1) / 5, 0, 1
    r0, r1 = 30, 220
    pal6 = [r0 / 255, r1 / 255] + [((5 - k) * r0 + k * r1) / 5 / 255 for k in range(1, 5)] + [0.0, 1.0]
    idx = [(3 * t) % 8 for t in range(16)]
    got = _oracle_decode(oracle_lib, _block(r0, r1, idx))
    assert np.allclose(got, [pal6[i] for i in idx], rtol=0, atol=2e-7)
    assert got[idx.index(6)] == 0.0
    # the full ranges: 255 / 0 and 0 / 255
    got = _oracle_decode(oracle_lib, _block(255, 0, list(range(8)) * 2))
    assert np.allclose(got[:8], [1, 0, 6 / 7, 5 / 7, 4 / 7, 3 / 7, 2 / 7, 1 / 7], atol=2e-7)
    got = _oracle_decode(oracle_lib, _block(0, 255, list(range(8)) * 2))
    assert np.allclose(got[:8], [0, 1, 1 / 5, 2 / 5, 3 / 5, 4 / 5, 0, 1], atol=2e-7)


def _palettes(w):
    """(n, 8) palettes of n blocks, float64, from the format definition."""
    r0 = (w & 255).astype(np.int64)
    r1 = ((w >> 8) & 255).astype(np.int64)
    k8 = np.array([0, 7, 1, 2, 3, 4, 5, 6])
    p8 = ((7 - k8)[None] * r0[:, None] + k8[None] * r1[:, None]) / 1785.0
    k6 = np.array([0, 5, 1, 2, 3, 4, 0, 0])
    p6 = ((5 - k6)[None] * r0[:, None] + k6[None] * r1[:, None]) / 1275.0
    p6[:, 6] = 0.0
    p6[:, 7] = 1.0
    return np.where((r0 > r1)[:, None], p8, p6), r0, r1


def _volumes(vlib):
    from volumetricrestirrelease_gb300.restir import Volume
    rng = np.random.default_rng(3)
    R = 32
    g = rng.random((R, R, R)).astype(np.float32)
    g[g < 0.35] = 0.0                                     # exact zeros next to nonzero voxels
    g[:, :, : R // 4] *= 1e-4                             # tiny values: the conservative rule
    g[R // 2:, R // 2:, R // 2:] = 0.0                    # empty bricks
    g[2, 3, 4] = g.max() * 1.0                            # the slot maximum decodes to 1
    args = (g, (-0.5, -0.5, -0.5), 1.0 / R)
    return Volume.dense(*args, num_mips=3, lib=vlib), Volume.dense(*args, num_mips=3, lib=vlib).compress_bc4()


def test_encoder_properties(vlib):
    from volumetricrestirrelease_gb300 import capi
    plain, bc4 = _volumes(vlib)
    assert plain.info().bc4 == 0 and bc4.info().bc4 == 1
    assert bc4.info().device_bytes < plain.info().device_bytes
    before = bc4.info().device_bytes
    vlib.vr_volume_compress_bc4(bc4._h)                   # a second call changes nothing
    assert bc4.info().device_bytes == before
    for s in range(capi.VR_NUM_SLOTS):
        a, b = plain.slot(s), bc4.slot(s)
        if not a.valid:
            continue
        nb = a.num_bricks
        orig = np.ctypeslib.as_array(a.brick_f32, shape=(nb * 1000,)).reshape(nb, 10, 10, 10)
        compressed = s % capi.VR_NUM_MAX_MIPS > 0 or s >= capi.VR_NUM_MAX_MIPS
        if not compressed:                                # normal mip 0 keeps its FP32 bricks
            assert bool(b.brick_f32) and not bool(b.brick_bc4)
            assert np.array_equal(np.ctypeslib.as_array(b.brick_f32, shape=(nb * 1000,)), orig.ravel())
            continue
        assert not bool(b.brick_f32) and bool(b.brick_bc4) and nb > 0
        conservative = s >= capi.VR_NUM_MAX_MIPS
        scale = b.bc4_scale
        assert scale == orig.max()
        w = np.ctypeslib.as_array(b.brick_bc4, shape=(nb * 90,)).astype(np.uint64)
        pal, r0, r1 = _palettes(w)
        # texel values in block order: block z * 9 + (y // 4) * 3 + x // 4, texel (y % 4) * 4 + x % 4
        u = np.zeros((nb, 10, 12, 12))
        used = np.zeros((nb, 10, 12, 12), bool)
        u[:, :, :10, :10] = np.clip(orig / scale, 0, 1)
        used[:, :, :10, :10] = True
        ub = u.reshape(nb, 10, 3, 4, 3, 4).transpose(0, 1, 2, 4, 3, 5).reshape(-1, 16)
        usedb = used.reshape(nb, 10, 3, 4, 3, 4).transpose(0, 1, 2, 4, 3, 5).reshape(-1, 16)
        idx = ((w[:, None] >> (16 + 3 * np.arange(16, dtype=np.uint64))) & np.uint64(7)).astype(np.int64)
        dec = np.take_along_axis(pal, idx, 1)
        # endpoints cover the used texels of eight-value blocks; 0 and 1 stay exact
        mode8 = r0 > r1
        umin = np.where(usedb, ub, 2.0).min(1)
        umax = np.where(usedb, ub, -1.0).max(1)
        assert np.all(r1[mode8] / 255.0 <= umin[mode8] + 1e-7) and np.all(r0[mode8] / 255.0 >= umax[mode8] - 1e-7)
        assert np.all(dec[usedb & (ub == 0.0)] == 0.0) if not conservative else True
        assert np.all(np.abs(dec[usedb & (ub == 1.0)] - 1.0) < 1e-6)
        # nearest entry (over the nonzero entries for nonzero texels of conservative mips)
        dist = np.abs(pal[:, None, :] - ub[:, :, None])
        if conservative:
            dist = np.where((pal[:, None, :] == 0.0) & (ub[:, :, None] > 0.0), np.inf, dist)
            assert np.all(dec[usedb & (ub > 0.0)] > 0.0)
        assert np.all(np.abs(dec - ub)[usedb] <= dist.min(2)[usedb] + 1e-6)
        # error: at most half the widest gap of the block's palette (0 and 1 always covered)
        if not conservative:
            srt = np.sort(pal, 1)
            half_gap = 0.5 * np.diff(srt, axis=1).max(1)
            assert np.all((np.abs(dec - ub) <= half_gap[:, None] + 1e-6)[usedb])
        # bounds are those of the decoded values
        bounds = np.ctypeslib.as_array(b.brick_bounds, shape=(nb * 4,)).reshape(nb, 4)
        vox = (dec.reshape(nb, 10, 3, 3, 4, 4).transpose(0, 1, 2, 4, 3, 5).reshape(nb, 10, 12, 12)[:, :, :10, :10]
               * scale)
        assert np.allclose(bounds[:, 1], vox.reshape(nb, -1).max(1), rtol=1e-6, atol=0)
        assert np.allclose(bounds[:, 0], vox.reshape(nb, -1).min(1), rtol=1e-6, atol=0)
        assert np.allclose(bounds[:, 2], vox.reshape(nb, -1).sum(1) / 512, rtol=1e-4, atol=1e-9)


def test_library_and_oracle_decoders_agree(vlib, oracle_lib):
    """The library computes the bounds with its decoder; the oracle's decoder gives the same maxima
    bit for bit."""
    from volumetricrestirrelease_gb300 import capi
    _, bc4 = _volumes(vlib)
    for s in (1, capi.VR_NUM_MAX_MIPS, capi.VR_NUM_MAX_MIPS + 2):
        b = bc4.slot(s)
        nb = b.num_bricks
        w = np.ctypeslib.as_array(b.brick_bc4, shape=(nb * 90,))
        dec = np.stack([_oracle_decode(oracle_lib, int(x)) for x in w]).astype(np.float32)
        vox = (dec.reshape(nb, 10, 3, 3, 4, 4).transpose(0, 1, 2, 4, 3, 5).reshape(nb, 10, 12, 12)[:, :, :10, :10]
               * np.float32(b.bc4_scale))
        bounds = np.ctypeslib.as_array(b.brick_bounds, shape=(nb * 4,)).reshape(nb, 4)
        assert np.array_equal(bounds[:, 1].view(np.uint32), vox.reshape(nb, -1).max(1).view(np.uint32))


@pytest.mark.gpu
@pytest.mark.parametrize("overrides", [
    {},
    dict(mInitialVisibilityUseLinearSampler=1, mSpatialVisibilityTrackingMethod=1, mSpatialLightingTrackingMethod=3),
    dict(mMaxBounces=3, mInitialM=8, mInitialLightingTrackingMethod=0),
], ids=["default", "linear+ratio", "bounces3+analytic"])
def test_bc4_frames_bit_exact(vlib, cuda, overrides):
    from oracle.oracle import Oracle
    from tests.test_parity_gpu import _compare_frame
    from volumetricrestirrelease_gb300 import capi, scenes
    from volumetricrestirrelease_gb300.restir import Volume, VolumetricReSTIR
    sc = scenes.small(width=80, height=64)
    vol = Volume.procedural(sc.volume, lib=vlib).compress_bc4()
    opts = capi.default_options(vlib)
    for k, v in {**sc.options, **overrides}.items():
        setattr(opts, k, v)
    gpu = VolumetricReSTIR(sc.width, sc.height, opts.as_dict(), lib=vlib)
    gpu.setScene(vol, sc.medium, sc.lights, sc.env_rgb, sc.env_scale)
    ora = Oracle(sc.width, sc.height, opts)
    ora.set_volume(vol, sc.medium)
    ora.set_lights(sc.lights, sc.env_rgb, sc.env_scale)
    imgs = [_compare_frame(gpu, ora, opts, cuda, sc.camera(f), f) for f in range(3)]
    assert imgs[-1][..., :3].mean() > 0.02


def test_oracle_renders_bc4_volumes(vlib, oracle_lib):
    """The oracle's BC4 path on the CPU: frames on a BC4 volume are deterministic across thread
    counts, finite, and close to the FP32 volume's frames (the coarse and conservative mips only
    steer sampling and the reuse targets; the shading reads mip 0)."""
    from oracle.oracle import Oracle
    from volumetricrestirrelease_gb300 import capi, scenes
    from volumetricrestirrelease_gb300.restir import Volume
    sc = scenes.small(width=32, height=24)
    opts = capi.default_options(vlib)
    for k, v in sc.options.items():
        setattr(opts, k, v)
    means = {}
    for form in ("fp32", "bc4"):
        vol = Volume.procedural(sc.volume, lib=vlib)
        if form == "bc4":
            vol.compress_bc4()
        imgs = []
        for threads in (1, 3):
            ora = Oracle(sc.width, sc.height, opts, threads=threads)
            ora.set_volume(vol, sc.medium)
            ora.set_lights(sc.lights, sc.env_rgb, sc.env_scale)
            for f in range(3):
                img = ora.render_frame(sc.camera(f))
            imgs.append(img)
        assert np.array_equal(imgs[0].view(np.uint32), imgs[1].view(np.uint32))
        assert np.isfinite(imgs[0]).all()
        means[form] = float(imgs[0][..., :3].mean())
    assert means["fp32"] > 0.02
    assert abs(means["bc4"] - means["fp32"]) < 0.1 * means["fp32"], means


def test_bad_arguments(vlib):
    assert vlib.vr_volume_compress_bc4(None) != 0
    assert vlib.vr_set_frame_hook(None, None, None) != 0
