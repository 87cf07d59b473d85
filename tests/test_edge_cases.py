"""Degenerate inputs of the frame loop, bit-exact against the oracle: an empty volume (nothing
but the environment), a single occupied brick in the box's last corner, the camera inside the
volume, and tiny or ragged image sizes (1x1, 7x3, 13x17: partial 8-pixel tiles on both axes)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scene_with(vlib, density, W, H, cam_radius=2.5):
    from volumetricrestirrelease_gb300 import scenes
    from volumetricrestirrelease_gb300.restir import Volume
    sc = scenes.small(width=W, height=H)
    sc.camera_radius = cam_radius
    vol = Volume.dense(density, (-0.5, -0.5, -0.5), 1.0 / density.shape[0], num_mips=3, lib=vlib)
    return sc, vol


def _run(vlib, cuda, sc, vol, frames=3):
    from oracle.oracle import Oracle
    from tests.test_parity_gpu import _compare_frame
    from volumetricrestirrelease_gb300 import capi
    from volumetricrestirrelease_gb300.restir import VolumetricReSTIR
    opts = capi.default_options(vlib)
    for k, v in sc.options.items():
        setattr(opts, k, v)
    gpu = VolumetricReSTIR(sc.width, sc.height, opts.as_dict(), lib=vlib)
    gpu.setScene(vol, sc.medium, sc.lights, sc.env_rgb, sc.env_scale)
    ora = Oracle(sc.width, sc.height, opts)
    ora.set_volume(vol, sc.medium)
    ora.set_lights(sc.lights, sc.env_rgb, sc.env_scale)
    imgs = [_compare_frame(gpu, ora, opts, cuda, sc.camera(f), f) for f in range(frames)]
    assert all(np.isfinite(i).all() for i in imgs)
    return imgs


def test_empty_volume(vlib, cuda):
    sc, vol = _scene_with(vlib, np.zeros((64, 64, 64), np.float32), 40, 24)
    imgs = _run(vlib, cuda, sc, vol)
    # only the environment remains: the constant 0.2 sky through an empty medium
    assert np.allclose(imgs[-1][..., :3], 0.2, rtol=1e-4)


def test_single_brick_in_the_last_corner(vlib, cuda):
    g = np.zeros((64, 64, 64), np.float32)
    g[56:64, 56:64, 56:64] = 0.8
    sc, vol = _scene_with(vlib, g, 48, 32)
    sc.camera_radius = 1.6
    _run(vlib, cuda, sc, vol)


def test_camera_inside_the_volume(vlib, cuda):
    rng = np.random.default_rng(5)
    g = (rng.random((64, 64, 64)) * 0.6).astype(np.float32)
    sc, vol = _scene_with(vlib, g, 40, 32, cam_radius=0.2)
    _run(vlib, cuda, sc, vol)


@pytest.mark.parametrize("size", [(1, 1), (7, 3), (13, 17)])
def test_tiny_and_ragged_images(vlib, cuda, size):
    from volumetricrestirrelease_gb300 import scenes
    from volumetricrestirrelease_gb300.restir import Volume
    W, H = size
    sc = scenes.small(width=W, height=H)
    vol = Volume.procedural(sc.volume, lib=vlib)
    _run(vlib, cuda, sc, vol)
