"""Analytic known answers for the oracle's volume tracking (the reference's tests pin only the
RNG; these pin the tracking estimators on media with closed-form answers)."""
import ctypes as C
import math

import numpy as np
import pytest

from volumetricrestirrelease_gb300 import capi
from volumetricrestirrelease_gb300.restir import Volume

SIGMA_T = 3.0
RES = 32


@pytest.fixture(scope="module")
def homogeneous(vlib):
    from oracle.oracle import Oracle
    g = np.full((RES, RES, RES), 0.5, np.float32)
    vol = Volume.dense(g, (-1.0, -1.0, -1.0), 2.0 / RES, num_mips=2, lib=vlib)
    m = capi.Medium()
    m.sigma_s[:] = [SIGMA_T * 0.8] * 3
    m.sigma_a[:] = [SIGMA_T - SIGMA_T * 0.8] * 3
    m.g = 0.0
    m.density_scale = 1.0
    o = Oracle(8, 8, capi.default_options(vlib))
    o.set_volume(vol, m)
    return o, vol


def _tr(o, origin, d, tmax, method, linear=1, mip=0, seed=1, tss=1.0):
    oa = (C.c_float * 3)(*origin)
    da = (C.c_float * 3)(*d)
    return o.L.vro_transmittance(o._h, oa, da, tmax, mip, linear, method, tss, seed)


# Closed forms for a ray along +z through the centre of the homogeneous box (32 voxels of
# density 0.5, sigma_t 3, voxel 1/16): point-sampled analytic tracking and midpoint ray
# marching integrate 32 voxels exactly (tau = 3); trilinear analytic tracking walks
# vertex-centred cells and starts at the first cell at or above index 0, skipping the
# half voxel [0, 0.5) where the trilinear field ramps from 0.25 to 0.5 (tau = 3*15.6875/16);
# the (residual) ratio trackers estimate the transmittance of the full trilinear field
# (tau = 3*15.875/16).
TAU_POINT = SIGMA_T * 0.5 * 2.0
TAU_TRI_ANALYTIC = SIGMA_T * 15.6875 * (2.0 / RES)
TAU_TRI = SIGMA_T * 15.875 * (2.0 / RES)


@pytest.mark.parametrize("direction", [(0.0, 0.0, 1.0), (0.03, -0.02, 1.0)])
def test_point_sampled_analytic_tracking(homogeneous, direction):
    o, _ = homogeneous
    d = np.array(direction, np.float64)
    d /= np.linalg.norm(d)
    t = _tr(o, (0.013, -0.021, -3.0), tuple(d), 1e30, capi.VR_TRACK_ANALYTIC, linear=0)
    chord = 2.0 / d[2]
    assert t == pytest.approx(math.exp(-SIGMA_T * 0.5 * chord), rel=2e-5)


def test_segment_ending_inside(homogeneous):
    o, _ = homogeneous
    t = _tr(o, (0.013, -0.021, -3.0), (0.0, 0.0, 1.0), 3.3, capi.VR_TRACK_ANALYTIC, linear=0)
    assert t == pytest.approx(math.exp(-SIGMA_T * 0.5 * 1.3), rel=2e-5)


def test_ray_marching_midpoint(homogeneous):
    o, _ = homogeneous
    for lin in (0, 1):
        t = _tr(o, (0.013, -0.021, -3.0), (0.0, 0.0, 1.0), 1e30, capi.VR_TRACK_RAY_MARCHING, linear=lin)
        assert t == pytest.approx(math.exp(-TAU_POINT), rel=2e-5)


def test_trilinear_analytic_tracking(homogeneous):
    o, _ = homogeneous
    t = _tr(o, (0.013, -0.021, -3.0), (0.0, 0.0, 1.0), 1e30, capi.VR_TRACK_ANALYTIC, linear=1)
    assert t == pytest.approx(math.exp(-TAU_TRI_ANALYTIC), rel=2e-5)


@pytest.mark.parametrize("method", [capi.VR_TRACK_RATIO, capi.VR_TRACK_RESIDUAL_RATIO, capi.VR_TRACK_ANALOG_RESIDUAL_RATIO])
def test_ratio_trackers_unbiased(homogeneous, method):
    o, _ = homogeneous
    vals = np.array([_tr(o, (0.1, 0.2, -3.0), (0.0, 0.0, 1.0), 1e30, method, seed=s) for s in range(3000)])
    expect = math.exp(-TAU_TRI)
    assert abs(vals.mean() - expect) < 4 * vals.std() / math.sqrt(len(vals)) + 1e-4


def test_distance_sampling_mean_free_path(homogeneous):
    o, _ = homogeneous
    sig = SIGMA_T * 0.5
    hits = []
    for s in range(2000):
        out = (C.c_float * 3)()
        o.L.vro_sample_distance(o._h, (C.c_float * 3)(0.05, 0.07, -3.0), (C.c_float * 3)(0, 0, 1), 0, 0, s, out)
        hits.append(out[0])
    hits = np.array(hits)
    inside = hits[hits < 1e30] - 2.0            # the box starts at distance 2
    frac_escape = np.mean(hits >= 1e30)
    assert abs(frac_escape - math.exp(-sig * 2.0)) < 0.03
    # truncated exponential mean on [0, 2]
    mean_trunc = 1 / sig - 2.0 * math.exp(-2 * sig) / (1 - math.exp(-2 * sig))
    assert abs(inside.mean() - mean_trunc) < 0.05


def test_density_lookup_trilinear(homogeneous):
    o, _ = homogeneous
    p = (C.c_float * 3)(0.3, -0.2, 0.1)
    assert o.L.vro_density_world(o._h, p, 0) == pytest.approx(0.5, abs=1e-7)
    p = (C.c_float * 3)(5.0, 0.0, 0.0)
    assert o.L.vro_density_world(o._h, p, 0) == 0.0


@pytest.mark.parametrize("method,linear", [(capi.VR_TRACK_ANALYTIC, 1), (capi.VR_TRACK_ANALYTIC, 0), (capi.VR_TRACK_RESIDUAL_RATIO, 1),
                                           (capi.VR_TRACK_RAY_MARCHING, 1)])
def test_segment_ending_before_the_next_brick(vlib, method, linear):
    """A shadow segment that ends in empty space before the next occupied brick: the tracker
    must stop at the segment's end (the reference's traversal enters the next brick with
    t > tFar and its analytic / residual-ratio adapters then integrate over a negative
    interval, returning T far above 1)."""
    from oracle.oracle import Oracle
    g = np.zeros((64, 64, 64), np.float32)
    g[:, :, 8:16] = 0.5            # first occupied slab of bricks along x (arrays are [z][y][x])
    g[:, :, 40:48] = 0.9           # second slab, beyond the segment's end
    vol = Volume.dense(g, (0.0, 0.0, 0.0), 1.0 / 64, num_mips=1, lib=vlib)
    m = capi.Medium()
    m.sigma_s[:] = [SIGMA_T * 0.8] * 3
    m.sigma_a[:] = [SIGMA_T - SIGMA_T * 0.8] * 3
    m.g = 0.0
    m.density_scale = 1.0
    o = Oracle(8, 8, capi.default_options(vlib))
    o.set_volume(vol, m)
    d = np.array([1.0, 0.013, 0.007])
    d /= np.linalg.norm(d)
    origin = (9.3 / 64, 30.1 / 64, 31.7 / 64)
    tmax = (30.0 - 9.3) / 64 / d[0]          # ends at x = 30 voxels, in the gap
    ts = [_tr(o, origin, tuple(d), tmax, method, linear=linear, seed=s) for s in range(1, 33)]
    if method != capi.VR_TRACK_RESIDUAL_RATIO:        # single ratio-tracking estimates may exceed 1
        for t in ts:
            assert 0.0 <= t <= 1.0 + 1e-6, t
    # about 6.7 voxels of density 0.5 (sigma_t 3, voxel 1/64) lie on the segment
    assert np.mean(ts) == pytest.approx(math.exp(-SIGMA_T * 0.5 * (16 - 9.3) / 64 / d[0]), rel=0.15)


@pytest.mark.parametrize("method,linear", [(capi.VR_TRACK_ANALYTIC, 0), (capi.VR_TRACK_RAY_MARCHING, 0)])
def test_ray_through_cell_corners(vlib, method, linear):
    """A ray along the cube diagonal from a lattice point crosses every cell at a corner, where
    the three side distances of the DDA tie.  The reference's DDA then sets no step mask and
    stalls: the brick walk drops the rest of each brick (here T came out near 1).  The whole
    chord must count, and a ray a hair off the lattice must agree."""
    from oracle.oracle import Oracle
    g = np.zeros((64, 64, 64), np.float32)
    g[16:48, 16:48, 16:48] = 0.5
    vol = Volume.dense(g, (0.0, 0.0, 0.0), 1.0 / 64, num_mips=1, lib=vlib)
    m = capi.Medium()
    m.sigma_s[:] = [SIGMA_T * 0.8] * 3
    m.sigma_a[:] = [SIGMA_T - SIGMA_T * 0.8] * 3
    m.g = 0.0
    m.density_scale = 1.0
    o = Oracle(8, 8, capi.default_options(vlib))
    o.set_volume(vol, m)
    d = (1.0 / math.sqrt(3.0),) * 3
    expect = math.exp(-SIGMA_T * 0.5 * (32 / 64) * math.sqrt(3.0))
    on = _tr(o, (8 / 64,) * 3, d, 1e30, method, linear=linear)
    off = _tr(o, (8.0013 / 64, 7.9991 / 64, 8.0007 / 64), d, 1e30, method, linear=linear)
    # ray marching is a fixed-step quadrature: within a few percent of the closed form
    tol = 0.05 if method == capi.VR_TRACK_RAY_MARCHING else 2e-3
    assert on == pytest.approx(expect, rel=tol)
    assert on == pytest.approx(off, rel=0.01 if method == capi.VR_TRACK_RAY_MARCHING else 2e-3)
