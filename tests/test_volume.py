"""Sparse brick grid builder (host code) against a numpy restatement of the reference's rules:
mip downsampling and conservative fill (gvdb_volume_gvdb.cpp:2702-2862), per-brick density
bounds over the 10^3 neighbourhood with avg = sum/512 (Scene.cpp:2983-3012), apron of 1."""
import ctypes as C

import numpy as np
import pytest

from volumetricrestirrelease_gb300 import capi
from volumetricrestirrelease_gb300.restir import Volume


def _grid(res, seed=3, sparsity=0.6):
    r = np.random.default_rng(seed)
    g = r.random((res, res, res), dtype=np.float32)
    g[g < sparsity] = 0.0
    # empty a few whole bricks so the grid is sparse
    g[:8, :8, :8] = 0.0
    g[16:24, 8:16, :] = 0.0
    return g


def _slot_arrays(view):
    nb, nl = view.num_bricks, view.num_l1
    root = np.ctypeslib.as_array(view.root_child, (32768,)).copy()
    l1v = np.ctypeslib.as_array(view.l1_vmin, (nl * 4,)).reshape(nl, 4).copy()
    l1c = np.ctypeslib.as_array(view.l1_child, (nl * 4096,)).reshape(nl, 4096).copy()
    bv = np.ctypeslib.as_array(view.brick_vmin, (nb * 4,)).reshape(nb, 4).copy()
    bb = np.ctypeslib.as_array(view.brick_bounds, (nb * 4,)).reshape(nb, 4).copy()
    data = np.ctypeslib.as_array(view.brick_f32, (nb * 1000,)).reshape(nb, 10, 10, 10).copy() if view.brick_f32 else None
    return root, l1v, l1c, bv, bb, data


def _downsample(g):
    h = g.shape[0] // 2
    out = np.zeros((h, h, h), np.float32)
    # res += 0.125 * d in the converter's (x, y, z) loop order; arrays are [z, y, x]
    for ii in range(2):
        for jj in range(2):
            for kk in range(2):
                out = (out + np.float32(0.125) * g[kk::2, jj::2, ii::2]).astype(np.float32)
    return np.where(out > 0, out, 0).astype(np.float32)


def _conservative(g):
    R = g.shape[0]
    p = np.pad(np.maximum(g, 0), 1)
    acc = np.zeros_like(g)
    for ii in (-1, 0, 1):
        for jj in (-1, 0, 1):
            for kk in (-1, 0, 1):
                acc = (acc + p[1 + kk:1 + kk + R, 1 + jj:1 + jj + R, 1 + ii:1 + ii + R]).astype(np.float32)
    avg = (acc / np.float32(27)).astype(np.float32)
    return np.where((g == 0) & (avg > 0), avg, g).astype(np.float32)


def _check_slot(view, g):
    R = g.shape[0]
    root, l1v, l1c, bv, bb, data = _slot_arrays(view)
    occupied = [(z, y, x) for z in range(R // 8) for y in range(R // 8) for x in range(R // 8)
                if (g[z * 8:z * 8 + 8, y * 8:y * 8 + 8, x * 8:x * 8 + 8] > 0).any()]
    assert view.num_bricks == len(occupied)
    pad = np.pad(g, 1)
    got = {}
    for b in range(view.num_bricks):
        x, y, z = bv[b, :3]
        got[(z // 8, y // 8, x // 8)] = b
        nb = pad[z:z + 10, y:y + 10, x:x + 10]
        assert np.array_equal(data[b], nb), "apron / voxel data"
        assert bb[b, 0] == nb.min() and bb[b, 1] == nb.max()
        # sum in the builder's (x, y, z) loop order
        s = np.float32(0)
        for i in range(10):
            for j in range(10):
                for k in range(10):
                    s = np.float32(s + nb[k, j, i])
        assert bb[b, 2] == np.float32(s / np.float32(512))
        # the tree finds the brick
        l1 = root[((z // 128) * 32 + (y // 128)) * 32 + (x // 128)]
        assert l1 >= 0 and tuple(l1v[l1, :3]) == ((x // 128) * 128, (y // 128) * 128, (z // 128) * 128)
        assert l1c[l1, (((z % 128) // 8) * 16 + ((y % 128) // 8)) * 16 + ((x % 128) // 8)] == b
    assert set(got) == set(occupied)


def test_mips_conservative_bounds(vlib):
    g = _grid(32)
    vol = Volume.dense(g, (0.0, 0.0, 0.0), 0.25, num_mips=2, lib=vlib)
    _check_slot(vol.slot(0), g)
    _check_slot(vol.slot(1), _downsample(g))
    c0 = _conservative(g)
    _check_slot(vol.slot(8), c0)
    _check_slot(vol.slot(9), _downsample(c0))
    assert not vol.slot(2).valid and not vol.slot(10).valid
    info = vol.info()
    assert info.num_mips == 2 and abs(info.supervoxel_diag - 8 * np.sqrt(3 * 0.25 ** 2)) < 1e-6


def test_world_to_index(vlib):
    g = _grid(16)
    vol = Volume.dense(g, (-1.0, 2.0, 0.5), 0.125, num_mips=1, lib=vlib)
    M = np.array(vol.slot(0).world_to_index[:], np.float32).reshape(4, 4)
    p = np.array([0.0, 2.5, 1.0, 1.0], np.float32)
    idx = p @ M
    assert np.allclose(idx[:3], [8.0, 4.0, 4.0]) and idx[3] == 1.0


def test_fp16_bricks_round_to_nearest_even(vlib):
    g = _grid(16, sparsity=0.3)
    v32 = Volume.dense(g, (0, 0, 0), 1.0, num_mips=1, lib=vlib)
    v16 = Volume.dense(g, (0, 0, 0), 1.0, num_mips=1, fp16=True, lib=vlib)
    a = v32.slot(0)
    b = v16.slot(0)
    n = a.num_bricks * 1000
    d32 = np.ctypeslib.as_array(a.brick_f32, (n,))
    d16 = np.ctypeslib.as_array(b.brick_f16, (n,)).view(np.float16)
    assert np.array_equal(d32.astype(np.float16), d16)


def test_procedural_sparse_occupancy(vlib):
    from volumetricrestirrelease_gb300 import scenes
    d = scenes.full().volume
    d.res, d.voxel_size, d.num_mips = 128, 2.0 / 128, 1
    vol = Volume.procedural(d, lib=vlib)
    frac = vol.info().num_bricks[0] / 16 ** 3
    assert 0.05 < frac < 0.3
