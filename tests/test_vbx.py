"""GVDB .vbx volume files (gvdb-voxel-src/GVDB_FILESPEC.txt, VolumeGVDB::LoadVBX).

Bars: a volume written and read back is slot-for-slot identical (every mip, normal and
conservative: topology, brick bounds and voxels; with FP16 bricks the topology and mip 0 exactly,
the data derived from mip 0 within FP16 rounding) and renders bit-identically in the oracle; a
file assembled here byte by byte from the specification's field table (unreferenced atlas
bricks, a pre-translation, scale and translation, leaves in two level-1 nodes) loads with the
voxels at the positions its nodes give and nothing else; signed grids keep their negative
values; malformed files are refused with a message, never read out of bounds.
"""
import struct

import numpy as np
import pytest


def _dense(view):
    """Densify mip slot `view` (a vr_grid_view) to a res^3 array (z, y, x)."""
    R = view.res[0]
    out = np.zeros((R, R, R), np.float32)
    n = view.num_bricks
    if n == 0:
        return out
    vmin = np.ctypeslib.as_array(view.brick_vmin, shape=(n * 4,)).reshape(n, 4)
    if view.brick_f32:
        data = np.ctypeslib.as_array(view.brick_f32, shape=(n * 1000,)).reshape(n, 10, 10, 10)
    else:
        data = np.ctypeslib.as_array(view.brick_f16, shape=(n * 1000,)).view(np.float16).astype(np.float32).reshape(n, 10, 10, 10)
    for b in range(n):
        x, y, z = vmin[b, :3]
        out[z:z + 8, y:y + 8, x:x + 8] = data[b, 1:9, 1:9, 1:9]
    return out


def _slot_arrays(view):
    n, l1 = view.num_bricks, view.num_l1
    A = np.ctypeslib.as_array
    d = {"root": A(view.root_child, shape=(32768,)).copy(), "l1vmin": A(view.l1_vmin, shape=(l1 * 4,)).copy() if l1 else None,
         "l1child": A(view.l1_child, shape=(l1 * 4096,)).copy() if l1 else None,
         "bvmin": A(view.brick_vmin, shape=(n * 4,)).copy() if n else None,
         "bounds": A(view.brick_bounds, shape=(n * 4,)).copy() if n else None}
    if n:
        d["data"] = (A(view.brick_f32, shape=(n * 1000,)) if view.brick_f32 else A(view.brick_f16, shape=(n * 1000,))).copy()
    return d


@pytest.mark.parametrize("fp16", [False, True])
def test_round_trip_is_identical(vlib, tmp_path, fp16):
    from volumetricrestirrelease_gb300 import scenes
    from volumetricrestirrelease_gb300.restir import Volume
    sc = scenes.animated(width=16, height=16, res=64, fp16=fp16)
    v = Volume.procedural(sc.volume, lib=vlib)
    path = tmp_path / "cloud.vbx"
    v.save_vbx(path)
    w = Volume.load_vbx(path, num_mips=sc.volume.num_mips, fp16=fp16, lib=vlib)
    a, b = v.info(), w.info()
    assert (a.res, a.num_mips) == (b.res, b.num_mips)
    assert a.voxel_size == b.voxel_size and list(a.world_min) == list(b.world_min)
    for s in range(16):
        va, vb = v.slot(s), w.slot(s)
        assert va.valid == vb.valid, s
        if not va.valid:
            continue
        if fp16:
            assert abs(va.max_value - vb.max_value) <= 2e-3 * va.max_value, s
        else:
            assert va.max_value == vb.max_value, s
        da, db = _slot_arrays(va), _slot_arrays(vb)
        for k in da:
            if da[k] is None:
                assert db[k] is None, (s, k)
            elif fp16 and (k == "bounds" or (k == "data" and s > 0)):
                # derived from FP32 values in the original, from the stored FP16 mip 0 on reload
                x = da[k].view(np.float16).astype(np.float32) if k == "data" else da[k]
                y = db[k].view(np.float16).astype(np.float32) if k == "data" else db[k]
                assert np.allclose(x, y, rtol=2e-3, atol=2e-3), (s, k)
            else:
                assert np.array_equal(da[k].view(np.uint8), db[k].view(np.uint8)), (s, k)


def test_loaded_volume_renders_identically(vlib, tmp_path):
    from oracle.oracle import Oracle
    from volumetricrestirrelease_gb300 import capi, scenes
    from volumetricrestirrelease_gb300.restir import Volume
    sc = scenes.animated(width=40, height=32, res=64)
    v = Volume.procedural(sc.volume, lib=vlib)
    v.save_vbx(tmp_path / "c.vbx")
    w = Volume.load_vbx(tmp_path / "c.vbx", num_mips=sc.volume.num_mips, lib=vlib)
    opts = capi.default_options(vlib)
    for k, val in sc.options.items():
        setattr(opts, k, val)
    imgs = []
    for vol in (v, w):
        ora = Oracle(sc.width, sc.height, opts)
        ora.set_volume(vol, sc.medium)
        ora.set_lights(sc.lights, sc.env_rgb, sc.env_scale)
        imgs.append([ora.render_frame(sc.camera(f)) for f in range(2)])
    for f in range(2):
        assert np.array_equal(imgs[0][f].view(np.uint32), imgs[1][f].view(np.uint32)), f


def test_signed_grid_round_trip(vlib, tmp_path):
    from volumetricrestirrelease_gb300.restir import Volume
    rng = np.random.default_rng(3)
    g = np.zeros((32, 32, 32), np.float32)
    g[4:20, 8:30, 0:12] = rng.normal(size=(16, 22, 12)).astype(np.float32)
    v = Volume.signed(g, (-1.0, 0.5, 2.0), 0.125, lib=vlib)
    v.save_vbx(tmp_path / "vx.vbx")
    w = Volume.load_vbx(tmp_path / "vx.vbx", signed=True, lib=vlib)
    assert np.array_equal(_dense(w.slot(0)), g)
    assert list(w.info().world_min) == [-1.0, 0.5, 2.0]
    assert (_dense(w.slot(0)) < 0).any()


def test_gvdb_folder_layout(vlib, tmp_path):
    from volumetricrestirrelease_gb300 import scenes
    from volumetricrestirrelease_gb300.restir import Volume, load_gvdb_volume
    sc = scenes.fire(width=16, height=16, res=64)
    dens, temp = scenes.make_volumes(sc, vlib)
    folder = tmp_path / "plume"
    folder.mkdir()
    dens.save_vbx(folder / "plume_mip0.vbx")
    temp.save_vbx(folder / "plume_temperature.vbx")
    g = np.full((64, 64, 64), -0.25, np.float32)
    info = dens.info()
    for a in "xyz":
        Volume.signed(g, tuple(info.world_min), info.voxel_size, lib=vlib).save_vbx(folder / f"plume_velocity_{a}.vbx")
    d2, t2, v2 = load_gvdb_volume(folder, num_mips=info.num_mips, lib=vlib)
    for s in range(16):
        a, b = dens.slot(s), d2.slot(s)
        assert a.valid == b.valid and a.num_bricks == b.num_bricks, s
    assert np.array_equal(_dense(t2.slot(0)), _dense(temp.slot(0)))
    assert v2 is not None and all(np.array_equal(_dense(v.slot(0)), g) for v in v2)


# ---- a file assembled from the specification -------------------------------------------
ID_UNDEF = 0xFFFFFFFFFFFFFFFF


def _pid(lev, index):          # pool id: group bits 0-7, level bits 8-15, index bits 16-47
    return (lev << 8) | (index << 16)


def _node(lev, pos, value, parent, child):
    return struct.pack("<BBBB3i3i3fQQQ", lev, 1, 0, 0, *pos, *value, 0.0, 0.0, 0.0, parent, child, ID_UNDEF)


def _spec_file(pretrans=(0.0, 0.0, 0.0), angles=(0.0, 0.0, 0.0), scale=(0.5, 0.5, 0.5), trans=(1.0, 2.0, 3.0),
               dtype=b"f", compression=0, truncate=0):
    """Three bricks in the atlas (cells of 10^3 with a one-voxel apron along x); leaves 0 and 2
    are referenced, leaf 1 is not.  Two level-1 nodes under the root."""
    apron, cell = 1, 10
    leaves = [((8, 16, 24), 0), ((200, 0, 8), 2), ((64, 64, 64), 1)]     # (index position, atlas cell)
    axiscnt = (3, 1, 1)
    axisres = (3 * cell, cell, cell)
    atlas = np.zeros((axisres[2], axisres[1], axisres[0]), np.float32)
    pattern = {}
    for li, (pos, c) in enumerate(leaves):
        vals = (np.arange(512, dtype=np.float32).reshape(8, 8, 8) + 1.0) * (li + 1)
        atlas[apron:apron + 8, apron:apron + 8, c * cell + apron:c * cell + apron + 8] = vals
        pattern[li] = vals
    # level 1 nodes: 0 covers [0,128)^3, 1 covers [128,256) x [0,128) x [0,128)
    l1 = [((0, 0, 0), 0), ((128, 0, 0), 1)]
    hdr = struct.pack("<BB", 1, 11) + struct.pack("<12f", *pretrans, *angles, *scale, *trans)
    body = bytearray()
    body += b"density".ljust(256, b"\0")
    body += dtype + struct.pack("<BB", 1, compression) + struct.pack("<3f", 1, 1, 1)
    body += struct.pack("<i3iii", 3, 8, 8, 8, apron, 1) + struct.pack("<Q", atlas.nbytes)
    body += struct.pack("<BiB", 2, 0, 0) + struct.pack("<3i3i", *axiscnt, *axisres)
    body += struct.pack("<iQ", 3, _pid(2, 0))
    for lev, (ld, cnt0, cnt1) in enumerate([(3, 3, 0), (4, 2, 2), (5, 1, 1)]):
        rng_ = 8 * 16 ** lev if lev < 2 else 4096
        body += struct.pack("<ii3iiiii", ld, 1 << ld, rng_, rng_, rng_, cnt0, 64, cnt1, 0 if lev == 0 else (1 << 3 * ld) * 8)
    # pool 0: leaves, level-1 nodes, root
    parent_of = {0: 0, 1: 0, 2: 1}
    for li, (pos, c) in enumerate(leaves):
        body += _node(0, pos, (c * cell + apron, apron, apron), _pid(1, parent_of[li]), ID_UNDEF)
    for i, (pos, _) in enumerate(l1):
        body += _node(1, pos, (0, 0, 0), _pid(2, 0), _pid(1, i))
    body += _node(2, (0, 0, 0), (0, 0, 0), ID_UNDEF, _pid(2, 0))
    # pool 1: level-1 child lists (16^3), root child list (32^3)
    for i, (lpos, _) in enumerate(l1):
        lst = np.full(4096, ID_UNDEF, np.uint64)
        if i == 0:
            p = leaves[0][0]
            lst[((p[2] // 8) * 16 + p[1] // 8) * 16 + p[0] // 8] = _pid(0, 0)
        else:
            p = leaves[1][0]
            lst[((p[2] // 8) * 16 + p[1] // 8) * 16 + (p[0] - 128) // 8] = _pid(0, 1)
        body += lst.tobytes()
    root = np.full(32768, ID_UNDEF, np.uint64)
    root[0] = _pid(1, 0)
    root[1] = _pid(1, 1)
    body += root.tobytes()
    body += struct.pack("<ii", 3, 4) + atlas.tobytes()
    grid_off = len(hdr) + 4 + 8
    data = hdr + struct.pack("<i", 1) + struct.pack("<Q", grid_off) + bytes(body)
    return data[:len(data) - truncate] if truncate else data, leaves, pattern


def test_spec_assembled_file(vlib, tmp_path):
    from volumetricrestirrelease_gb300.restir import Volume
    data, leaves, pattern = _spec_file()
    (tmp_path / "spec.vbx").write_bytes(data)
    v = Volume.load_vbx(tmp_path / "spec.vbx", num_mips=1, lib=vlib)
    info = v.info()
    # the leaves' box: x [8, 208), y [0, 24), z [8, 32); corner aligned down to 8 -> (8, 0, 8)
    lo = (8, 0, 8)
    assert info.res == 200
    assert list(info.world_min) == [lo[0] * 0.5 + 1.0, lo[1] * 0.5 + 2.0, lo[2] * 0.5 + 3.0]
    assert info.voxel_size == 0.5
    d = _dense(v.slot(0))
    expect = np.zeros_like(d)
    # leaf 0 (position (8,16,24)) holds pattern 0; leaf 1 at (200,0,8) holds the third brick's
    # pattern (its node points at atlas cell 2); the brick in cell 1 is not referenced
    for li, (pos, cellv) in enumerate(leaves[:2]):
        x, y, z = pos[0] - lo[0], pos[1] - lo[1], pos[2] - lo[2]
        src = [k for k, (p, c) in enumerate(leaves) if c == cellv][0]
        expect[z:z + 8, y:y + 8, x:x + 8] = pattern[src]
    assert np.array_equal(d, expect)
    assert v.slot(0).num_bricks == 2


@pytest.mark.parametrize("kwargs,msg", [
    (dict(truncate=5000), "truncated"),
    (dict(compression=1), "compressed"),
    (dict(dtype=b"d"), "float"),
    (dict(angles=(0.0, 0.3, 0.0)), "rotated"),
    (dict(scale=(0.5, 0.25, 0.5)), "anisotropic"),
])
def test_malformed_files_are_refused(vlib, tmp_path, kwargs, msg):
    from volumetricrestirrelease_gb300.restir import Volume
    data, _, _ = _spec_file(**kwargs)
    (tmp_path / "bad.vbx").write_bytes(data)
    with pytest.raises(ValueError, match=msg):
        Volume.load_vbx(tmp_path / "bad.vbx", num_mips=1, lib=vlib)


def test_missing_file(vlib, tmp_path):
    from volumetricrestirrelease_gb300.restir import Volume
    with pytest.raises(ValueError, match="cannot open"):
        Volume.load_vbx(tmp_path / "none.vbx", lib=vlib)
