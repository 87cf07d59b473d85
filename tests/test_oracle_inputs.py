"""The oracle's own inputs for CPU-only runs (the benchmark's CPU baseline and reference arm):
option defaults, the procedural grid built by the oracle's library, the initial network and the
host-side training step.  No GPU is needed; libvrestir.so is loaded only to compare with its
host-side builder and defaults (no device call)."""
import ctypes as C

import numpy as np


def test_option_defaults_match_library(vlib):
    from oracle import oracle as O
    from volumetricrestirrelease_gb300 import capi
    a, b = capi.default_options(vlib), O.default_options()
    assert bytes(a) == bytes(b), {k: (getattr(a, k), getattr(b, k)) for k, _ in a._fields_ if getattr(a, k) != getattr(b, k)}


def _slot_arrays(v):
    out = {}
    n_l1, n_b = v.num_l1, v.num_bricks
    for name, n in (("root_child", 32 ** 3), ("l1_vmin", 4 * n_l1), ("l1_child", 4096 * n_l1), ("brick_vmin", 4 * n_b),
                    ("brick_bounds", 4 * n_b), ("brick_f32", 1000 * n_b), ("brick_f16", 1000 * n_b)):
        p = getattr(v, name)
        out[name] = np.ctypeslib.as_array(p, shape=(n,)).copy() if p and n else None
    return out


def test_oracle_grid_builder_matches_library(vlib):
    from oracle import oracle as O
    from volumetricrestirrelease_gb300 import scenes
    from volumetricrestirrelease_gb300.restir import Volume
    dense = scenes.small().volume
    sparse = scenes.full(fp16=True).volume           # the full scene's thresholded fBm, at 128^3
    sparse.res, sparse.voxel_size = 128, 2.0 / 128
    for desc in (dense, sparse):
        a, b = Volume.procedural(desc, lib=vlib), O.OracleVolume(desc)
        ia, ib = a.info(), b.info()
        assert (ia.num_mips, ia.res, ia.voxel_size, ia.supervoxel_diag) == (ib.num_mips, ib.res, ib.voxel_size, ib.supervoxel_diag)
        for s in range(16):
            va, vb = a.slot(s), b.slot(s)
            assert va.valid == vb.valid
            if not va.valid:
                continue
            assert (va.num_l1, va.num_bricks, va.max_value) == (vb.num_l1, vb.num_bricks, vb.max_value)
            xa, xb = _slot_arrays(va), _slot_arrays(vb)
            for k in xa:
                if xa[k] is None:
                    assert xb[k] is None, k
                else:
                    assert np.array_equal(xa[k].view(np.uint8), xb[k].view(np.uint8)), f"slot {s}: {k} differs"


def test_host_training_step_lowers_the_loss():
    from oracle import oracle as O
    rng = np.random.default_rng(5)
    box = (np.array([-1, -1, -1], np.float32), np.array([0.5, 0.5, 0.5], np.float32))
    n = 4096
    s = np.zeros((n, 8), np.float32)
    s[:, :3] = rng.uniform(-1, 1, (n, 3))
    d = rng.standard_normal((n, 3))
    s[:, 3:6] = d / np.linalg.norm(d, axis=1, keepdims=True)
    s[:, 6] = 1.0
    s[:, 7] = np.exp(-2.0 * (s[:, 0] + 1.0))           # a smooth transmittance field to fit
    w0 = O.net_init(1)
    assert w0.shape == (O.NET_PARAMS,) and np.all(w0[4 * 4160 + 64:] == 0) and np.abs(w0).max() <= np.sqrt(6 / 60) + 1e-6
    tr = O.CpuTrainer(w0, box, lr=1e-3, threads=4)
    losses = [tr.step(s) for _ in range(40)]
    assert losses[-1] < 0.5 * losses[0], losses[::8]
