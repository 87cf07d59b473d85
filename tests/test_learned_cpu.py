"""The oracle's restatement of the learned target's network, checked on the CPU.

The forward pass against an independent float64 NumPy evaluation (BF16 rounding of weights
and activations as defined), the backward pass against PyTorch autograd on the same network with
straight-through BF16 rounding, and the learned-target initial pass for determinism.
"""
import numpy as np
import pytest

NP = 16705
LS = 64 * 64 + 64


def _params(seed):
    rng = np.random.default_rng(seed)
    p = np.zeros(NP, np.float32)
    for l in range(4):
        fan = 60 if l == 0 else 64
        w = rng.uniform(-1, 1, (64, 64)).astype(np.float32) * np.float32(np.sqrt(6.0 / fan))
        if l == 0:
            w[:, 60:] = 0
        p[l * LS:l * LS + 4096] = w.ravel()
        p[l * LS + 4096:l * LS + 4160] = rng.uniform(-0.1, 0.1, 64)
    p[4 * LS:4 * LS + 64] = rng.uniform(-0.3, 0.3, 64)
    p[-1] = -1.0
    return p


def _samples(seed, n, box):
    rng = np.random.default_rng(seed)
    bmin, binv = box
    s = np.zeros((n, 8), np.float32)
    s[:, :3] = bmin + rng.uniform(0, 1, (n, 3)) / binv
    w = rng.normal(size=(n, 3))
    s[:, 3:6] = w / np.linalg.norm(w, axis=1, keepdims=True)
    s[:, 6] = 1.0
    s[:, 7] = rng.uniform(0, 1, n)
    s[rng.uniform(0, 1, n) < 0.1, 6] = -1.0
    return s


BOX = (np.array([-0.5, -0.5, -0.5], np.float32), np.array([1.0, 1.0, 1.0], np.float32))


def _bf(x):
    """float32 -> bf16 -> float32, round to nearest even."""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def _features(s):
    x, w = s[:, :3].astype(np.float64), s[:, 3:6].astype(np.float64)
    sc = np.zeros((len(s), 5))
    sc[:, :3] = (x - BOX[0]) * BOX[1]
    sc[:, 3] = np.arccos(np.clip(w[:, 1], -1, 1)) / np.pi
    sc[:, 4] = np.arctan2(w[:, 2], w[:, 0]) / (2 * np.pi) + 0.5
    f = np.zeros((len(s), 64))
    for i in range(5):
        for k in range(6):
            f[:, 12 * i + 2 * k] = np.sin(2 ** k * np.pi * sc[:, i])
            f[:, 12 * i + 2 * k + 1] = np.cos(2 ** k * np.pi * sc[:, i])
    return f


def test_forward_matches_numpy(oracle_lib):
    from oracle.oracle import net_forward
    p = _params(1)
    s = _samples(2, 300, BOX)
    t = net_forward(p, BOX, 1e-6, s)
    h = _bf(_features(s).astype(np.float32)).astype(np.float64)
    for l in range(4):
        W = _bf(p[l * LS:l * LS + 4096].reshape(64, 64)).astype(np.float64)
        b = p[l * LS + 4096:l * LS + 4160].astype(np.float64)
        h = _bf(np.maximum(h @ W.T + b, 0).astype(np.float32)).astype(np.float64)
    o = h @ _bf(p[4 * LS:4 * LS + 64]).astype(np.float64) + p[-1]
    ref = np.clip(np.exp(o), 1e-6, 1)
    rel = np.abs(t - ref) / ref
    # float32 index-order sums against float64 (and sin/cos recurrences against direct
    # evaluation): BF16 rounding boundaries may flip for a few activations
    assert np.median(rel) < 1e-4 and np.quantile(rel, 0.99) < 1e-2


def test_backward_matches_autograd(oracle_lib):
    torch = pytest.importorskip("torch")
    from oracle.oracle import net_gradients
    p = _params(3)
    s = _samples(4, 300, BOX)
    loss, g = net_gradients(p, BOX, s)

    def st(x):      # straight-through BF16 rounding
        return x + (torch.from_numpy(_bf(x.detach().numpy())) - x).detach()

    P = torch.from_numpy(p.copy()).requires_grad_(True)
    f = torch.from_numpy(_features(s).astype(np.float32))
    h = st(f)
    for l in range(4):
        W = P[l * LS:l * LS + 4096].reshape(64, 64)
        b = P[l * LS + 4096:l * LS + 4160]
        h = st(torch.relu(h @ st(W).T + b))
    o = h @ st(P[4 * LS:4 * LS + 64]) + P[-1]
    valid = torch.from_numpy(s[:, 6] >= 0)
    d = torch.exp(o) - torch.from_numpy(s[:, 7])
    L = (d * d * valid).sum() / len(s)
    L.backward()
    gt = P.grad.numpy()
    assert abs(loss - L.item()) < 1e-3 * L.item()
    err = np.linalg.norm(g - gt) / np.linalg.norm(gt)
    assert err < 2e-2, err
    # layer 0's pad columns never see a non-zero input
    pads = np.array([r * 64 + k for r in range(64) for k in range(60, 64)])
    assert np.all(g[pads] == 0)


def test_learned_oracle_frames_deterministic(oracle_lib):
    from oracle.oracle import Oracle
    from volumetricrestirrelease_gb300 import capi, scenes
    from volumetricrestirrelease_gb300.restir import Volume
    vl = capi.load()
    sc = scenes.small(width=24, height=16)
    vol = Volume.procedural(sc.volume, lib=vl)
    opts = capi.default_options(vl)
    for k, v in {**sc.options, "mUseLearnedPHat": 1, "mLearnedTrainSamples": 512}.items():
        setattr(opts, k, v)
    imgs = []
    for threads in (1, 3):
        ora = Oracle(24, 16, opts, threads=threads)
        ora.set_volume(vol, sc.medium)
        ora.set_lights(sc.lights, sc.env_rgb, sc.env_scale)
        ora.set_net(_params(5), BOX)
        for f in range(2):
            img = ora.render_frame(sc.camera(f))
        q = ora.export_lp(0)
        tr = ora.export_lp(2)
        imgs.append((img, q, tr))
    assert np.array_equal(imgs[0][0], imgs[1][0])
    assert np.array_equal(imgs[0][1], imgs[1][1]) and (imgs[0][1][:, 6] >= 0).sum() > 0
    assert np.array_equal(imgs[0][2], imgs[1][2]) and (imgs[0][2][:, 6] >= 0).mean() > 0.2
    assert np.isfinite(imgs[0][0]).all() and imgs[0][0][..., :3].mean() > 0.01
