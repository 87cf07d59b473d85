"""Learned target (transmittance network) on the GPU against the CPU oracle.

Bars:
  * training step (tcgen05 forward and backward, FP32 accumulation in TMEM): loss and gradient
    against the oracle's restatement with the same BF16 operands, within the tolerance that the
    tensor core's accumulation order leaves (relative L2 error 2e-3); the Adam update bit-exact
    given the kernel's own gradient;
  * inference (tcgen05, hardware sine/cosine for the encoding): T within relative 5e-3 on 99.9 % of
    the queries (a BF16 rounding of a feature or an activation may land on the other side);
  * the split initial pass (generate / infer / select): training samples and the query list
    bit-exact, and -- given the GPU's T -- images, reservoirs and features bit-exact.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NP = 16705


def _params(seed, out_bias=-2.0):
    rng = np.random.default_rng(seed)
    p = np.zeros(NP, np.float32)
    for l in range(4):
        fan = 60 if l == 0 else 64
        w = rng.uniform(-1, 1, (64, 64)).astype(np.float32) * np.float32(np.sqrt(6.0 / fan))
        if l == 0:
            w[:, 60:] = 0
        base = l * (64 * 64 + 64)
        p[base:base + 4096] = w.ravel()
        p[base + 4096:base + 4160] = rng.uniform(-0.1, 0.1, 64).astype(np.float32)
    p[4 * 4160:4 * 4160 + 64] = rng.uniform(-0.1, 0.1, 64).astype(np.float32)
    p[-1] = out_bias
    return p


def _samples(seed, n, box, invalid_frac=0.1):
    rng = np.random.default_rng(seed)
    bmin, binv = box
    size = 1.0 / binv
    x = bmin + rng.uniform(0, 1, (n, 3)) * size
    w = rng.normal(size=(n, 3))
    w /= np.linalg.norm(w, axis=1, keepdims=True)
    s = np.zeros((n, 8), np.float32)
    s[:, :3] = x
    s[:, 3:6] = w
    s[:, 6] = rng.uniform(0.5, 3.0, n)
    s[:, 7] = rng.uniform(0, 1, n)
    s[rng.uniform(0, 1, n) < invalid_frac, 6] = -1.0
    return s


def _ctx(vlib, cuda, overrides=None, W=64, H=48, bc4=False):
    from oracle.oracle import Oracle
    from volumetricrestirrelease_gb300 import capi, scenes
    from volumetricrestirrelease_gb300.restir import Volume, VolumetricReSTIR
    sc = scenes.small(width=W, height=H)
    vol = Volume.procedural(sc.volume, lib=vlib)
    if bc4:
        vol.compress_bc4()
    opts = capi.default_options(vlib)
    for k, v in {**sc.options, "mUseLearnedPHat": 1, "mLearnedTrainSamples": 2048, "mLearnedBatch": 512,
                 **(overrides or {})}.items():
        setattr(opts, k, v)
    gpu = VolumetricReSTIR(W, H, opts.as_dict(), lib=vlib)
    gpu.setScene(vol, sc.medium, sc.lights, sc.env_rgb, sc.env_scale)
    ora = Oracle(W, H, opts)
    ora.set_volume(vol, sc.medium)
    ora.set_lights(sc.lights, sc.env_rgb, sc.env_scale)
    return sc, vol, opts, gpu, ora


def _same(a, b):
    return np.array_equal(np.asarray(a, np.float32).view(np.uint32), np.asarray(b, np.float32).view(np.uint32))


@pytest.mark.parametrize("loss_log", [0, 1])
def test_net_gradients_match_oracle(vlib, cuda, loss_log):
    from oracle.oracle import net_gradients
    sc, vol, opts, gpu, ora = _ctx(vlib, cuda, dict(mLearnedLoss=loss_log))
    box = gpu.net_box()
    p = _params(3)
    gpu.set_net_params(p)
    s = _samples(4, 1000, box)                       # 8 CTAs, the last one partial
    d = cuda.from_numpy(s).cuda()
    loss, g = gpu.net_gradients(d.data_ptr(), len(s))
    lo, go = net_gradients(p, box, s, loss_log, opts.mLearnedTFloor)
    assert np.isfinite(loss) and loss > 0
    assert abs(loss - lo) <= 1e-3 * lo, (loss, lo)
    for name, sl in (("hidden 0", slice(0, 4160)), ("hidden 1", slice(4160, 8320)), ("hidden 2", slice(8320, 12480)),
                     ("hidden 3", slice(12480, 16640)), ("output", slice(16640, NP))):
        err = np.linalg.norm(g[sl] - go[sl]) / max(np.linalg.norm(go[sl]), 1e-30)
        assert err < 2e-3, (name, err)
    # repeated evaluation is bit-identical (no atomics)
    loss2, g2 = gpu.net_gradients(d.data_ptr(), len(s))
    assert _same(g, g2) and loss == loss2


def test_net_adam_step_bit_exact(vlib, cuda):
    from oracle.oracle import net_gradients
    sc, vol, opts, gpu, ora = _ctx(vlib, cuda)
    box = gpu.net_box()
    p = _params(5)
    gpu.set_net_params(p)
    s = _samples(6, 512, box)
    d = cuda.from_numpy(s).cuda()
    _, g = gpu.net_gradients(d.data_ptr(), len(s))
    gpu.net_train_step(d.data_ptr(), len(s))
    p1 = gpu.net_params()
    f = np.float32
    m = f(0.1) * g
    v = f(0.001) * g * g
    c1, c2 = f(1 - 0.9), f(1 - 0.999)
    lr = f(opts.mLearnedLearningRate)
    want = p - lr * (m / c1) / (np.sqrt(v / c2) + f(1e-8))
    assert _same(p1, want.astype(np.float32))
    # the step moved the weights and lowered the loss on its batch
    loss0, _ = net_gradients(p, box, s, 0, opts.mLearnedTFloor)
    loss1, _ = net_gradients(p1, box, s, 0, opts.mLearnedTFloor)
    assert loss1 < loss0


def test_net_inference_tensor_cores(vlib, cuda):
    from oracle.oracle import net_forward
    sc, vol, opts, gpu, ora = _ctx(vlib, cuda, dict(mLearnedTFloor=1e-6))
    box = gpu.net_box()
    p = _params(7)
    gpu.set_net_params(p)
    q = _samples(8, 128 * 37 + 5, box, invalid_frac=0.0)
    d = cuda.from_numpy(q).cuda()
    out = cuda.zeros(len(q), device="cuda", dtype=cuda.float32)
    gpu.net_infer(d.data_ptr(), len(q), out.data_ptr())
    cuda.cuda.synchronize()
    t = out.cpu().numpy()
    ref = net_forward(p, box, 1e-6, q)
    assert np.all(np.isfinite(t)) and t.std() > 0.01
    rel = np.abs(t - ref) / np.maximum(ref, 1e-6)
    assert np.quantile(rel, 0.999) < 5e-3, np.quantile(rel, [0.5, 0.99, 0.999, 1.0])
    assert rel.max() < 5e-2


@pytest.mark.parametrize("bc4", [False, True], ids=["fp32", "bc4"])
def test_learned_frames_match_oracle(vlib, cuda, bc4):
    from oracle.oracle import net_forward
    from volumetricrestirrelease_gb300.restir import as_reservoirs
    sc, vol, opts, gpu, ora = _ctx(vlib, cuda, bc4=bc4)
    W, H = gpu.width, gpu.height
    out = cuda.empty((H, W, 4), device="cuda", dtype=cuda.float32)
    losses = []
    for f in range(3):
        cam = sc.camera(f)
        params, box = gpu.net_params(), gpu.net_box()     # the weights this frame infers with
        gpu.execute(cam, out.data_ptr())
        cuda.cuda.synchronize()
        img = out.cpu().numpy()
        T = gpu.export_learned(0)
        qg = gpu.export_learned(1)
        tg = gpu.export_learned(2)
        losses.append(gpu.export_learned(3))
        assert not _same(params, gpu.net_params()), "the frame's training step did not change the weights"
        ora.set_lp_T(T)
        ref = ora.render_frame(cam)
        # training samples of the frame
        to = ora.export_lp(2)
        assert _same(tg, to), f"frame {f}: training samples differ"
        # the query list (any order on the GPU) against the oracle's per-slot queries
        qo = ora.export_lp(0)
        slots = qg[:, 7].view(np.int32)
        assert len(np.unique(slots)) == len(slots)
        assert len(slots) == int((qo[:, 6] >= 0).sum()) > 0
        assert _same(qg[:, :7], qo[slots, :7]), f"frame {f}: queries differ"
        # tensor-core T of the frame against the CPU network with the same weights
        tcpu = net_forward(params, box, opts.mLearnedTFloor, qg)
        rel = np.abs(T[slots] - tcpu) / tcpu
        assert np.quantile(rel, 0.999) < 5e-3
        # given the GPU's T, the frame is bit-exact
        nbad = int((img.view(np.uint32) != ref.view(np.uint32)).any(-1).sum())
        assert nbad == 0, f"frame {f}: {nbad} pixels differ"
        for which in (0, 1):
            rg = as_reservoirs(gpu.export_reservoirs(which), opts.mMaxBounces)
            ro = ora.export_reservoirs(which)
            for k in ("runningSum", "M", "depth", "p_y", "lightUV", "lightID", "sampledPixel"):
                assert _same(rg[k], ro[k]) if rg[k].dtype.kind == "f" else np.array_equal(rg[k], ro[k]), \
                    f"frame {f} buffer {which}: {k} differs"
    assert all(np.all(np.isfinite(l)) and len(l) == 4 for l in losses)
    assert img[..., :3].mean() > 0.02


def test_learned_options_validation(vlib, cuda):
    from volumetricrestirrelease_gb300 import capi
    from volumetricrestirrelease_gb300.restir import VolumetricReSTIR
    opts = capi.default_options(vlib)
    opts.mUseLearnedPHat = 1
    opts.mEnableTemporalReuse = 0
    opts.mEnableSpatialReuse = 0
    with pytest.raises(Exception):
        VolumetricReSTIR(32, 32, opts.as_dict(), lib=vlib)


def test_trained_network_lowers_relmse(vlib, cuda):
    """What the trained network gains over the method without it: relMSE against an FP64
    path-traced reference of the learned-target form with online training, against the same form
    with a network frozen at T = 1 (zero weights: the initial RIS target without any light
    visibility), on the small scene at a static camera."""
    from volumetricrestirrelease_gb300 import capi, scenes
    from volumetricrestirrelease_gb300.restir import Volume, VolumetricReSTIR
    W, H, frames, first = 96, 96, 48, 16
    sc = scenes.small(width=W, height=H)
    vol = Volume.procedural(sc.volume, lib=vlib)

    def ctx(train):
        o = capi.default_options(vlib)
        for k, v in {**sc.options, "mUseLearnedPHat": 1, "mLearnedTrainSamples": 65536 if train else 0,
                     "mLearnedBatch": 16384}.items():
            setattr(o, k, v)
        r = VolumetricReSTIR(W, H, o.as_dict(), lib=vlib)
        r.setScene(vol, sc.medium, sc.lights, sc.env_rgb, sc.env_scale)
        if not train:
            r.set_net_params(np.zeros(NP, np.float32))
        return r

    ref_ctx = ctx(True)
    acc = cuda.zeros((H, W, 3), device="cuda", dtype=cuda.float64)
    for f0 in range(0, 512, 64):
        ref_ctx.render_reference(sc.camera(0), acc.data_ptr(), f0, 64)
    cuda.cuda.synchronize()
    ref = (acc / 512).cpu().numpy()
    out = cuda.empty((H, W, 4), device="cuda", dtype=cuda.float32)
    rel = {}
    for name, train in (("trained", True), ("without", False)):
        r = ctx(train)
        errs = []
        for f in range(frames):
            r.execute(sc.camera(0), out.data_ptr())
            if f >= first:
                cuda.cuda.synchronize()
                x = out.cpu().numpy()[..., :3].astype(np.float64)
                errs.append(np.mean((x - ref) ** 2 / (ref ** 2 + 1e-2)))
        rel[name] = float(np.mean(errs))
    assert rel["trained"] < rel["without"], rel
