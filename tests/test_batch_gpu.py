"""Batched rendering (persistent launches over many instances + CUDA graph + autotuned launch
shape) against the same instances rendered one by one with vr_render_frame.

Bar: bit-identical images every frame, for a batch that mixes resolutions, candidate counts,
volumes (including an emissive fire plume and FP16 bricks) and the learned target, through the
graph's capture, its replays, and the autotuner's trial frames and shape change.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _instances(vlib):
    from volumetricrestirrelease_gb300 import capi, scenes
    specs = [
        (scenes.small(width=64, height=48), dict(mMaxBounces=3, mInitialM=8)),
        (scenes.fire(width=72, height=56, res=64), dict(mInitialM=12)),
        (scenes.small(width=80, height=40, fp16=True), dict(mMaxBounces=3, mInitialM=6, mUseLearnedPHat=1,
                                                           mLearnedTrainSamples=1024, mLearnedBatch=512)),
        (scenes.fire(width=40, height=72, res=64), dict(mInitialM=5, mUseLearnedPHat=1, mLearnedTrainSamples=512,
                                                       mLearnedBatch=256)),
    ]
    out = []
    for sc, ov in specs:
        vols = scenes.make_volumes(sc, vlib)
        opts = capi.default_options(vlib)
        for k, v in {**sc.options, **ov}.items():
            setattr(opts, k, v)
        out.append((sc, vols, opts))
    return out


def _renderer(vlib, sc, vols, opts):
    from volumetricrestirrelease_gb300.restir import VolumetricReSTIR
    r = VolumetricReSTIR(sc.width, sc.height, opts.as_dict(), lib=vlib)
    r.setScene(vols[0], sc.medium, sc.lights, sc.env_rgb, sc.env_scale)
    if vols[1] is not None:
        r.setEmission(vols[1], *sc.fire[2:])
    return r


@pytest.mark.parametrize("graph", [True, False])
def test_batch_matches_single_instances(vlib, cuda, graph):
    from volumetricrestirrelease_gb300.restir import Batch
    inst = _instances(vlib)
    batched = [_renderer(vlib, *x) for x in inst]
    single = [_renderer(vlib, *x) for x in inst]
    batch = Batch(batched, graph=graph)
    outs_b = [cuda.empty((x[0].height, x[0].width, 4), device="cuda", dtype=cuda.float32) for x in inst]
    outs_s = [cuda.empty((x[0].height, x[0].width, 4), device="cuda", dtype=cuda.float32) for x in inst]

    def check(frame_ids):
        for f in frame_ids:
            cams = [x[0].camera(f) for x in inst]
            for r, o, c in zip(single, outs_s, cams):
                r.execute(c, o.data_ptr())
        cuda.cuda.synchronize()
        for i, (a, b) in enumerate(zip(outs_b, outs_s)):
            A, B = a.cpu().numpy(), b.cpu().numpy()
            nbad = int((A.view(np.uint32) != B.view(np.uint32)).any(-1).sum())
            assert nbad == 0, f"instance {i}, frame {frame_ids[-1]}: {nbad} pixels differ"
            assert np.isfinite(A).all()

    for f in range(3):
        batch.render([x[0].camera(f) for x in inst], [o.data_ptr() for o in outs_b])
        check([f])
    assert batch.last_launch_count() > 0
    # the autotuner renders real frames (one per trial) and then switches the launch shape
    ms, shape = batch.autotune([x[0].camera(3) for x in inst], [o.data_ptr() for o in outs_b], max_trials=3)
    assert all(m > 0 for m in ms) and shape[0] * shape[1] == 128
    check([3, 3, 3])
    for f in range(4, 6):
        batch.render([x[0].camera(f) for x in inst], [o.data_ptr() for o in outs_b])
        check([f])
    for r in batched:
        assert r.frame_count == 8


def test_batch_rejects_mismatched_options(vlib, cuda):
    from volumetricrestirrelease_gb300.restir import Batch
    inst = _instances(vlib)
    r0 = _renderer(vlib, *inst[0])
    sc, vols, opts = inst[1]
    opts.mMaxBounces = 2
    r1 = _renderer(vlib, sc, vols, opts)
    with pytest.raises(RuntimeError):
        Batch([r0, r1])
