"""Benchmark of the Volumetric ReSTIR frame loop on GB300.

Workload (one "step" = one frame): 1920x1080, 512^3 sparse fBm cloud in 8^3 bricks with a
4-level conservative pyramid, max path length 3, temporal reuse + 3 spatial neighbours, 16 point
lights + procedural sky, camera orbiting 0.5 deg per frame.  Synthetic data (the reference's .vbx
clouds are not available).

Metric: 1080p frames/s of the learned-target form (transmittance MLP in the initial RIS target,
FP16 bricks, LEARNED_M candidates) against the plain form (FP32 bricks) at matched relMSE.  The
match is made in the run: every form renders the orbiting camera path at 960x540 for 128
frames, and at every 8th frame from 32 on each image's relMSE is taken against a 512-spp FP64
reference of that frame rendered on the GPU.  The plain form runs at several candidate counts
(PLAIN_SWEEP_M and 32); the count at which its relMSE equals the learned form's is interpolated
linearly in 1/M between the two sweep counts that bracket it, and the plain form's 1080p
frame time at that count linearly in M between its timed frames at those two counts.  The
speed-up at equal relMSE is the learned form's frames/s over that plain frames/s.  Beside it:
the paired per-frame comparison of the learned form with the plain form at 32 candidates (mean
difference, standard error, z) and with the two bracketing plain counts, and a learned-form
sweep over SWEEP_M.

Output: one JSON line (rank 0).  `value` = frames/s with every input resident in HBM
(vr_render_frame into a device buffer, CUDA events on the launching stream); `e2e` = the same
frames through vr_render_frame_host_async, every image copied back to pinned host memory
inside the timed region (the copy of a frame overlaps the next frame's kernels).  The working
set (bricks of all mip slots + reservoir/history buffers) is larger than the 129 MB L2, so no
explicit flush is done between frames.

`--impl reference` times the CPU restatement of the reference shader logic (the reference
itself is D3D12/Slang-only) on all host cores: full 1920x1080 frames of the same learned form
(LEARNED_M candidates, FP16 bricks, the network trained on the host by the same 64 Adam steps
per frame), with its input grid built by the oracle's own library; the plain form is timed
beside it.  It renders as many of the requested frames as fit a time budget and reports the
frames it timed.

Multi-GPU: the frame loop does not shard across GPUs here; N ranks run N independent
replicas (weak scaling, no collective) and `value` sums their frames.
"""
import argparse
import ctypes as C
import json
import os
import pathlib
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "1080p frames/s at matched relMSE vs FP64 ref; learned-p-hat vs plain, 1 GB300"
WORKLOAD = ("learned-p-hat + FP16-brick ReSTIR frame, 1920x1080, 512^3 sparse fBm (8^3 bricks, 4-level conservative mips), "
            "max path length 3, temporal + 3 spatial neighbours, 16 point lights + 512x256 sky, orbiting camera; "
            "36 candidates; the plain form (FP32 bricks) compared at the candidate count of equal relMSE")
# the learned form's candidate count (fixed; the learned sweep below shows how its relMSE moves
# with the count), the plain form's counts for the equal-relMSE interpolation (with 32), and the
# learned form's sweep
LEARNED_M = 36
PLAIN_SWEEP_M = (8, 12, 16, 24)
SWEEP_M = (24, 36, 48)


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _bf16_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        if "bf16_tflops" in d:
            return float(d["bf16_tflops"]), "measured (burst)"
    return 1900.0, "fallback"


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self._proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "200",
                                           "-i", str(self.index)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, FileNotFoundError):
            self._proc = None
        return self

    def _read(self):
        for line in self._proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self._proc:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if len(s) > 2 and s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if len(s) > 2 and s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for i, n in enumerate(names):
                if len(s) > 5 + i and s[5 + i].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


def max_over_ranks(x, ws, device="cuda"):
    """The largest of every rank's x (the slowest replica's time); x itself when ws == 1."""
    if ws <= 1:
        return float(x)
    import torch
    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(ws, steps, ms):
    """Frames per second of the whole job: every rank renders `steps` frames of its replica in
    the slowest rank's `ms` milliseconds."""
    return ws * steps / (ms / 1000.0)


def _scene(args, fp16=False, static=False, width=None, height=None):
    from volumetricrestirrelease_gb300 import scenes
    sc = scenes.full(width=width or args.width, height=height or args.height, fp16=fp16)
    if static:
        sc.orbit_deg_per_frame = 0.0
    return sc


def _options(lib, sc, learned=False, M=None):
    from volumetricrestirrelease_gb300 import capi
    o = capi.default_options(lib)
    for k, v in sc.options.items():
        setattr(o, k, v)
    if learned:
        o.mUseLearnedPHat = 1
    if M:
        o.mInitialM = M
    return o


def stream_bytes_per_pixel(mb, K):
    """Algorithmic SoA stream bytes per pixel of the plain form's fused kernels (reservoir a/b =
    32 B, one extra-bounce record = 16 B, feature = 4 B, output pixel = 16 B)."""
    ex = 16 * (mb - 1)
    initial = 4 + 32 + ex + (32 + ex + 4)           # features + reservoir + suffix written; history tap + prev feature read
    spatial = K * 32 + 4 + (32 + ex) + (32 + ex) + 16   # K taps + centre feature; output + history; image
    return {"k_initial": initial, "k_spatial": spatial}


def generate_stream_bytes_per_pixel(M, vertices_px, queries_px):
    """The generate stage's algorithmic stream bytes per pixel: feature 4 B, random state 16 B,
    candidate record 8 B per candidate, vertex record 32 B per vertex, suffix record 16 B per
    indirect vertex, query 32 B + slot index 4 B per query."""
    return 4 + 16 + 8 * M + 32 * vertices_px + 16 * max(vertices_px - M, 0) + 36 * queries_px


NET_FLOP_PER_QUERY = 4 * 2 * 64 * 64 + 2 * 64      # four 64x64 layers and the output dot product
# the plain path's reservoir and feature stream per pixel and frame (path length 3, 4 spatial
# taps): the SoA bytes its two fused kernels read and write, by stream_bytes_per_pixel
SURVEY_STREAM_PX = sum(stream_bytes_per_pixel(3, 4).values())


def _relmse(img, ref):
    return float(np.mean((img[..., :3].astype(np.float64) - ref) ** 2 / (ref ** 2 + 1e-2)))


def quality(lib, vols, args, forms, QW=960, QH=540, frames=128, first=32, every=8, spp=512):
    """relMSE of each form against an FP64 path-traced reference at QWxQH on the orbiting camera
    path of the timed workload: every form renders frames 0..frames-1, and at frames first,
    first+every, ... each image is compared with a `spp`-sample FP64 reference of that frame.
    forms: {name: (fp16, learned, M[, volume key])} -> ({name: per-frame relMSE array}, info)."""
    import torch
    from volumetricrestirrelease_gb300.restir import VolumetricReSTIR
    sc = _scene(args, width=QW, height=QH)
    evals = list(range(first, frames, every))
    rd = VolumetricReSTIR(QW, QH, _options(lib, sc).as_dict(), lib=lib)
    rd.setScene(vols[False], sc.medium, sc.lights, sc.env_rgb, sc.env_scale)
    refs = {}
    for f in evals:
        acc = torch.zeros((QH, QW, 3), device="cuda", dtype=torch.float64)
        for f0 in range(0, spp, 128):
            rd.render_reference(sc.camera(f), acc.data_ptr(), f0, min(128, spp - f0))
        torch.cuda.synchronize()
        refs[f] = (acc / spp).cpu().numpy()
    del rd
    out = torch.empty((QH, QW, 4), device="cuda")
    res, plain_imgs, vs_fp32 = {}, {}, {}
    for name, form in forms.items():
        fp16, learned, M = form[:3]
        vkey = form[3] if len(form) > 3 else fp16
        scf = _scene(args, fp16=fp16, width=QW, height=QH)
        rd = VolumetricReSTIR(QW, QH, _options(lib, scf, learned, M).as_dict(), lib=lib)
        rd.setScene(vols[vkey], scf.medium, scf.lights, scf.env_rgb, scf.env_scale)
        errs, cross = [], []
        for f in range(frames):
            rd.execute(scf.camera(f), out.data_ptr())
            if f in refs:
                torch.cuda.synchronize()
                img = out.cpu().numpy()
                errs.append(_relmse(img, refs[f]))
                if name == "plain":
                    plain_imgs[f] = img[..., :3].astype(np.float64)
                elif name in ("plain_fp16", "plain_bc4") and f in plain_imgs:
                    cross.append(_relmse(img, plain_imgs[f]))
        if cross:
            vs_fp32[name] = float(np.mean(cross))
        res[name] = np.asarray(errs)
        del rd
    info = {"fp16_vs_fp32_relmse": vs_fp32.get("plain_fp16"), "bc4_vs_fp32_relmse": vs_fp32.get("plain_bc4"),
            "resolution": f"{QW}x{QH}", "camera": "orbiting 0.5 deg per frame (the timed path)",
            "frames": f"{len(evals)} frames ({first}, {first + every}, ..., {evals[-1]}) of {frames}",
            "reference": f"{spp} spp FP64 path tracer on the GPU, per evaluated frame",
            "relmse": "mean over pixels and RGB of (x-r)^2/(r^2+0.01)",
            "standard_error": "of the mean over the evaluated frames of the per-frame difference to the plain form"}
    return res, info


def paired(rel, a, b):
    """The paired comparison of forms a and b over the evaluated frames: mean per-frame relMSE
    difference (a - b), its standard error and z = mean / SE."""
    d = rel[a] - rel[b]
    se = float(d.std(ddof=1) / np.sqrt(len(d))) if len(d) > 1 else float("inf")
    return {"relmse": float(rel[a].mean()), "diff": float(d.mean()), "se": se, "z": float(d.mean() / se) if se > 0 else float("inf")}


def plain_key(M):
    return "plain" if M == 32 else f"plain_M{M}"


def equal_relmse(rel, learned_key, plain_ms):
    """The plain form's candidate count at the learned form's relMSE, interpolated linearly in 1/M
    between the two plain counts whose relMSE brackets it, and the plain form's 1080p frame time
    there, interpolated linearly in M between its timed frames at those counts.  plain_ms: {M:
    ms per frame}.  None when the learned relMSE lies outside the plain sweep."""
    target = float(rel[learned_key].mean())
    ms = sorted(plain_ms)
    r = {M: float(rel[plain_key(M)].mean()) for M in ms}
    for lo, hi in zip(ms, ms[1:]):
        if r[lo] >= target >= r[hi] and r[lo] > r[hi]:
            t = (r[lo] - target) / (r[lo] - r[hi])
            m_eq = 1.0 / (1.0 / lo + t * (1.0 / hi - 1.0 / lo))
            frame_ms = plain_ms[lo] + (m_eq - lo) / (hi - lo) * (plain_ms[hi] - plain_ms[lo])
            return {"candidates": m_eq, "bracket": [lo, hi], "plain_relmse": [r[lo], r[hi]], "learned_relmse": target,
                    "plain_ms_per_frame": frame_ms, "plain_frames_per_s": 1000.0 / frame_ms,
                    "vs_bracket": {str(lo): paired(rel, learned_key, plain_key(lo)), str(hi): paired(rel, learned_key, plain_key(hi))}}
    return None


def _time_frames(rd, sc, out, sptr, warmup, steps, first=0, clock_index=None, barrier=lambda: None):
    import torch
    for f in range(first, first + warmup):
        rd.execute(sc.camera(f), out.data_ptr(), stream=sptr)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    rd.kernel_time_totals(reset=True)
    launches = 0
    clk = ClockSampler(clock_index) if clock_index is not None else None
    if clk:
        clk.__enter__()
    try:
        e0.record(stream)
        for f in range(first + warmup, first + warmup + steps):
            rd.execute(sc.camera(f), out.data_ptr(), stream=sptr)
            launches += rd.last_launch_count()
        e1.record(stream)
        torch.cuda.synchronize()
    finally:
        if clk:
            clk.__exit__()
    barrier()
    tot, nfr = rd.kernel_time_totals(reset=True)
    ms = e0.elapsed_time(e1)
    return ms, [t / max(nfr, 1) for t in tot], launches, (clk.summary() if clk else None)


def _oracle_frames(args, threads, learned, M, warm, timed, budget_s=None):
    """Full-resolution frames of the workload on the oracle (the CPU restatement) on `threads`
    host cores, with the input grid built by the oracle's own library.  learned: the learned
    form (FP16 bricks), the network trained on the host after every frame by the frame's 64
    Adam steps, as the GPU form does.  Returns the wall-clock seconds of each timed frame
    (render + training), after `warm` untimed frames; with budget_s, stops once the timed frames
    have used it (at least two timed frames)."""
    from oracle import oracle as O
    sc = _scene(args, fp16=learned)
    vol = O.OracleVolume(sc.volume)
    over = dict(sc.options, mInitialM=M)
    if learned:
        over["mUseLearnedPHat"] = 1
    opts = O.default_options(**over)
    ora = O.Oracle(args.width, args.height, opts, threads=threads)
    ora.set_volume(vol, sc.medium)
    ora.set_lights(sc.lights, sc.env_rgb, sc.env_scale)
    trainer, box = None, None
    if learned:
        info = vol.info()
        box = (np.asarray(info.world_min, np.float32), np.full(3, 1.0 / (info.res * info.voxel_size), np.float32))
        trainer = O.CpuTrainer(O.net_init(opts.mLearnedSeed), box, lr=opts.mLearnedLearningRate, threads=threads)
    steps = opts.mLearnedTrainSamples // opts.mLearnedBatch

    def frame(f):
        if learned:
            ora.set_net(trainer.w, box)
        ora.render_frame(sc.camera(f))
        if learned:
            smp = ora.export_lp(2)
            for k in range(steps):
                trainer.step(smp[k * opts.mLearnedBatch:(k + 1) * opts.mLearnedBatch])
    for f in range(warm):
        frame(f)
    times = []
    t_all = time.perf_counter()
    for f in range(warm, warm + timed):
        t = time.perf_counter()
        frame(f)
        times.append(time.perf_counter() - t)
        if budget_s is not None and len(times) >= 2 and time.perf_counter() - t_all > budget_s:
            break
    return times


def roofline_counts(args, threads, M, params, box, scale=4):
    """Per-pixel voxel reads, vertex records and queries of the learned form's generate stage,
    counted by the oracle on frame 1 at a quarter of the resolution per axis."""
    from oracle import oracle as O
    W, H = args.width // scale, args.height // scale
    sc = _scene(args, fp16=True, width=W, height=H)
    vol = O.OracleVolume(sc.volume)
    ol = O.Oracle(W, H, O.default_options(**dict(sc.options, mUseLearnedPHat=1, mInitialM=M)), threads=threads)
    ol.set_volume(vol, sc.medium)
    ol.set_lights(sc.lights, sc.env_rgb, sc.env_scale)
    ol.set_net(params, box)
    ol.render_frame(sc.camera(0))
    O.voxel_reads()
    ol.render_frame(sc.camera(1))
    r = O.voxel_reads().astype(np.float64) / (W * H)
    q = ol.export_lp(0)
    return {"generate_voxel_reads_px": float(r[0] + r[1]), "select_voxel_reads_px": float(r[7] + r[2]),
            "vertices_px": float(ol.export_lp(3)[0]) / (W * H), "queries_px": float((q[:, 6] >= 0).sum()) / (W * H),
            "counted_at": f"{W}x{H}"}


def run_reference(args):
    """The CPU restatement of the reference shaders on all host cores, on the workload itself:
    full 1920x1080 frames of the learned form at LEARNED_M candidates (FP16 bricks, host-side
    training), as many of the requested frames as fit the time budget; then the plain form (FP32
    bricks, 32 candidates) on two frames beside it.  Uses the oracle's library only."""
    ws, rank = _dist()
    if rank != 0:
        return
    from oracle import build as obuild
    obuild.build()
    threads = os.cpu_count() or 1
    warm = min(max(args.warmup, 0), 1)
    t0 = time.perf_counter()
    times = _oracle_frames(args, threads, True, LEARNED_M, warm, args.steps, budget_s=args.ref_budget_s)
    fps = len(times) / sum(times)
    ptimes = _oracle_frames(args, threads, False, 32, 1, 2)
    pfps = len(ptimes) / sum(ptimes)
    sample = (f"oracle (CPU restatement of the reference shaders; the reference itself is D3D12/Slang-only) on {threads} "
              f"host threads: {len(times)} full {args.width}x{args.height} frames of the learned form (M={LEARNED_M}, FP16 "
              f"bricks, 64 host Adam steps per frame) after {warm} untimed, of {args.steps} requested within a "
              f"{args.ref_budget_s:.0f} s budget")
    line = {"impl": "reference", "metric": METRIC, "value": fps, "unit": "frames/s", "n_gpus": ws, "steps": len(times),
            "warmup": warm, "ms_per_step": 1000.0 * sum(times) / len(times), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (bf16 MLP, fp16 bricks)", "data": "synthetic",
            "plain": {"value": pfps, "unit": "frames/s", "frames": len(ptimes), "candidates": 32, "bricks": "fp32",
                      "ms_per_frame": [1000.0 * t for t in ptimes]},
            "config": _config(args, LEARNED_M, ws),
            "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": threads, "kind": "port", "sample": sample,
                             "ms_per_frame": [1000.0 * t for t in times], "requested_steps": args.steps},
            "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": time.perf_counter() - t0}
    print(json.dumps(line), flush=True)


def _config(args, M, ws=1):
    """The workload's config, the same dict in both arms."""
    return {"workload": WORKLOAD, "width": args.width, "height": args.height, "max_path_length": 3, "candidates": M,
            "spatial_samples": 4, "bricks": "fp16", "l2": "inputs larger than L2 (bricks + reservoir buffers), no flush",
            "parallelism": f"replicas x{ws}"}


def _traffic_from_profile(kernel):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, if present."""
    p = ROOT / "profiles" / f"{kernel}_full1080p.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


def run_batched(args, lib):
    """The batched form: 32 instances (8 fire plumes) in persistent launches replayed from a CUDA
    graph, launch shape from the autotuner.  Returns a summary dict."""
    import torch
    from volumetricrestirrelease_gb300 import scenes
    from volumetricrestirrelease_gb300.restir import Batch, VolumetricReSTIR
    t0 = time.time()
    descs = scenes.batch()
    rends, keep = [], []
    for sc in descs:
        vol, temp = scenes.make_volumes(sc, lib)
        o = _options(lib, sc)
        r = VolumetricReSTIR(sc.width, sc.height, o.as_dict(), lib=lib)
        r.setScene(vol, sc.medium, sc.lights, sc.env_rgb, sc.env_scale)
        if temp is not None:
            r.setEmission(temp, *sc.fire[2:])
        rends.append(r)
        keep.append((vol, temp))
    build_s = time.time() - t0
    outs = [torch.empty((sc.height, sc.width, 4), device="cuda") for sc in descs]
    ptrs = [o.data_ptr() for o in outs]
    b = Batch(rends, graph=True)
    f = 0
    b.render([sc.camera(f) for sc in descs], ptrs)
    f += 1
    trials, shape = b.autotune([sc.camera(f) for sc in descs], ptrs, max_trials=args.batch_trials)
    f += len(trials)
    b.render([sc.camera(f) for sc in descs], ptrs)          # graph capture
    f += 1
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for k in range(args.batch_steps):
        b.render([sc.camera(f + k) for sc in descs], ptrs)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.batch_steps
    px = sum(sc.width * sc.height for sc in descs)
    launches = b.last_launch_count()
    del b
    # the same instances rendered one after another, each by its own vr_render_frame (the
    # alternative to batching)
    fs = f + args.batch_steps
    ms_seq = None
    for k in (range(2) if not args.no_batch_sequential else ()):
        for r, sc, o in zip(rends, descs, ptrs):
            r.execute(sc.camera(fs + k), o)
    if not args.no_batch_sequential:
        torch.cuda.synchronize()
        e0.record()
        for k in range(2, 2 + args.batch_steps):
            for r, sc, o in zip(rends, descs, ptrs):
                r.execute(sc.camera(fs + k), o)
        e1.record()
        torch.cuda.synchronize()
        ms_seq = e0.elapsed_time(e1) / args.batch_steps
    res = {"workload": "32 instances (8 fire plumes), resolutions from {256^2, 512^2, 960x540, 1280x720, 1920x1080}, "
                       "128^3..512^3 sparse fBm, max path length 3, 16..32 candidates, temporal + spatial, FP16 bricks, "
                       "learned target (2^15 training samples per instance and frame)",
           "instances": len(descs), "pixels_per_frame": px, "ms_per_batch_frame": ms, "batch_frames_per_s": 1000.0 / ms,
           "pixels_per_s": px * 1000.0 / ms, "equivalent_1080p_frames_per_s": px * 1000.0 / ms / (1920 * 1080),
           "sequential": {"ms_per_frame": ms_seq, "pixels_per_s": px * 1000.0 / ms_seq if ms_seq else None,
                          "what": "the 32 instances rendered one after another with vr_render_frame"},
           "speedup_vs_sequential": ms_seq / ms if ms_seq else None,
           "graph": True, "launches_per_frame": launches,
           "autotune": {"chosen_tile": f"{shape[0]}x{shape[1]}", "blocks_per_sm": shape[2], "trial_ms": trials,
                        "candidates": "tiles 8x16, 16x8, 32x4 x 5, 4, 3 blocks per SM (each pass capped at the blocks it keeps resident)"},
           "volume_build_s": round(build_s, 1), "timed_frames": args.batch_steps}
    return res


def run_small_configs(args, lib):
    """The 256^2 configurations: cfg1 (plain, FP32), cfg3 (FP16 bricks, and BC4 coarse and
    conservative mips), cfg4 (learned target),
    16 frames at the static camera of the small scene; relMSE of every frame against a 4096-spp
    FP64 reference, FP16 against FP32 frame by frame, frames/s, and the oracle on all host cores
    for cfg1."""
    import torch
    from oracle import oracle as O
    from volumetricrestirrelease_gb300 import scenes
    from volumetricrestirrelease_gb300.restir import Volume, VolumetricReSTIR
    W = H = 256
    sc32, sc16 = scenes.small(width=W, height=H), scenes.small(width=W, height=H, fp16=True)
    vol32, vol16 = Volume.procedural(sc32.volume, lib=lib), Volume.procedural(sc16.volume, lib=lib)
    volbc4 = Volume.procedural(sc32.volume, lib=lib).compress_bc4()

    def ctx(sc, vol, learned=False):
        o = _options(lib, sc, learned)
        r = VolumetricReSTIR(W, H, o.as_dict(), lib=lib)
        r.setScene(vol, sc.medium, sc.lights, sc.env_rgb, sc.env_scale)
        return r, o
    r, o = ctx(sc32, vol32)
    acc = torch.zeros((H, W, 3), device="cuda", dtype=torch.float64)
    for f0 in range(0, 4096, 256):
        r.render_reference(sc32.camera(0), acc.data_ptr(), f0, 256)
    torch.cuda.synchronize()
    ref = (acc / 4096).cpu().numpy()
    del r
    out = torch.empty((H, W, 4), device="cuda")
    res, imgs32 = {}, {}
    for name, sc, vol, learned in (("cfg1_plain_fp32", sc32, vol32, False), ("cfg3_plain_fp16", sc16, vol16, False),
                                   ("cfg3_plain_bc4", sc32, volbc4, False), ("cfg4_learned_fp32", sc32, vol32, True)):
        r, o = ctx(sc, vol, learned)
        errs, cross = [], []
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for f in range(16):
            r.execute(sc.camera(f), out.data_ptr())
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / 16
        r2, _ = ctx(sc, vol, learned)                  # the same 16 frames again, read back one by one
        for f in range(16):
            r2.execute(sc.camera(f), out.data_ptr())
            torch.cuda.synchronize()
            img = out.cpu().numpy()
            errs.append(_relmse(img, ref))
            if name == "cfg1_plain_fp32":
                imgs32[f] = img[..., :3].astype(np.float64)
            elif name in ("cfg3_plain_fp16", "cfg3_plain_bc4"):
                cross.append(_relmse(img, imgs32[f]))
        res[name] = {"frames_per_s": 1000.0 / ms, "relmse_frames_8_15": float(np.mean(errs[8:])),
                     "relmse_range": [float(np.min(errs)), float(np.max(errs))]}
        if cross:
            res[name]["relmse_vs_fp32_range"] = [float(np.min(cross)), float(np.max(cross))]
        del r, r2
    # the oracle on the host cores, cfg1, all 16 frames
    threads = os.cpu_count() or 1
    ora = O.Oracle(W, H, _options(lib, sc32), threads=threads)
    ora.set_volume(vol32, sc32.medium)
    ora.set_lights(sc32.lights, sc32.env_rgb, sc32.env_scale)
    t = time.perf_counter()
    for f in range(16):
        ora.render_frame(sc32.camera(f))
    res["cfg1_cpu_oracle"] = {"frames_per_s": 16 / (time.perf_counter() - t), "cores": threads}
    res["reference"] = "4096 spp FP64 path tracer on the GPU, static camera"
    return res


def run_animated(args, lib):
    """Animated volume: a 128^3 cloud drifting 1.5 voxels per frame over 16 frames (no wrap of the
    sequence inside the measured frames), 256^2, plain FP32, temporal + spatial, static camera.
    frames/s against the same scene held static (each after 3 untimed frames), and relMSE
    (frames 8..15) of the temporal pass with the previous-frame grids and velocity reprojection,
    with velocity only, and with neither, each frame against a 1024-spp FP64 reference of that
    frame's volume."""
    import torch
    from volumetricrestirrelease_gb300 import scenes
    from volumetricrestirrelease_gb300.restir import Volume, VolumetricReSTIR
    W = H = 256
    NF = 16
    sc = scenes.animated(width=W, height=H, frames=NF, res=128)
    frames, temps, vels = scenes.make_animation(sc, lib)
    base = Volume.procedural(sc.volume, lib=lib)

    def ctx(over=None, anim=True, velocity=True):
        o = _options(lib, sc)
        for k, v in (over or {}).items():
            setattr(o, k, v)
        r = VolumetricReSTIR(W, H, o.as_dict(), lib=lib)
        r.setScene(base, sc.medium, sc.lights, sc.env_rgb, sc.env_scale)
        if anim:
            r.set_animation(frames, temps, vels if velocity else None, 1.0)
        return r
    out = torch.empty((H, W, 4), device="cuda")
    refs = {}
    rr = ctx()
    for f in range(NF):
        rr.execute(sc.camera(f), out.data_ptr())             # binds animation frame f
        if f >= 8:
            acc = torch.zeros((H, W, 3), device="cuda", dtype=torch.float64)
            for f0 in range(0, 1024, 256):
                rr.render_reference(sc.camera(f), acc.data_ptr(), f0, 256)
            torch.cuda.synchronize()
            refs[f] = (acc / 1024).cpu().numpy()
    del rr
    res = {"workload": "256^2, 128^3 cloud drifting 1.5 voxels per frame over 16 frames, plain FP32, temporal + 3 spatial "
                       "neighbours, static camera; relMSE frames 8..15 against a 1024-spp FP64 reference of each frame's volume"}
    for name, over, anim, velocity in (("static", {}, False, False), ("prev_grid_and_velocity", {}, True, True),
                                       ("velocity_only", dict(mUsePrevVolumeForReproj=0), True, True),
                                       ("neither", dict(mUsePrevVolumeForReproj=0), True, False)):
        r = ctx(over, anim, velocity)
        for f in range(3):
            r.execute(sc.camera(f), out.data_ptr())
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for f in range(3, NF):
            r.execute(sc.camera(f), out.data_ptr())
        e1.record()
        torch.cuda.synchronize()
        fps = (NF - 3) * 1000.0 / e0.elapsed_time(e1)
        if name == "static":
            res["static_frames_per_s"] = fps
            continue
        r2 = ctx(over, anim, velocity)
        errs = []
        for f in range(NF):
            r2.execute(sc.camera(f), out.data_ptr())
            if f >= 8:
                torch.cuda.synchronize()
                errs.append(_relmse(out.cpu().numpy(), refs[f]))
        res[name] = {"frames_per_s": fps, "relmse_frames_8_15": float(np.mean(errs))}
        del r, r2
    return res


def run_gpu(args):
    import torch
    ws, rank = _dist()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    from volumetricrestirrelease_gb300 import build as vbuild
    from volumetricrestirrelease_gb300 import capi
    from volumetricrestirrelease_gb300.restir import Volume, VolumetricReSTIR
    vbuild.build()
    lib = capi.load()
    W, H = args.width, args.height
    t0 = time.time()
    vols = {False: Volume.procedural(_scene(args).volume, lib=lib), True: Volume.procedural(_scene(args, fp16=True).volume, lib=lib)}
    if args.only_batched:
        # the batched form alone (profiling runs)
        print(json.dumps({"batched": run_batched(args, lib)}), flush=True)
        return
    vols["bc4"] = Volume.procedural(_scene(args).volume, lib=lib).compress_bc4()
    build_s = time.time() - t0

    def barrier():
        if ws > 1:
            torch.distributed.barrier()

    # ---- relMSE matching (960x540, the orbiting camera path, per-frame FP64 references) ----
    forms = {"plain": (False, False, 32), "plain_fp16": (True, False, 32), "plain_bc4": (False, False, 32, "bc4")}
    for M in PLAIN_SWEEP_M:
        forms[plain_key(M)] = (False, False, M)
    for M in SWEEP_M:
        forms[f"learned_M{M}"] = (True, True, M)
    rel, qinfo = quality(lib, vols, args, forms) if not args.no_quality else ({}, {})
    M_sel = LEARNED_M
    lkey = f"learned_M{M_sel}"
    sweep = {str(M): paired(rel, f"learned_M{M}", "plain") for M in SWEEP_M} if rel else {}
    vs32 = sweep.get(str(M_sel))
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    out = torch.empty((H, W, 4), device="cuda", dtype=torch.float32)
    # ---- learned form, device-resident frames ----
    sc = _scene(args, fp16=True)
    opts = _options(lib, sc, True, M_sel)
    rd = VolumetricReSTIR(W, H, opts.as_dict(), lib=lib)
    rd.setScene(vols[True], sc.medium, sc.lights, sc.env_rgb, sc.env_scale)
    ms, kms, launches, clocks = _time_frames(rd, sc, out, sptr, args.warmup, args.steps, clock_index=local, barrier=barrier)
    ms = max_over_ranks(ms, ws)
    value = whole_job_rate(ws, args.steps, ms)
    stage_names = ["initial_stage", "spatial_final", "training", "generate_stage", "k_net_infer", "k_lp_select"]
    kernel_ms = dict(zip(stage_names, kms))

    # ---- learned form, end to end through the pipelined host entry point, on the same frames
    # (a fresh context, the same warm-up): each frame's image lands in one of two pinned host
    # buffers while the next frame renders; the timed region ends when the last image is in
    # host memory ----
    queries = len(rd.export_learned(1)) if rank == 0 else 0
    net_params, net_box = rd.net_params(), rd.net_box()
    del rd
    rd = VolumetricReSTIR(W, H, opts.as_dict(), lib=lib)
    rd.setScene(vols[True], sc.medium, sc.lights, sc.env_rgb, sc.env_scale)
    pinned = [torch.empty((H, W, 4), dtype=torch.float32).pin_memory() for _ in range(2)]
    hptr = [C.cast(C.c_void_p(p.data_ptr()), C.POINTER(C.c_float)) for p in pinned]
    for f in range(args.warmup):
        assert lib.vr_render_frame_host_async(rd._h, C.byref(sc.camera(f)), hptr[f % 2], C.c_void_p(sptr)) == 0
    assert lib.vr_host_frames_wait(rd._h) == 0
    barrier()
    torch.cuda.synchronize()
    t = time.perf_counter()
    for f in range(args.warmup, args.warmup + args.steps):
        r = lib.vr_render_frame_host_async(rd._h, C.byref(sc.camera(f)), hptr[f % 2], C.c_void_p(sptr))
        assert r == 0, r
    assert lib.vr_host_frames_wait(rd._h) == 0
    e2e_s = time.perf_counter() - t
    h2d, d2h = C.c_int64(), C.c_int64()
    lib.vr_last_transfer_bytes(rd._h, C.byref(h2d), C.byref(d2h))
    e2e = whole_job_rate(ws, args.steps, max_over_ranks(e2e_s * 1000.0, ws))
    del rd

    # ---- plain form (FP32 bricks, M=32), same frames ----
    scp = _scene(args)
    optp = _options(lib, scp)
    rp = VolumetricReSTIR(W, H, optp.as_dict(), lib=lib)
    rp.setScene(vols[False], scp.medium, scp.lights, scp.env_rgb, scp.env_scale)
    msp, kmsp, _, _ = _time_frames(rp, scp, out, sptr, args.warmup, args.steps, barrier=barrier)
    plain_fps = whole_job_rate(ws, args.steps, max_over_ranks(msp, ws))
    del rp
    # the plain form at the sweep's other counts, for the frame time at equal relMSE
    plain_ms = {32: max_over_ranks(msp, ws) / args.steps}
    sweep_steps = min(args.steps, 5)
    for M in (PLAIN_SWEEP_M if rel else ()):
        rq = VolumetricReSTIR(W, H, _options(lib, scp, False, M).as_dict(), lib=lib)
        rq.setScene(vols[False], scp.medium, scp.lights, scp.env_rgb, scp.env_scale)
        msq, _, _, _ = _time_frames(rq, scp, out, sptr, args.warmup, sweep_steps, barrier=barrier)
        plain_ms[M] = max_over_ranks(msq, ws) / sweep_steps
        del rq
    eq = equal_relmse(rel, lkey, plain_ms) if rel else None
    # at equal relMSE the plain form renders one replica per rank like the learned form
    plain_eq_fps = ws * eq["plain_frames_per_s"] if eq else None
    # ---- plain form on BC4 coarse and conservative mips (the reference's texture form) ----
    rb = VolumetricReSTIR(W, H, optp.as_dict(), lib=lib)
    rb.setScene(vols["bc4"], scp.medium, scp.lights, scp.env_rgb, scp.env_scale)
    bc4_steps = min(args.steps, 8)
    msb, kmsb, _, _ = _time_frames(rb, scp, out, sptr, args.warmup, bc4_steps, barrier=barrier)
    bc4_fps = whole_job_rate(ws, bc4_steps, max_over_ranks(msb, ws))
    del rb

    batched = None
    if not args.no_batched and rank == 0:
        batched = run_batched(args, lib)
    small = None
    if not args.no_small and rank == 0:
        small = run_small_configs(args, lib)
    animated = None
    if not args.no_animated and rank == 0:
        animated = run_animated(args, lib)

    if rank != 0:
        return
    # ---- CPU baseline (the same learned form, full 1080p frames) and the roofline's counts ----
    peak, peak_kind = _peaks()
    cpu, lpc = None, None
    threads = os.cpu_count() or 1
    if not args.no_cpu:
        ct = _oracle_frames(args, threads, True, M_sel, 1, 3)
        med = float(np.median(ct))
        cpu = {"value": 1.0 / med, "unit": "frames/s", "cores": threads, "kind": "port",
               "sample": (f"oracle on {threads} host threads, learned form (M={M_sel}, FP16 bricks, 64 host Adam steps per frame), "
                          f"median of 3 full {W}x{H} frames after 1 untimed"),
               "ms_per_frame": [1000.0 * t for t in ct]}
        lpc = roofline_counts(args, threads, M_sel, net_params, net_box)
    dom = max(("generate_stage", "k_net_infer", "k_lp_select", "spatial_final", "training"), key=lambda k: kernel_ms[k] or 0.0)
    roof, roof_tc = None, None
    if lpc is not None and kernel_ms["generate_stage"]:
        vox_bytes = 2
        per_px = lpc["generate_voxel_reads_px"] * vox_bytes + generate_stream_bytes_per_pixel(M_sel, lpc["vertices_px"], lpc["queries_px"])
        survey_px = lpc["generate_voxel_reads_px"] * vox_bytes + SURVEY_STREAM_PX
        alg = per_px * W * H
        achieved = alg / (kernel_ms["generate_stage"] / 1000.0) / 1e9
        achieved_s = survey_px * W * H / (kernel_ms["generate_stage"] / 1000.0) / 1e9
        roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": _traffic_from_profile("generate_stage"),
                "kernel": "the generate stage (k_lp_rounds: features and primary distance rounds; k_lp_vertex0: first vertices; per bounce a sort, the walks and the vertices)",
                "peak_source": peak_kind,
                "dominant_by_time": dom, "algorithmic_bytes_per_launch": alg, "algorithmic_bytes_per_pixel": per_px,
                "voxel_reads_per_pixel": lpc["generate_voxel_reads_px"], "vertex_records_per_pixel": lpc["vertices_px"],
                "queries_per_pixel": lpc["queries_px"], "kernel_ms": kernel_ms["generate_stage"],
                "counts_from": f"oracle, learned form, frame 1 at {lpc['counted_at']}",
                "stream_and_voxel_only": {"bytes_per_pixel": survey_px, "achieved": achieved_s, "frac": achieved_s / peak,
                                          "definition": "voxel reads x 2 B + the plain path's reservoir/feature stream bytes "
                                                        f"({SURVEY_STREAM_PX} B per pixel), without this design's own vertex, "
                                                        "query and queue records"}}
    if kernel_ms["k_net_infer"]:
        tf = queries * NET_FLOP_PER_QUERY / (kernel_ms["k_net_infer"] / 1000.0) / 1e12
        pk = _bf16_peak()
        roof_tc = {"bound": "tensor", "kernel": "k_net_infer", "achieved": tf, "peak": pk[0], "unit": "TFLOP/s",
                   "frac": tf / pk[0] if pk[0] else None, "peak_source": pk[1], "queries_per_frame": queries,
                   "flop_per_query": NET_FLOP_PER_QUERY, "kernel_ms": kernel_ms["k_net_infer"]}
    line = {"metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (bf16 MLP, fp16 bricks)", "data": "synthetic",
            "relmse_summary": {"matched": eq is not None, "learned": float(rel[lkey].mean()) if rel else None, "candidates": M_sel,
                               "plain_candidates_at_equal_relmse": eq["candidates"] if eq else None,
                               "plain_value_at_equal_relmse": plain_eq_fps,
                               "speedup_at_equal_relmse": value / plain_eq_fps if eq else None,
                               "vs_plain_m32": vs32},
            "plain_value": plain_eq_fps, "speedup_learned_vs_plain": value / plain_eq_fps if eq else None,
            "plain_m32_value": plain_fps, "speedup_vs_plain_m32": value / plain_fps,
            "config": _config(args, M_sel, ws),
            "e2e": {"value": e2e, "unit": "frames/s", "h2d_bytes_per_step": int(h2d.value), "d2h_bytes_per_step": int(d2h.value)},
            "gpu_launches": launches,
            "roofline": roof,
            "roofline_tensor": roof_tc,
            "cpu_baseline": cpu,
            "details": {"volume_build_s": round(build_s, 2), "samples_per_s": value * W * H * (M_sel + opts.mSpatialSampleCount + 1),
                        "kernel_ms": kernel_ms,
                        "training": {"samples_per_frame": opts.mLearnedTrainSamples, "batch": opts.mLearnedBatch,
                                     "lr": opts.mLearnedLearningRate}},
            "plain": {"value": plain_fps, "unit": "frames/s", "candidates": 32, "bricks": "fp32",
                      "kernel_ms": {"k_initial": kmsp[0], "k_spatial": kmsp[1]},
                      "bc4": {"value": bc4_fps, "unit": "frames/s", "frames": bc4_steps, "kernel_ms": {"k_initial": kmsb[0], "k_spatial": kmsb[1]},
                              "bricks": "mip 0 fp32; coarse and conservative mips BC4",
                              "relmse": float(rel["plain_bc4"].mean()) if rel else None}},
            "relmse": {"matched": eq is not None,
                       "criterion": ("the plain form's candidate count at the learned form's relMSE, interpolated in 1/M "
                                     "between the bracketing plain counts; its 1080p frame time interpolated in M"),
                       "equal_relmse": eq,
                       "plain": {str(M): float(rel[plain_key(M)].mean()) for M in sorted(plain_ms)} if rel else None,
                       "plain_ms_per_frame_1080p": {str(M): v for M, v in sorted(plain_ms.items())},
                       "learned_sweep_vs_plain_m32": sweep,
                       "plain_fp16": float(rel["plain_fp16"].mean()) if rel else None, **qinfo},
            "batched": batched,
            "small_configs": small,
            "animated": animated,
            "clocks": clocks}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-quality", action="store_true", help="skip the relMSE matching sweep")
    ap.add_argument("--ref-budget-s", type=float, default=150.0, help="reference arm: seconds of timed frames at most")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched 32-instance form")
    ap.add_argument("--no-small", action="store_true", help="skip the 256^2 configurations (cfg1, cfg3, cfg4)")
    ap.add_argument("--no-animated", action="store_true", help="skip the animated-volume measurement")
    ap.add_argument("--batch-steps", type=int, default=4)
    ap.add_argument("--batch-trials", type=int, default=9)
    ap.add_argument("--only-batched", action="store_true", help="run the batched form alone and print its summary")
    ap.add_argument("--no-batch-sequential", action="store_true", help="skip the batch's one-after-another comparison")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "gb300" else max(args.warmup, 0)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
