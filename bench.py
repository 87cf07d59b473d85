"""Benchmark of the Volumetric ReSTIR frame loop on GB300.

Workload (one "step" = one frame of the plain method): 1920x1080, 512^3 sparse fBm cloud in
8^3 bricks with a 4-level conservative pyramid, max path length 3, 32 initial candidates,
temporal reuse + 3 spatial neighbours, 16 point lights + procedural sky, camera orbiting
0.5 deg per frame.  Synthetic data (the reference's .vbx clouds are not available).

Output: one JSON line (rank 0).  `value` = frames/s with every input resident in HBM
(vr_render_frame into a device buffer, CUDA events on the launching stream); `e2e` = the same
frames through vr_render_frame_host, with the image copied back to pinned host memory inside
the timed region.  The working set (bricks of all mip slots + reservoir/history buffers) is
larger than the 129 MB L2, so no explicit flush is done between frames.

`--impl reference` times the CPU restatement of the reference shader logic (the reference
itself is D3D12/Slang-only) on all host cores over a bounded sample of the same workload.

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
WORKLOAD = "plain ReSTIR frame, 1920x1080, 512^3 sparse fBm (8^3 bricks, 4-level conservative mips), max path length 3, M=32, temporal + 3 spatial neighbours, 16 point lights + 512x256 sky, orbiting camera"


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


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


def _scene(args):
    from volumetricrestirrelease_gb300 import scenes
    return scenes.full(width=args.width, height=args.height)


def _options(lib, sc):
    from volumetricrestirrelease_gb300 import capi
    o = capi.default_options(lib)
    for k, v in sc.options.items():
        setattr(o, k, v)
    return o


def stream_bytes_per_pixel(mb, K):
    """Algorithmic SoA stream bytes per pixel of each fused kernel (reservoir a/b = 32 B, one
    extra-bounce record = 16 B, feature = 4 B, output pixel = 16 B)."""
    ex = 16 * (mb - 1)
    initial = 4 + 32 + ex + (32 + ex + 4)           # features + reservoir + suffix written; history tap + prev feature read
    spatial = K * 32 + 4 + (32 + ex) + (32 + ex) + 16   # K taps + centre feature; output + history; image
    return {"k_initial": initial, "k_spatial": spatial}


def cpu_sample(args, threads, frames=2, scale_w=4, scale_h=4):
    """Times the oracle (CPU restatement) on a crop-free reduced-resolution run of the same
    scene: frame 0 untimed, frame 1 timed (temporal + spatial), scaled by pixel count."""
    from oracle import oracle as O
    from volumetricrestirrelease_gb300 import capi
    from volumetricrestirrelease_gb300.restir import Volume
    lib = capi.load()
    W, H = args.width // scale_w, args.height // scale_h
    sc = _scene(args)
    vol = Volume.procedural(sc.volume, lib=lib)
    opts = _options(lib, sc)
    ora = O.Oracle(W, H, opts, threads=threads)
    ora.set_volume(vol, sc.medium)
    ora.set_lights(sc.lights, sc.env_rgb, sc.env_scale)
    ora.render_frame(sc.camera(0))
    O.voxel_reads()
    times = []
    for f in range(1, frames):
        t = time.perf_counter()
        ora.render_frame(sc.camera(f))
        times.append(time.perf_counter() - t)
    reads = O.voxel_reads()
    t = float(np.median(times))
    fps = 1.0 / (t * (args.width * args.height) / (W * H))
    per_px = reads.astype(np.float64) / (W * H * len(times))
    return fps, t, W, H, per_px


def run_reference(args):
    """CPU restatement of the reference shaders on all host cores.  Each step renders one frame
    of the workload at a quarter of the resolution per axis (after the previous frames built the
    temporal history), and frames/s is scaled by the pixel count."""
    ws, rank = _dist()
    if rank != 0:
        return
    from oracle import oracle as O
    from volumetricrestirrelease_gb300 import build as vbuild
    from volumetricrestirrelease_gb300 import capi
    from volumetricrestirrelease_gb300.restir import Volume
    vbuild.build()
    lib = capi.load()
    threads = os.cpu_count() or 1
    sc = _scene(args)
    W, H = args.width // 4, args.height // 4
    vol = Volume.procedural(sc.volume, lib=lib)
    ora = O.Oracle(W, H, _options(lib, sc), threads=threads)
    ora.set_volume(vol, sc.medium)
    ora.set_lights(sc.lights, sc.env_rgb, sc.env_scale)
    for f in range(max(args.warmup, 1)):
        ora.render_frame(sc.camera(f))
    times = []
    for f in range(max(args.warmup, 1), max(args.warmup, 1) + args.steps):
        t = time.perf_counter()
        ora.render_frame(sc.camera(f))
        times.append(time.perf_counter() - t)
    scale = (args.width * args.height) / (W * H)
    fps = args.steps / (sum(times) * scale)
    sample = (f"oracle (CPU restatement of the reference shaders; the reference itself is D3D12/Slang-only), "
              f"{args.steps} frames at {W}x{H} after {max(args.warmup, 1)} untimed, scaled by pixel count to "
              f"{args.width}x{args.height}")
    line = {"impl": "reference", "metric": METRIC, "value": fps, "unit": "frames/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 / fps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "width": args.width, "height": args.height},
            "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


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
    sc = _scene(args)
    t0 = time.time()
    vol = Volume.procedural(sc.volume, lib=lib)
    build_s = time.time() - t0
    opts = _options(lib, sc)
    W, H = args.width, args.height
    rd = VolumetricReSTIR(W, H, opts.as_dict(), lib=lib)
    rd.setScene(vol, sc.medium, sc.lights, sc.env_rgb, sc.env_scale)
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    out = torch.empty((H, W, 4), device="cuda", dtype=torch.float32)

    def barrier():
        if ws > 1:
            torch.distributed.barrier()

    # ---- device-resident frames ----
    for f in range(args.warmup):
        rd.execute(sc.camera(f), out.data_ptr(), stream=sptr)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    rd.kernel_time_totals(reset=True)
    launches = 0
    with ClockSampler(local) as clk:
        e0.record(stream)
        for f in range(args.warmup, args.warmup + args.steps):
            rd.execute(sc.camera(f), out.data_ptr(), stream=sptr)
            launches += rd.last_launch_count()
        e1.record(stream)
        torch.cuda.synchronize()
    barrier()
    tot, nfr = rd.kernel_time_totals(reset=True)
    kernel_ms = {"k_initial": tot[0] / max(nfr, 1), "k_spatial": tot[1] / max(nfr, 1)}
    ms = e0.elapsed_time(e1)
    if ws > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = ws * args.steps / (ms / 1000.0)

    # ---- end to end through the host entry point ----
    pinned = torch.empty((H, W, 4), dtype=torch.float32).pin_memory()
    hptr = C.cast(C.c_void_p(pinned.data_ptr()), C.POINTER(C.c_float))
    n0 = args.warmup + args.steps
    for f in range(n0, n0 + 2):
        lib.vr_render_frame_host(rd._h, C.byref(sc.camera(f)), hptr, C.c_void_p(sptr))
    barrier()
    torch.cuda.synchronize()
    t = time.perf_counter()
    for f in range(n0 + 2, n0 + 2 + args.steps):
        r = lib.vr_render_frame_host(rd._h, C.byref(sc.camera(f)), hptr, C.c_void_p(sptr))
        assert r == 0, r
    e2e_s = time.perf_counter() - t
    h2d, d2h = C.c_int64(), C.c_int64()
    lib.vr_last_transfer_bytes(rd._h, C.byref(h2d), C.byref(d2h))
    e2e = ws * args.steps / e2e_s

    if rank != 0:
        return
    # ---- roofline of the dominant kernel ----
    peak, peak_kind = _peaks()
    fps_cpu, t_cpu, cw, ch, per_px = (None, None, 0, 0, None)
    cpu = None
    if not args.no_cpu:
        threads = os.cpu_count() or 1
        fps_cpu, t_cpu, cw, ch, per_px = cpu_sample(args, threads)
        cpu = {"value": fps_cpu, "unit": "frames/s", "cores": threads, "kind": "port",
               "sample": f"oracle frame 1 (temporal+spatial) at {cw}x{ch} ({t_cpu:.2f} s), scaled by pixel count to {W}x{H}"}
    avg = kernel_ms
    dom = max(avg, key=lambda k: avg[k] or 0.0)
    roof = None
    if per_px is not None and avg[dom]:
        vox_bytes = 2 if sc.volume.fp16 else 4
        sb = stream_bytes_per_pixel(opts.mMaxBounces, opts.mSpatialSampleCount)
        vox = {"k_initial": per_px[0] + per_px[1] + per_px[2], "k_spatial": per_px[3] + per_px[4]}
        alg = (sb[dom] + vox[dom] * vox_bytes) * W * H
        achieved = alg / (avg[dom] / 1000.0) / 1e9
        traffic = _traffic_from_profile(dom)
        roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "kernel": dom, "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": alg, "voxel_reads_per_pixel": float(vox[dom]),
                "kernel_ms": avg[dom]}
    line = {"metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "width": W, "height": H, "max_path_length": opts.mMaxBounces,
                       "candidates": opts.mInitialM, "spatial_samples": opts.mSpatialSampleCount,
                       "l2": "inputs larger than L2 (bricks + reservoir buffers), no flush",
                       "parallelism": f"replicas x{ws}", "volume_build_s": round(build_s, 2),
                       "samples_per_s": value * W * H * (opts.mInitialM + opts.mSpatialSampleCount + 1),
                       "kernel_ms": avg},
            "e2e": {"value": e2e, "unit": "frames/s", "h2d_bytes_per_step": int(h2d.value), "d2h_bytes_per_step": int(d2h.value)},
            "gpu_launches": launches,
            "roofline": roof,
            "cpu_baseline": cpu,
            "clocks": clk.summary()}
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
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "gb300" else max(args.warmup, 0)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
