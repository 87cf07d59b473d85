"""Builds libvrestir.so (CUDA kernels for sm_103a + the C ABI) in-tree.

Objects go to volumetricrestirrelease_gb300/_build/, the library to
volumetricrestirrelease_gb300/_lib/libvrestir.so.  The four kernel variants (one per maximum
path length) compile in parallel.  Floating-point flags: no FMA contraction (-fmad=false on the
device, -ffp-contract=off on the host), IEEE division and square root, no flush-to-zero, so the
kernels round exactly like the CPU oracle.
"""
import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess

PKG = pathlib.Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "_lib" / "libvrestir.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
                     "-ftz=false", "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math", "-Xptxas", "-v"]
HEADERS = ["vr_math.h", "vr_device.cuh", "vr_kernels.cuh", "vr_volume.h", "vr_noalloc.h", "vr_lp.h", "vr_lp_kernels.cuh", "lp_net.h",
           "vr_batch.h"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(out, srcs):
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(p.stat().st_mtime > t for p in srcs)


def _run(cmd, log):
    r = subprocess.run(cmd, capture_output=True, text=True)
    log.write_text(r.stdout + r.stderr)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stderr[-4000:]}")
    return log


def build(force=False, jobs=None):
    BUILD.mkdir(parents=True, exist_ok=True)
    LIB.parent.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    hdrs = [CSRC / h for h in HEADERS] + [ROOT / "include" / "vrestir.h"]
    units = []
    for mb in (1, 2, 3, 4):
        obj = BUILD / f"frame_kernels_mb{mb}.o"
        src = CSRC / "frame_kernels.cu"
        units.append((obj, [src] + hdrs, [nvcc] + NVCC_FLAGS + [f"-DVR_MB={mb}", "-c", str(src), "-o", str(obj)]))
    for mb in (1, 2, 3, 4):
        obj = BUILD / f"batch_mb{mb}.o"
        src = CSRC / "batch.cu"
        units.append((obj, [src, CSRC / "vr_batch.h", CSRC / "vr_batch_kernels.cuh"] + hdrs, [nvcc] + NVCC_FLAGS + [f"-DVR_MB={mb}", "-DVR_BATCHED", "-c", str(src), "-o", str(obj)]))
    obj = BUILD / "lp.o"
    src = CSRC / "lp.cu"
    units.append((obj, [src, CSRC / "umma.cuh"] + hdrs, [nvcc] + NVCC_FLAGS + ["-c", str(src), "-o", str(obj)]))
    obj = BUILD / "noalloc.o"
    src = CSRC / "noalloc.cu"
    units.append((obj, [src, CSRC / "vr_noalloc.h"] + hdrs, [nvcc] + NVCC_FLAGS + ["-c", str(src), "-o", str(obj)]))
    obj = BUILD / "post.o"
    src = CSRC / "post.cu"
    units.append((obj, [src] + hdrs, [nvcc] + NVCC_FLAGS + ["-c", str(src), "-o", str(obj)]))
    obj = BUILD / "context.o"
    src = CSRC / "context.cu"
    units.append((obj, [src] + hdrs, [nvcc] + NVCC_FLAGS + ["-c", str(src), "-o", str(obj)]))
    obj = BUILD / "volume.o"
    src = CSRC / "volume.cpp"
    units.append((obj, [src] + hdrs, ["g++", "-O2", "-std=c++17", "-fPIC", "-pthread", "-ffp-contract=off", "-fno-fast-math",
                                      "-c", str(src), "-o", str(obj)]))
    obj = BUILD / "vbx.o"
    src = CSRC / "vbx.cpp"
    units.append((obj, [src] + hdrs, ["g++", "-O2", "-std=c++17", "-fPIC", "-pthread", "-ffp-contract=off", "-fno-fast-math",
                                      "-c", str(src), "-o", str(obj)]))
    todo = [(o, c) for (o, s, c) in units if force or _stale(o, s)]
    with cf.ThreadPoolExecutor(max_workers=jobs or max(1, min(len(todo), os.cpu_count() or 4))) as ex:
        futs = [ex.submit(_run, c, o.with_suffix(".log")) for (o, c) in todo]
        for f in futs:
            f.result()
    objs = [o for (o, _, _) in units]
    if force or todo or _stale(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc] + ARCH + ["-shared", "-o", str(tmp)] + [str(o) for o in objs] + ["-lpthread"],
             BUILD / "link.log")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv))
