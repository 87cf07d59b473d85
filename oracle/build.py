"""Builds the oracle (test infrastructure) into oracle/_build/liboracle.so.

g++ with FMA contraction and fast-math off, so the oracle's float operations round exactly
as written (the CUDA side is built with -fmad=false for the same reason).
"""
import os
import pathlib
import subprocess

HERE = pathlib.Path(__file__).resolve().parent
OUT = HERE / "_build" / "liboracle.so"
CSRC = HERE.parent / "volumetricrestirrelease_gb300" / "csrc"
# the oracle, and the input-grid builder (vro_volume.cpp + the builder source the GPU library also
# compiles) so that CPU-only runs need no GPU library
SRC = [HERE / "vr_oracle.cpp", HERE / "vro_volume.cpp", CSRC / "volume.cpp"]
DEPS = SRC + [CSRC / "vr_math.h", CSRC / "vr_volume.h", CSRC / "vr_bc4.h", HERE.parent / "include" / "vrestir.h"]


def build(force=False):
    if not force and OUT.exists() and all(OUT.stat().st_mtime >= p.stat().st_mtime for p in DEPS):
        return OUT
    OUT.parent.mkdir(parents=True, exist_ok=True)
    cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-pthread", "-ffp-contract=off",
           "-fno-fast-math", "-fno-unsafe-math-optimizations", "-Wall", "-Wno-unused-function", "-Wl,--no-undefined",
           "-o", str(OUT) + ".tmp"] + [str(s) for s in SRC]
    subprocess.run(cmd, check=True)
    os.replace(str(OUT) + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
