"""Regenerates tests/golden/rng_golden.json from the reference's own RNG sources.

Builds oracle/_ref/rng_golden with oracle/ref/Makefile (which compiles
Source/Externals/xoshiro/{xoshiro128starstar,splitmix64}.c in place from the reference
tree) and stores its output.  Run where the reference tree is present, with its root as the
first argument or in VRESTIR_REFERENCE; the fixture itself is committed so tests never need
the reference.
"""
import os
import json
import pathlib
import subprocess
import sys

ROOT = pathlib.Path(__file__).resolve().parents[2]


def main(ref=None):
    ref = ref or os.environ.get("VRESTIR_REFERENCE")
    if not ref:
        sys.exit("usage: make_rng_golden.py <root of the reference tree> (or set VRESTIR_REFERENCE)")
    subprocess.run(["make", "-C", str(ROOT / "oracle" / "ref"), f"REF={ref}"], check=True)
    out = subprocess.run([str(ROOT / "oracle" / "_ref" / "rng_golden")], check=True,
                         capture_output=True, text=True).stdout
    data = json.loads(out)
    (ROOT / "tests" / "golden" / "rng_golden.json").write_text(json.dumps(data, separators=(",", ":")))


if __name__ == "__main__":
    main(*sys.argv[1:])
