"""Regenerates tests/golden/rng_golden.json from the reference's own RNG sources.

Builds oracle/_ref/rng_golden with oracle/ref/Makefile (which compiles
Source/Externals/xoshiro/{xoshiro128starstar,splitmix64}.c in place from the reference
tree) and stores its output.  Run in a checkout that has the reference tree; the fixture
itself is committed so tests never need the reference.
"""
import json
import pathlib
import subprocess
import sys

ROOT = pathlib.Path(__file__).resolve().parents[2]


def main(ref="/root/reference"):
    subprocess.run(["make", "-C", str(ROOT / "oracle" / "ref"), f"REF={ref}"], check=True)
    out = subprocess.run([str(ROOT / "oracle" / "_ref" / "rng_golden")], check=True,
                         capture_output=True, text=True).stdout
    data = json.loads(out)
    (ROOT / "tests" / "golden" / "rng_golden.json").write_text(json.dumps(data, separators=(",", ":")))


if __name__ == "__main__":
    main(*sys.argv[1:])
