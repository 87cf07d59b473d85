"""The feature march's early exit without an exponential per step (CPU, no GPU needed).

FeatureMarch in csrc/vr_device.cuh stops when the transmittance falls below 0.01
(ReservoirFeatureRayMarching, GenerateFeatures.slang), tested as "Tr <= kFeatureCutoff" instead
of "vr::exp_(Tr) < 0.01f".  The two agree for every float if kFeatureCutoff is the largest float
whose exp_ is below 0.01f and exp_ does not decrease: checked here for every float of
[-5.3, -4.4] (where exp_(x) crosses 0.01) and on a stride through all other floats."""
import pathlib
import re
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
CSRC = ROOT / "volumetricrestirrelease_gb300" / "csrc"

CHECK = r"""
#include <cstdio>
#include <cstring>
#include <cstdint>
#include "vr_math.h"
static float u2f_(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static uint32_t f2u_(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
int main(int argc, char** argv) {
    const float c = CUTOFF;
    long bad = 0, n = 0;
    auto check = [&](float x) {
        bool a = vr::exp_(x) < 0.01f, b = x <= c;
        if (a != b) { if (bad < 5) printf("mismatch %.9g\n", x); bad++; }
        n++;
    };
    for (uint32_t u = f2u_(-4.4f); u <= f2u_(-5.3f); ++u) check(u2f_(u));       // every float of the crossing
    for (uint64_t u = 0; u < (1ull << 32); u += 4099) check(u2f_((uint32_t)u)); // a stride through all bit patterns
    check(-INFINITY); check(INFINITY); check(NAN);
    // the cutoff is the largest float below 0.01 after exp_
    bool largest = vr::exp_(c) < 0.01f && !(vr::exp_(u2f_(f2u_(c) - 1)) < 0.01f);
    printf("checked %ld mismatches %ld largest %d\n", n, bad, (int)largest);
    return bad == 0 && largest ? 0 : 1;
}
"""


def test_feature_cutoff_matches_exp(tmp_path):
    src = (CSRC / "vr_device.cuh").read_text()
    m = re.search(r"constexpr float kFeatureCutoff = (-?[0-9.]+)f;", src)
    assert m, "kFeatureCutoff not found"
    cpp = tmp_path / "check.cpp"
    cpp.write_text(CHECK.replace("CUTOFF", m.group(1) + "f"))
    exe = tmp_path / "check"
    try:
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{CSRC}", str(cpp), "-o", str(exe)],
                       check=True, capture_output=True, text=True)
    except FileNotFoundError:
        pytest.skip("no g++")
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
