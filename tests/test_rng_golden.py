"""The per-pixel RNG against known-answer vectors generated from the reference's own generator
sources (Source/Externals/xoshiro/{xoshiro128starstar,splitmix64}.c; seeding as in
Source/Tools/FalcorTest/Tests/Sampling/PseudorandomTests.cpp:94-149 and
Source/Falcor/Utils/Sampling/UniformSampleGenerator.slang:49-68)."""
import ctypes as C
import json
import pathlib

import numpy as np
import pytest

GOLD = json.loads((pathlib.Path(__file__).parent / "golden" / "rng_golden.json").read_text())


def test_xoshiro128starstar_matches_reference(oracle_lib):
    seeds = np.array(GOLD["xoshiro_seed"], np.uint32).reshape(-1, 4)
    ref = np.array(GOLD["xoshiro_out"], np.uint32).reshape(len(seeds), -1)
    for i, s in enumerate(seeds):
        out = np.zeros(ref.shape[1], np.uint32)
        oracle_lib.vro_xoshiro(s.ctypes.data_as(C.c_void_p), ref.shape[1], out.ctypes.data_as(C.c_void_p))
        assert np.array_equal(out, ref[i]), f"instance {i}"


def test_splitmix64_matches_reference(oracle_lib):
    seeds = np.array(GOLD["splitmix_seed"], np.uint32).reshape(-1, 2)
    ref = np.array([int(x) for x in GOLD["splitmix_out"]], np.uint64).reshape(len(seeds), -1)
    for i, s in enumerate(seeds):
        out = np.zeros(ref.shape[1], np.uint64)
        seed = (int(s[1]) << 32) | int(s[0])
        oracle_lib.vro_splitmix(C.c_uint64(seed), ref.shape[1], out.ctypes.data_as(C.c_void_p))
        assert np.array_equal(out, ref[i]), f"instance {i}"


def test_pixel_sample_generator_matches_reference():
    from oracle import oracle
    cases = np.array(GOLD["pixel_cases"], np.uint32)
    u24 = np.array(GOLD["pixel_u24"], np.uint32).reshape(len(cases), -1)
    out = oracle.rng(cases, u24.shape[1])
    assert np.array_equal(out, u24.astype(np.float32) * np.float32(2.0 ** -24))


@pytest.mark.gpu
def test_device_rng_matches_reference(vlib, cuda):
    cases = np.ascontiguousarray(GOLD["pixel_cases"], np.uint32)
    u24 = np.array(GOLD["pixel_u24"], np.uint32).reshape(len(cases), -1)
    out = np.zeros(u24.shape, np.float32)
    r = vlib.vr_selftest_rng(cases.ctypes.data_as(C.POINTER(C.c_uint32)), len(cases), u24.shape[1],
                             out.ctypes.data_as(C.POINTER(C.c_float)))
    assert r == 0
    assert np.array_equal(out, u24.astype(np.float32) * np.float32(2.0 ** -24))
