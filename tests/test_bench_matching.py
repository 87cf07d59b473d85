"""The benchmark's matched-relMSE arithmetic (host logic, no GPU): the plain form's candidate count
at the learned form's relMSE, interpolated in 1/M between the bracketing plain counts, and its
frame time interpolated in M."""
import numpy as np
import pytest


def _rel(plain_means, learned_mean, frames=12, seed=3):
    rng = np.random.default_rng(seed)
    noise = rng.normal(0, 1e-4, frames)
    rel = {}
    for M, m in plain_means.items():
        rel["plain" if M == 32 else f"plain_M{M}"] = m + noise + rng.normal(0, 1e-5, frames)
    rel["learned_M36"] = learned_mean + noise + rng.normal(0, 1e-5, frames)
    return rel


def test_equal_relmse_interpolates_count_and_time():
    import bench
    plain = {8: 0.0448, 12: 0.0432, 16: 0.0426, 24: 0.0418, 32: 0.0413}
    rel = _rel(plain, 0.0422)
    ms = {8: 160.0, 12: 200.0, 16: 240.0, 24: 320.0, 32: 400.0}
    eq = bench.equal_relmse(rel, "learned_M36", ms)
    assert eq["bracket"] == [16, 24]
    r16, r24 = rel["plain_M16"].mean(), rel["plain_M24"].mean()
    t = (r16 - rel["learned_M36"].mean()) / (r16 - r24)
    m_eq = 1.0 / (1.0 / 16 + t * (1.0 / 24 - 1.0 / 16))
    assert eq["candidates"] == pytest.approx(m_eq)
    assert 16 < eq["candidates"] < 24
    assert eq["plain_ms_per_frame"] == pytest.approx(240.0 + (m_eq - 16) * 10.0)
    assert eq["plain_frames_per_s"] == pytest.approx(1000.0 / eq["plain_ms_per_frame"])
    # the learned form lies between the two bracketing counts in the paired comparison too
    assert eq["vs_bracket"]["16"]["diff"] < 0 < eq["vs_bracket"]["24"]["diff"]


def test_equal_relmse_outside_the_sweep_is_none():
    import bench
    plain = {8: 0.0448, 12: 0.0432, 16: 0.0426, 24: 0.0418, 32: 0.0413}
    ms = {M: 10.0 * M for M in plain}
    assert bench.equal_relmse(_rel(plain, 0.0400), "learned_M36", ms) is None   # better than every plain count
    assert bench.equal_relmse(_rel(plain, 0.0500), "learned_M36", ms) is None   # worse than every plain count


def test_paired_comparison():
    import bench
    rel = {"a": np.array([1.0, 2.0, 3.0, 4.0]), "b": np.array([0.5, 1.5, 2.0, 3.5])}
    p = bench.paired(rel, "a", "b")
    d = rel["a"] - rel["b"]
    assert p["diff"] == pytest.approx(d.mean())
    assert p["se"] == pytest.approx(d.std(ddof=1) / 2.0)
    assert p["z"] == pytest.approx(d.mean() / p["se"])
