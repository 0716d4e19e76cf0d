"""Known-answer and property checks of the CPU oracle itself."""
import numpy as np
import pytest

import oracle


def test_imfs_telescope_to_input():
    rng = np.random.default_rng(5)
    y = rng.standard_normal((3, 700)).cumsum(axis=1)
    d = oracle.directions(3, 12)
    imfs, info = oracle.memd(y, d, 5, 7)
    assert info["n_imfs"] == 4
    assert np.abs(imfs.sum(axis=0) - y).max() < 1e-10 * np.abs(y).max()


def test_spline_interpolates_knots_and_lines():
    pos = np.array([0, 3, 7, 8, 15, 20, 29], dtype=np.int32)
    L = 30
    val = 2.5 * pos - 1.0  # a line: the natural spline reproduces it exactly
    env = oracle.envelope(pos, val, L)
    n = np.arange(L)
    assert np.allclose(env, 2.5 * n - 1.0, rtol=0, atol=1e-12)
    val2 = np.sin(pos / 3.0)
    env2 = oracle.envelope(pos, val2, L)
    assert np.allclose(env2[pos], val2, rtol=0, atol=1e-13)


def test_directions_unit_norm_and_closed_form():
    for C, K in ((1, 4), (2, 8), (3, 16), (8, 64), (32, 128)):
        d = oracle.directions(C, K)
        assert np.abs(np.linalg.norm(d, axis=1) - 1).max() < 1e-14
    # C = 2: h0 = (k + 1.5) / K, h1 = radical inverse base 2 of k+1;
    # s = 2h - 1, theta = atan2(|s1|, s0), dir = (cos theta, sin theta)
    K = 8
    d = oracle.directions(2, K)
    for k in range(K):
        h0 = (k + 1.5) / K
        h1 = float(oracle.lib().oracle_radical_inverse(2, k + 1))
        s0, s1 = 2 * h0 - 1, 2 * h1 - 1
        th = np.arctan2(abs(s1), s0)
        assert abs(d[k, 0] - np.cos(th)) < 1e-15 and abs(d[k, 1] - np.sin(th)) < 1e-15


def test_radical_inverse_values():
    ri = oracle.lib().oracle_radical_inverse
    assert ri(2, 1) == 0.5 and ri(2, 2) == 0.25 and ri(2, 3) == 0.75
    assert abs(ri(3, 1) - 1 / 3) < 1e-7 and abs(ri(3, 4) - (1 / 3 + 1 / 9)) < 1e-7


def test_mex_prime_convention_differs_from_standalone():
    """Standalone: table {-K, 2, 3, 5, ...}; MEX: the caller's primes(2000)(1:C)
    = {2, 3, 5, ...}, so coordinate 0 becomes (k + 1.5) / -2 and dimension c
    uses the next prime."""
    C, K = 4, 16
    a = oracle.directions(C, K)
    b = oracle.directions(C, K, primes=[2, 3, 5, 7])
    assert np.abs(a - b).max() > 0.1
    assert np.abs(np.linalg.norm(b, axis=1) - 1).max() < 1e-14


def test_no_qualified_direction_gives_nan_like_reference():
    # a monotone ramp has no interior extrema: every direction has 2 knots,
    # none qualifies, and the reference's mean divides 0 by 0
    y = np.tile(np.arange(50, dtype=np.float64), (2, 1))
    d = oracle.directions(2, 4)
    imfs, _ = oracle.memd(y, d, 2, 1)
    assert np.isnan(imfs[0]).all()


def test_stop_mode_terminates_and_telescopes():
    rng = np.random.default_rng(1)
    t = np.arange(2000) / 1000.0
    y = np.stack([np.sin(2 * np.pi * 5 * t + p) + 0.5 * np.sin(2 * np.pi * 60 * t + 2 * p) + 0.05 * rng.standard_normal(2000)
                  for p in (0.1, 0.7, 1.3)])
    d = oracle.directions(3, 16)
    imfs, info = oracle.memd(y, d, 10, 50, stop_mode=True)
    assert 1 <= info["n_imfs"] <= 9
    assert all(0 <= s <= 50 for s in info["sifts"])
    assert np.abs(imfs.sum(axis=0) - y).max() < 1e-9


@pytest.mark.parametrize("L", [4, 5, 33, 242, 243, 4096, 30504])
def test_window_cover_formula(L):
    # 240 interior samples per block of 242, ceil(L / 242) blocks
    assert oracle.window_cover(L) == 240 * ((L + 241) // 242)


def _tones(freqs_amps, L=2000, fs=1000.0):
    n = np.arange(L) / fs
    return np.stack([sum(a * np.sin(2 * np.pi * f * n + ph) for f, a, ph in ch) for ch in freqs_amps])


def _rel_core(a, b, edge=200):
    core = slice(edge, a.shape[1] - edge)
    return np.linalg.norm(a[:, core] - b[:, core]) / np.linalg.norm(b[:, core])


def test_two_tone_separation():
    """Two well-separated tones (60 and 5 Hz, two channels with their own
    amplitudes and phases): the first IMF is the fast tone and the remaining
    slots add up to the slow one, away from the record's ends."""
    hi = _tones([[(60, 1.0, 0.0)], [(60, 0.7, 1.0)]])
    lo = _tones([[(5, 1.0, 0.3)], [(5, 1.3, 2.0)]])
    imfs, _ = oracle.memd(hi + lo, oracle.directions(2, 16), 3, 10)
    assert _rel_core(imfs[0], hi) < 0.03
    assert _rel_core(imfs[1] + imfs[2], lo) < 0.03


def test_single_tone_is_one_imf():
    y = _tones([[(20, 1.0, 0.0)], [(20, 0.5, 0.5)]])
    imfs, _ = oracle.memd(y, oracle.directions(2, 16), 2, 10)
    assert _rel_core(imfs[0], y) < 0.01
    assert np.abs(imfs[1][:, 200:-200]).max() < 0.02
