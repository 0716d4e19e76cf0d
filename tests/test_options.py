"""Spline end conditions (natural / not-a-knot) and end handling (reference
clamp / mirrored extrema): the oracle's restatement pinned against scipy and
hand-worked cases, and the host-side option checks of the C ABI (no GPU)."""
import numpy as np
import pytest

import memd_gb300 as mg
import oracle


@pytest.mark.parametrize("E", [4, 5, 9, 31])
def test_not_a_knot_spline_matches_scipy(E):
    interp = pytest.importorskip("scipy.interpolate")
    rng = np.random.default_rng(E)
    for _ in range(5):
        pos = np.sort(rng.choice(np.arange(-20, 200), E, replace=False)).astype(np.int32)
        val = rng.standard_normal(E)
        L = int(pos[-1]) + 3  # past the last knot: the last piece extended, like scipy
        n = np.arange(L)
        want = interp.CubicSpline(pos.astype(float), val, bc_type="not-a-knot")(n)
        got = oracle.envelope(pos, val, L, nak=True)
        assert np.abs(got - want).max() < 1e-11 * max(1.0, np.abs(want).max())
        want_nat = interp.CubicSpline(pos.astype(float), val, bc_type="natural")(n)
        got_nat = oracle.envelope(pos, val, L, nak=False)
        assert np.abs(got_nat - want_nat).max() < 1e-11 * max(1.0, np.abs(want_nat).max())


def test_not_a_knot_reproduces_cubics_and_handles_equal_spacing():
    # a cubic is reproduced exactly by the not-a-knot spline (not by the natural one),
    # including equal spacings, where the reference's unused setup has a zero pivot
    pos = np.arange(0, 40, 5, dtype=np.int32)
    f = lambda t: 0.01 * t ** 3 - 0.3 * t ** 2 + t - 2.0
    L = 36
    got = oracle.envelope(pos, f(pos.astype(float)), L, nak=True)
    assert np.abs(got - f(np.arange(L, dtype=float))).max() < 1e-10
    nat = oracle.envelope(pos, f(pos.astype(float)), L, nak=False)
    assert np.abs(nat - f(np.arange(L, dtype=float))).max() > 1e-3


def test_mirror_known_answer():
    # P = [0, 3, 1, 4, 0, 5, 2, 1]: maxima 1, 3, 5; minima 2, 4.
    # Left: a maximum leads and P[0] = 0 is not above the first minimum (1), so
    # sample 0 acts as a minimum: maxima 3, 1 and minima 2, 0 mirror about 0.
    # Right: a maximum is last and P[7] = 1 lies above the last minimum (0):
    # maxima 3, 1 and minima 4, 2 mirror about the last maximum (5).
    P = np.array([0, 3, 1, 4, 0, 5, 2, 1], dtype=float)
    m = oracle.mirror(P, [1, 3, 5], [2, 4])
    assert m["lsym"] == 0 and m["rsym"] == 5
    assert m["left"] == [[3, 1], [2, 0]]
    assert m["right"] == [[3, 1], [4, 2]]
    # leading minimum with P[0] below the first maximum: mirror about the first minimum
    P2 = np.array([2, 1, 3, 0, 4, 1, 5, 0, 0.5], dtype=float)
    # maxima 2, 4, 6; minima 1, 3, 5, 7
    m2 = oracle.mirror(P2, [2, 4, 6], [1, 3, 5, 7])
    # about sample 1: maxima 4, 2 -> -2, 0 and minima 5, 3 -> -3, -1; the
    # outermost knots lie at or before sample 0, so no move to sample 0
    assert m2["lsym"] == 1
    assert m2["left"] == [[4, 2], [5, 3]]
    # right: the last extremum is a minimum (7) and P[8] = 0.5 lies below the
    # last maximum (5): maxima 6, 4 and minima 5, 3 mirror about 7 -> 8, 10 / 9, 11
    assert m2["rsym"] == 7
    assert m2["right"] == [[6, 4], [5, 3]]


def test_mirror_moves_symmetry_point_when_knots_stay_inside():
    # first maximum at 10, minima at 12 and 30: mirrored about 10 the minima land
    # at -10 and 8 (fine), but the maxima after the first (13, 40) land at -20, 7:
    # all reach past 0.  With maxima 10, 15, 16 the maxima land at 4, 5 > 0, so
    # the symmetry point moves to sample 0.
    L = 60
    P = np.zeros(L)
    imax, imin = [10, 15, 16], [12, 30]
    P[0] = 5.0  # above the first minimum: mirror about the first maximum
    P[12] = -1.0
    m = oracle.mirror(P, imax, imin)
    assert m["lsym"] == 0
    assert m["left"][0] == [15, 10]  # the first two maxima, mirrored about 0
    assert m["left"][1] == [30, 12]


def test_mirror_knots_cover_the_record_and_increase():
    rng = np.random.default_rng(7)
    seen = set()
    for _ in range(3000):
        L = int(rng.integers(8, 90))
        P = rng.standard_normal(L)
        n = np.arange(1, L - 1)
        imax = n[(P[n] > P[n - 1]) & (P[n] > P[n + 1])]
        imin = n[(P[n] < P[n - 1]) & (P[n] < P[n + 1])]
        if len(imax) < 2 or len(imin) < 2:
            continue
        m = oracle.mirror(P, imax, imin)
        seen.add((m["lsym"] == 0, m["rsym"] == L - 1))
        for e, ie in ((0, imax), (1, imin)):
            pos = [2 * m["lsym"] - s for s in m["left"][e]] + list(ie) + \
                  [2 * m["rsym"] - s for s in m["right"][e]]
            assert np.all(np.diff(pos) > 0)
            assert pos[0] <= 0 and pos[-1] >= L - 1
            assert 1 <= len(m["left"][e]) <= 2 and 1 <= len(m["right"][e]) <= 2
    assert len(seen) == 4  # every combination of symmetry points occurs


@pytest.mark.parametrize("spline_end,boundary", [(1, 0), (0, 1), (1, 1)])
def test_oracle_options_telescope_and_differ(spline_end, boundary):
    rng = np.random.default_rng(11)
    y = rng.standard_normal((3, 600)).cumsum(axis=1)
    d = oracle.directions(3, 12)
    a, _ = oracle.memd(y, d, 4, 5)
    b, info = oracle.memd(y, d, 4, 5, spline_end=spline_end, boundary=boundary, trace=True)
    assert np.abs(b.sum(axis=0) - y).max() < 1e-10 * np.abs(y).max()
    assert np.isfinite(b).all()
    assert np.abs(a - b).max() > 1e-6
    if boundary:
        # the trace counts the mirrored knots: qualifying directions have >= 4 per envelope
        assert (info["trace"]["count"][0, 0] >= 4).all()


def test_oracle_mirror_stop_mode_runs():
    rng = np.random.default_rng(12)
    y = rng.standard_normal((2, 800)).cumsum(axis=1)
    d = oracle.directions(2, 8)
    imfs, info = oracle.memd(y, d, 6, 20, stop_mode=True, spline_end=1, boundary=1)
    assert info["n_imfs"] >= 2
    assert np.abs(imfs.sum(axis=0) - y).max() < 1e-10 * np.abs(y).max()


@pytest.mark.parametrize("kw", [dict(spline_end=2), dict(spline_end=-1), dict(boundary=2)])
def test_plan_rejects_bad_options_on_host(kw):
    with pytest.raises(mg.MemdError) as ei:
        mg.Plan(2, 100, 4, **kw)
    assert ei.value.status == mg.MEMD_ERR_INVALID


@pytest.mark.parametrize("kw", [
    dict(max_epochs=4, boundary=mg.BOUNDARY_MIRROR),
    dict(precision=mg.PREC_MIXED, mean_eval=2, boundary=mg.BOUNDARY_MIRROR),
])
def test_unbuilt_option_combinations_are_refused(kw):
    with pytest.raises(mg.MemdError) as ei:
        mg.Plan(2, 100, 4, **kw)
    assert ei.value.status == mg.MEMD_ERR_UNSUPPORTED
