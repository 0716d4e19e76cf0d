"""The identity behind the mixed form's mean envelope (CPU, numpy): a sum of
natural cubic splines over integer samples is rebuilt from the jumps of its
cubic coefficients at the knots and the sum's state at one anchor sample.

A cubic spline with knots x_j equals P_0(n) + sum_j (d_j - d_{j-1}) (n - x_j)_+^3
for n >= x_0 (adjacent pieces agree in value, slope and curvature).  The
fourth forward difference of (n - x)_+^3 over integers is 1, 4, 1 at
n = x-3, x-2, x-1 and 0 elsewhere, so the mean M of many splines satisfies
Delta^4 M(n) = sum of the jumps {1, 4, 1}: four prefix sums from an anchor
rebuild M.  In integers (jumps and anchor quantised to a common unit) the
sums are exact and independent of the order in which envelopes are added,
which is what makes the GPU kernel's result deterministic."""
import numpy as np
import pytest


def natural_spline_coeffs(x, y):
    """Piece coefficients (a, b, c, d) of the natural cubic spline through
    (x, y): S(n) = a_i + b_i u + c_i u^2 + d_i u^3, u = n - x_i on piece i."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    E = len(x)
    h = np.diff(x)
    A = np.zeros((E, E))
    r = np.zeros(E)
    A[0, 0] = A[-1, -1] = 1.0
    for i in range(1, E - 1):
        A[i, i - 1] = h[i - 1]
        A[i, i] = 2.0 * (h[i - 1] + h[i])
        A[i, i + 1] = h[i]
        r[i] = 3.0 * ((y[i + 1] - y[i]) / h[i] - (y[i] - y[i - 1]) / h[i - 1])
    c = np.linalg.solve(A, r)  # c = S''/2 at the knots
    d = (c[1:] - c[:-1]) / (3.0 * h)
    b = (y[1:] - y[:-1]) / h - h * (2.0 * c[:-1] + c[1:]) / 3.0
    return y[:-1], b, c[:-1], d


def eval_spline(x, coeffs, n):
    a, b, c, d = coeffs
    i = np.clip(np.searchsorted(x, n, side="right") - 1, 0, len(x) - 2)
    u = n - x[i]
    return a[i] + u * (b[i] + u * (c[i] + u * d[i]))


def random_knots(rng, L):
    gaps = rng.integers(1, 9, size=L)
    x = np.concatenate([[0], np.cumsum(gaps)])
    x = x[x < L - 1]
    return np.concatenate([x, [L - 1]]).astype(np.int64)


def test_fourth_difference_of_truncated_cube():
    x = 20
    n = np.arange(0, 40)
    f = lambda t: np.where(t > x, (t - x).astype(np.float64) ** 3, 0.0)  # noqa: E731
    d4 = f(n + 4) - 4 * f(n + 3) + 6 * f(n + 2) - 4 * f(n + 1) + f(n)
    want = np.zeros_like(d4)
    want[x - 3], want[x - 2], want[x - 1] = 1.0, 4.0, 1.0
    assert np.array_equal(d4, want)


def impulses(splines, L):
    """Delta^4 M(n) for n in [0, L - 4) from the jumps of d at interior knots."""
    d4 = np.zeros(L + 4)
    for x, coeffs in splines:
        d = coeffs[3]
        for j in range(1, len(x) - 1):
            jump = d[j] - d[j - 1]
            for off, w in ((-3, 1.0), (-2, 4.0), (-1, 1.0)):
                if 0 <= x[j] + off < L:
                    d4[x[j] + off] += w * jump
    return d4[:L]


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_sum_of_splines_rebuilt_from_jumps_and_one_anchor(seed):
    rng = np.random.default_rng(seed)
    L, n_env = 160, 24
    splines = []
    for _ in range(n_env):
        x = random_knots(rng, L)
        y = rng.standard_normal(len(x))
        splines.append((x, natural_spline_coeffs(x, y)))
    n = np.arange(L)
    direct = sum(eval_spline(x, c, n.astype(np.float64)) for x, c in splines)
    d4 = impulses(splines, L)
    # anchor: M at four consecutive samples in the middle, then the recurrence
    # M(n + 4) = 4 M(n + 3) - 6 M(n + 2) + 4 M(n + 1) - M(n) + Delta^4 M(n)
    # forward, and the same solved for M(n) backward
    na = L // 2
    M = np.full(L, np.nan)
    M[na:na + 4] = direct[na:na + 4]
    for t in range(na, L - 4):
        M[t + 4] = 4 * M[t + 3] - 6 * M[t + 2] + 4 * M[t + 1] - M[t] + d4[t]
    for t in range(na - 1, -1, -1):
        M[t] = d4[t] - M[t + 4] + 4 * M[t + 3] - 6 * M[t + 2] + 4 * M[t + 1]
    scale = np.max(np.abs(direct))
    assert np.max(np.abs(M - direct)) <= 1e-8 * scale


def test_integer_form_is_exact_and_independent_of_order():
    """Jumps and anchor state quantised to a common unit q: the integer
    recurrence gives the same integers whatever the order of the envelopes,
    and lands within the quantisation error of the direct sum."""
    rng = np.random.default_rng(7)
    L, n_env = 96, 16
    splines = []
    for _ in range(n_env):
        x = random_knots(rng, L)
        splines.append((x, natural_spline_coeffs(x, rng.standard_normal(len(x)))))
    q = 2.0 ** -40
    na = L // 2
    n = np.arange(L, dtype=np.float64)

    def integer_mean(order):
        d4 = [0] * L
        anchor = [0, 0, 0, 0]
        for e in order:
            x, c = splines[e]
            d = c[3]
            for j in range(1, len(x) - 1):
                # the jump of the quantised cubic coefficients, as the kernel adds it
                jump = int(round(d[j] / q)) - int(round(d[j - 1] / q))
                for off, w in ((-3, 1), (-2, 4), (-1, 1)):
                    if 0 <= x[j] + off < L:
                        d4[x[j] + off] += w * jump
            vals = eval_spline(x, c, n[na:na + 4])
            for k in range(4):
                anchor[k] += int(round(vals[k] / q))
        M = [None] * L
        M[na:na + 4] = anchor
        for t in range(na, L - 4):
            M[t + 4] = 4 * M[t + 3] - 6 * M[t + 2] + 4 * M[t + 1] - M[t] + d4[t]
        for t in range(na - 1, -1, -1):
            M[t] = d4[t] - M[t + 4] + 4 * M[t + 3] - 6 * M[t + 2] + 4 * M[t + 1]
        return M

    base = integer_mean(range(n_env))
    for _ in range(3):
        assert integer_mean(rng.permutation(n_env)) == base
    direct = sum(eval_spline(x, c, n) for x, c in splines)
    got = np.array(base, dtype=np.float64) * q
    # rounding of each jump (<= q/2 per envelope and knot) carried by the
    # cubic recurrence over at most L/2 samples, plus the anchor's rounding
    bound = n_env * (L // 2) ** 3 * q
    assert np.max(np.abs(got - direct)) <= bound
