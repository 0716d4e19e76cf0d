"""The contraction bounds behind the windowed factorisation and substitution
(CPU): the natural-spline pivot recurrence c_i = u / (2 (l + u) - l c_{i-1})
(l, u the knot spacings left and right of row i) keeps c in [0, 1/2) and
changes by at most 1/12 per unit change of c_{i-1}, so a truncated start
decays at least 12x per row: 16 warm-up rows leave < 6e-18 (double-float).
The forward elimination's multiplier l / g is below 2/3 and the back
substitution's c below 1/2, so both sweeps forget a truncated start."""
import numpy as np


def test_pivot_recurrence_stays_below_half_and_contracts_by_twelve():
    sp = np.arange(1, 121, dtype=np.float64)
    l, u = np.meshgrid(sp, sp, indexing="ij")
    worst = 0.0
    for c in np.linspace(0.0, 0.5, 11):
        g = 2.0 * (l + u) - l * c
        assert np.all(u / g < 0.5)
        worst = max(worst, float(np.max(u * l / g**2)))
    assert worst <= 1.0 / 12.0 + 1e-15
    # the maximum is reached at l / u = 4/3 with c = 1/2
    assert abs(4.0 * 3.0 / (2.0 * 7.0 - 4.0 * 0.5) ** 2 - 1.0 / 12.0) < 1e-15
    assert (1.0 / 12.0) ** 16 < 6e-18


def test_truncated_start_converges_on_random_spacings():
    rng = np.random.default_rng(5)
    h = rng.integers(1, 40, size=400).astype(np.float64)

    def run(c0):
        c, out, mult = c0, [], []
        for i in range(1, len(h)):
            g = 2.0 * (h[i - 1] + h[i]) - h[i - 1] * c  # row i: l = h[i-1], u = h[i]
            mult.append(h[i - 1] / g)
            c = h[i] / g
            out.append(c)
        return np.array(out), np.array(mult)

    (exact, lm), (start0, _) = run(0.0), run(0.5)
    diff = np.abs(exact - start0)
    # after 16 rows the two starts agree to the bound; thereafter to rounding
    assert diff[15] <= 0.5 * (1.0 / 12.0) ** 16 + 1e-16
    assert np.all(diff[16:] <= 1e-16)
    assert np.all(lm < 2.0 / 3.0) and np.all(exact < 0.5)
