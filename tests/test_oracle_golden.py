"""The CPU oracle against the reference's own outputs (tests/golden, produced by
running the reference build; see tests/golden/make_golden.py)."""
import numpy as np
import pytest

import make_golden
import oracle

CASES = [c["name"] for c in make_golden.CASES]


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("name", CASES)
def test_oracle_f64_matches_reference_build(name):
    g = make_golden.load_case(name)
    imfs, info = oracle.memd(g["in_f64"], g["dirs_f64"], g["nimf"], g["max_iter"])
    for i in range(g["nimf"]):
        # the reference solves with cusparse gtsv2 and projects with cuBLAS;
        # only summation order differs, so the IMFs agree to rounding
        assert rel_l2(imfs[i], g["ref_f64"][i]) < 1e-12, (name, i)


@pytest.mark.parametrize("name", CASES)
def test_oracle_f32_close_to_reference_build(name):
    g = make_golden.load_case(name)
    imfs, _ = oracle.memd(g["in_f32"], g["dirs_f32"], g["nimf"], g["max_iter"])
    for i in range(g["nimf"]):
        assert rel_l2(imfs[i], g["ref_f32"][i]) < 5e-4, (name, i)


@pytest.mark.parametrize("name", CASES)
def test_oracle_directions_match_reference(name):
    g = make_golden.load_case(name)
    d64 = oracle.directions(g["C"], g["K"], dtype=np.float64)
    d32 = oracle.directions(g["C"], g["K"], dtype=np.float32)
    assert np.abs(d64 - g["dirs_f64"]).max() < 4e-15
    assert np.abs(d32 - g["dirs_f32"]).max() < 4e-7


def test_window_quirk_is_what_the_reference_does():
    """L = 4096: the reference's extrema launch skips samples 4081..4094; with
    the skip the oracle matches to rounding, without it it does not."""
    g = make_golden.load_case("pink_c2_l4096_k16")
    assert oracle.window_cover(4096) == 4080
    imfs, _ = oracle.memd(g["in_f64"], g["dirs_f64"], g["nimf"], g["max_iter"], ref_window=False)
    worst = max(rel_l2(imfs[i], g["ref_f64"][i]) for i in range(g["nimf"]))
    assert worst > 1e-9


def test_golden_manifest_hashes():
    import hashlib
    import json
    import os

    here = os.path.dirname(make_golden.__file__)
    man = json.load(open(os.path.join(here, "manifest.json")))
    for case in man["cases"]:
        for suffix, meta in case["files"].items():
            p = os.path.join(here, f"{case['name']}.{suffix}")
            assert hashlib.sha256(open(p, "rb").read()).hexdigest() == meta["sha256"]
