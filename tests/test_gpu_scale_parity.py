"""Full-size parity of the FP64 path against the reference build itself.

The committed fixtures (tests/golden/manifest_scale.json, made by
make_golden.py run-scale on a GB300) hold, for the FP64-patched reference
build run with its extrema dump hook, the knot count and the index-set hash of
every (IMF, sift, direction, envelope) of a full 9-slot x 10-sift
decomposition, the IMF values at 4096 seeded positions and the per-IMF norms:

  * the reference's own main() configuration on its own input fixture
    (EEGsample_32CH_30504.bin, C = 32, K = 64; memReducedEpochs_dev.cu:1473-1484),
  * the benchmark record (32 x 30,504 EEG-shaped, K = 128).

Bar (FP64 path): identical extrema index sets at all 80 sifts, IMFs within
1e-10 relative L2 (on the kept positions and in norm); against the CPU oracle
the full IMFs within 1e-10.  The mixed form keeps the FP64 path's extrema sets
at every sift on the same float32 numbers and stays within 1e-6 per IMF.
"""
import os

import numpy as np
import pytest

import make_golden
import memd_gb300 as mg
import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

NAMES = [c["name"] for c in make_golden.SCALE_CASES]
MANIFEST = os.path.join(os.path.dirname(make_golden.__file__), "manifest_scale.json")


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def run_gpu(y, dirs, nimf, max_iter, precision=mg.PREC_F64, **kw):
    C, L = y.shape
    K = dirs.shape[0]
    tdt = torch.float64 if precision == mg.PREC_F64 else torch.float32
    plan = mg.Plan(C, L, K, nimf, max_iter, precision=precision, **kw)
    plan.set_trace(True)
    dy = torch.as_tensor(np.ascontiguousarray(y), dtype=tdt).cuda()
    dd = torch.as_tensor(np.ascontiguousarray(dirs), dtype=tdt).cuda()
    out = torch.empty((nimf, C, L), dtype=tdt, device="cuda")
    st = plan.run(dy, dd, out)
    res = out.cpu().numpy().astype(np.float64)
    tr = plan.trace()[: nimf - 1, :max_iter].copy()
    plan.close()
    return res, st, tr


def _case(name):
    if not os.path.exists(MANIFEST):
        pytest.fail("tests/golden/manifest_scale.json is missing (make_golden.py run-scale / collect-scale)")
    case = make_golden.load_scale_case(name)
    y = make_golden.scale_input(case)
    if y is None:
        pytest.skip("the reference's input fixture is not in oracle/_ref (oracle/ref_recipe.py generate)")
    assert make_golden.input_sha(y) == case["input_sha256"], "input differs from the one the reference ran on"
    return case, y


def _trace_mismatches(ours, ref):
    bad = (ours["count"] != ref["count"]) | (ours["hash"] != ref["hash"])
    where = np.argwhere(bad)
    return int(bad.sum()), (tuple(int(v) for v in where[0]) if len(where) else None)


@pytest.mark.parametrize("name", NAMES)
def test_f64_extrema_sets_and_imfs_match_reference_build(name):
    case, y = _case(name)
    nimf, it = case["nimf"], case["max_iter"]
    imfs, st, tr = run_gpu(y, case["dirs"], nimf, it)
    assert st.flags == 0
    nbad, first = _trace_mismatches(tr, case["trace"])
    assert nbad == 0, f"{nbad} (IMF, sift, direction, envelope) extrema sets differ; first at {first}"
    flat = imfs.reshape(nimf, -1)[:, case["positions"]]
    for i in range(nimf):
        assert rel_l2(flat[i], case["sub"][i]) < 1e-10, i
    norms = np.linalg.norm(imfs, axis=2)
    assert np.abs(norms - case["norms"]).max() <= 1e-10 * case["norms"].max()


def test_f64_full_decomposition_matches_oracle_on_benchmark_record():
    """32 x 30,504, K = 128, all 9 slots x 10 sifts: the whole IMF array
    against the CPU oracle, and the extrema sets at every sift."""
    case, y = _case("eegsynth_c32_l30504_k128")
    nimf, it = case["nimf"], case["max_iter"]
    imfs, st, tr = run_gpu(y, case["dirs"], nimf, it)
    oimfs, info = oracle.memd(y, case["dirs"], nimf, it, trace=True)
    otr = info["trace"][: nimf - 1, :it]
    nbad, first = _trace_mismatches(tr, otr)
    assert nbad == 0, f"{nbad} extrema sets differ from the oracle; first at {first}"
    for i in range(nimf):
        assert rel_l2(imfs[i], oimfs[i]) < 1e-10, i


@pytest.mark.parametrize("name", NAMES)
def test_mixed_form_keeps_fp64_extrema_sets_at_full_size(name):
    """The mixed form (float32 input, directions and output; double-float
    arithmetic) against the FP64 path on the same float32 numbers: the FP64
    path's extrema sets at every sift, IMFs within 1e-6 (the float32 output
    rounding is ~3e-8)."""
    case, y = _case(name)
    nimf, it = case["nimf"], case["max_iter"]
    y32 = y.astype(np.float32)
    d32 = case["dirs"].astype(np.float32)
    a, sa, ta = run_gpu(y32.astype(np.float64), d32.astype(np.float64), nimf, it)
    b, sb, tb = run_gpu(y32, d32, nimf, it, precision=mg.PREC_MIXED)
    assert sa.flags == 0 and sb.flags == 0
    nbad, first = _trace_mismatches(tb, ta)
    assert nbad == 0, f"{nbad} extrema sets differ from the FP64 path; first at {first}"
    for i in range(nimf):
        assert rel_l2(b[i], a[i]) < 1e-6, i
