"""GPU parity of the optional end handling: not-a-knot splines and mirrored
end extrema, against the CPU oracle (FP64 path: identical extrema index sets
at every sift, IMFs within 1e-10 relative L2) and across the precision forms."""
import numpy as np
import pytest

import memd_gb300 as mg
import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

OPTS = [(mg.SPLINE_NOT_A_KNOT, mg.BOUNDARY_REFERENCE), (mg.SPLINE_NATURAL, mg.BOUNDARY_MIRROR),
        (mg.SPLINE_NOT_A_KNOT, mg.BOUNDARY_MIRROR)]


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def run_gpu(y, dirs, nimf, max_iter, precision=mg.PREC_F64, trace=False, **kw):
    C, L = y.shape
    K = dirs.shape[0]
    tdt = torch.float64 if precision == mg.PREC_F64 else torch.float32
    plan = mg.Plan(C, L, K, nimf, max_iter, precision=precision, **kw)
    if trace:
        plan.set_trace(True)
    dy = torch.as_tensor(np.ascontiguousarray(y), dtype=tdt).cuda()
    dd = torch.as_tensor(np.ascontiguousarray(dirs), dtype=tdt).cuda()
    out = torch.empty((nimf, C, L), dtype=tdt, device="cuda")
    st = plan.run(dy, dd, out)
    res = out.cpu().numpy().astype(np.float64)
    tr = plan.trace().copy() if trace else None
    plan.close()
    return res, st, tr


@pytest.mark.parametrize("spline_end,boundary", OPTS)
@pytest.mark.parametrize("C,L,K,ref_window", [(5, 4097, 17, 1), (3, 1000, 40, 1), (12, 2049, 33, 0), (4, 613, 9, 1)])
def test_f64_options_match_oracle(spline_end, boundary, C, L, K, ref_window):
    y = mg.synth_eeg(C, L, 256.0, C * 7 + L)
    d = oracle.directions(C, K)
    nimf, it = 4, 3
    kw = dict(spline_end=spline_end, boundary=boundary, ref_window=ref_window)
    imfs, st, tr = run_gpu(y, d, nimf, it, trace=True, **kw)
    oimfs, info = oracle.memd(y, d, nimf, it, trace=True, ref_window=bool(ref_window), spline_end=spline_end,
                              boundary=boundary)
    assert np.array_equal(tr["count"], info["trace"]["count"])
    assert np.array_equal(tr["hash"], info["trace"]["hash"])
    for i in range(nimf):
        assert rel_l2(imfs[i], oimfs[i]) < 1e-10, i
    assert st.flags == 0


@pytest.mark.parametrize("spline_end,boundary", OPTS)
def test_f64_options_stop_mode_match_oracle(spline_end, boundary):
    y = mg.synth_eeg(3, 3000, 256.0, 21)
    d = oracle.directions(3, 16)
    nimf, it = 6, 30
    kw = dict(spline_end=spline_end, boundary=boundary, stop_mode=mg.STOP_CRITERION)
    imfs, st, _ = run_gpu(y, d, nimf, it, **kw)
    oimfs, info = oracle.memd(y, d, nimf, it, stop_mode=True, spline_end=spline_end, boundary=boundary)
    assert st.n_imfs == info["n_imfs"]
    assert list(st.sifts[:st.n_imfs]) == list(info["sifts"][:st.n_imfs])
    for i in range(nimf):
        assert rel_l2(imfs[i], oimfs[i]) < 1e-10, i


@pytest.mark.parametrize("spline_end,boundary", OPTS)
def test_mixed_options_track_f64(spline_end, boundary):
    # not-a-knot with the reference boundary runs the impulse-accumulation
    # mean; the mirror boundary runs the direct evaluation
    # both forms see the same float32 record and directions
    y = mg.synth_eeg(16, 6000, 256.0, 33).astype(np.float32)
    d = oracle.directions(16, 48).astype(np.float32)
    nimf, it = 5, 5
    kw = dict(spline_end=spline_end, boundary=boundary)
    a, _, ta = run_gpu(y.astype(np.float64), d.astype(np.float64), nimf, it, trace=True, **kw)
    b, st, tb = run_gpu(y, d, nimf, it, precision=mg.PREC_MIXED, trace=True, **kw)
    assert np.array_equal(ta["count"], tb["count"])
    assert np.array_equal(ta["hash"], tb["hash"])
    for i in range(nimf):
        assert rel_l2(b[i], a[i]) < 1e-6, i
    assert st.flags == 0


@pytest.mark.parametrize("spline_end,boundary", OPTS)
def test_f32_options_run_and_telescope(spline_end, boundary):
    y = mg.synth_eeg(8, 4000, 256.0, 44)
    d = oracle.directions(8, 24)
    kw = dict(spline_end=spline_end, boundary=boundary)
    a, _, _ = run_gpu(y, d, 4, 4, **kw)
    b, st, _ = run_gpu(y.astype(np.float32), d.astype(np.float32), 4, 4, precision=mg.PREC_F32, **kw)
    assert np.isfinite(b).all() and st.flags == 0
    assert np.abs(b.sum(axis=0) - y).max() < 1e-4 * np.abs(y).max()
    assert rel_l2(b[0], a[0]) < 1e-2


def test_default_options_unchanged():
    # the reference configuration is the default: natural splines, forced end knots
    y = mg.synth_eeg(4, 1500, 256.0, 55)
    d = oracle.directions(4, 12)
    a, _, _ = run_gpu(y, d, 3, 3)
    b, _, _ = run_gpu(y, d, 3, 3, spline_end=mg.SPLINE_NATURAL, boundary=mg.BOUNDARY_REFERENCE)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("boundary", [mg.BOUNDARY_REFERENCE, mg.BOUNDARY_MIRROR])
def test_f64_multi_chunk_compaction_matches_oracle(boundary):
    # 140,000 samples = 4,375 bitmask words: the knot lists are written by two
    # compaction CTAs per (direction, envelope), the second finishing the slot
    y = mg.synth_eeg(2, 140000, 256.0, 66)
    d = oracle.directions(2, 6)
    nimf, it = 3, 2
    imfs, st, tr = run_gpu(y, d, nimf, it, trace=True, boundary=boundary)
    oimfs, info = oracle.memd(y, d, nimf, it, trace=True, boundary=boundary)
    assert np.array_equal(tr["count"], info["trace"]["count"])
    assert np.array_equal(tr["hash"], info["trace"]["hash"])
    for i in range(nimf):
        assert rel_l2(imfs[i], oimfs[i]) < 1e-10, i
    assert st.flags == 0
