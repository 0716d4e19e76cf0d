"""GPU parity: the CUDA path (through the C ABI) against the reference build's
goldens and the CPU oracle.

Bar for the FP64 path: identical extrema index sets at every sift (knot count
and set hash per direction and envelope), IMFs within 1e-10 relative L2.
"""
import numpy as np
import pytest

import make_golden
import memd_gb300 as mg
import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

CASES = [c["name"] for c in make_golden.CASES]


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def run_gpu(y, dirs, nimf, max_iter, precision=mg.PREC_F64, trace=False, x=None, **kw):
    C, L = y.shape
    K = dirs.shape[0]
    tdt = torch.float64 if precision == mg.PREC_F64 else torch.float32
    plan = mg.Plan(C, L, K, nimf, max_iter, precision=precision, **kw)
    if trace:
        plan.set_trace(True)
    dy = torch.as_tensor(np.ascontiguousarray(y), dtype=tdt).cuda()
    dd = torch.as_tensor(np.ascontiguousarray(dirs), dtype=tdt).cuda()
    out = torch.empty((nimf, C, L), dtype=tdt, device="cuda")
    st = plan.run(dy, dd, out, x=x)
    res = out.cpu().numpy()
    tr = plan.trace().copy() if trace else None
    plan.close()
    return res, st, tr


@pytest.mark.parametrize("name", CASES)
def test_f64_matches_reference_build(name):
    g = make_golden.load_case(name)
    imfs, st, tr = run_gpu(g["in_f64"], g["dirs_f64"], g["nimf"], g["max_iter"], trace=True)
    for i in range(g["nimf"]):
        assert rel_l2(imfs[i], g["ref_f64"][i]) < 1e-10, (name, i)
    # extrema index sets, sift by sift, against the oracle on the same input
    _, info = oracle.memd(g["in_f64"], g["dirs_f64"], g["nimf"], g["max_iter"], trace=True)
    otr = info["trace"]
    assert np.array_equal(tr["count"], otr["count"])
    assert np.array_equal(tr["hash"], otr["hash"])
    assert st.n_imfs == g["nimf"] - 1 and st.flags == 0


@pytest.mark.parametrize("name", CASES)
def test_f32_close_to_reference_build(name):
    g = make_golden.load_case(name)
    imfs, st, _ = run_gpu(g["in_f32"], g["dirs_f32"], g["nimf"], g["max_iter"], precision=mg.PREC_F32)
    for i in range(g["nimf"]):
        assert rel_l2(imfs[i], g["ref_f32"][i]) < 5e-4, (name, i)


@pytest.mark.parametrize("name", CASES)
def test_directions_match_reference(name):
    g = make_golden.load_case(name)
    d64 = mg.directions(g["C"], g["K"], dtype="f64").cpu().numpy()
    d32 = mg.directions(g["C"], g["K"], dtype="f32").cpu().numpy()
    assert np.abs(d64 - g["dirs_f64"]).max() < 1e-14
    assert np.abs(d32 - g["dirs_f32"]).max() < 2e-6


def test_directions_mex_convention():
    primes = [2, 3, 5, 7, 11, 13]
    d = mg.directions(6, 40, primes=primes, dtype="f64").cpu().numpy()
    o = oracle.directions(6, 40, primes=primes)
    assert np.abs(d - o).max() < 1e-14


def eeg(C, L, seed=0, fs=256.0):
    return mg.synth_eeg(C, L, fs, seed)


@pytest.mark.parametrize("C,L,K", [(5, 4097, 17), (32, 30504, 128), (3, 1000, 40), (12, 2049, 33)])
def test_f64_vs_oracle_traces_and_imfs(C, L, K):
    y = eeg(C, L, seed=C + L)
    d = oracle.directions(C, K)
    nimf, it = 3, 3
    imfs, st, tr = run_gpu(y, d, nimf, it, trace=True)
    oimfs, info = oracle.memd(y, d, nimf, it, trace=True)
    assert np.array_equal(tr["count"], info["trace"]["count"])
    assert np.array_equal(tr["hash"], info["trace"]["hash"])
    for i in range(nimf):
        assert rel_l2(imfs[i], oimfs[i]) < 1e-10, i
    assert np.abs(imfs.sum(axis=0) - y).max() < 1e-9 * np.abs(y).max()


def test_exact_solve_equals_windowed_solve():
    y = eeg(8, 6000, seed=11)
    d = oracle.directions(8, 24)
    a, _, _ = run_gpu(y, d, 3, 4, solve_window=-1)
    b, _, _ = run_gpu(y, d, 3, 4)
    for i in range(3):
        assert rel_l2(b[i], a[i]) < 1e-12


def test_direction_chunks_do_not_change_results():
    y = eeg(8, 3000, seed=12)
    d = oracle.directions(8, 40)
    a, _, _ = run_gpu(y, d, 3, 3)
    b, _, _ = run_gpu(y, d, 3, 3, dir_chunk=16)
    assert np.array_equal(a, b)


def test_relaunch_is_deterministic():
    y = eeg(4, 2500, seed=13)
    d = oracle.directions(4, 16)
    C, L = y.shape
    plan = mg.Plan(C, L, 16, 4, 5)
    dy = torch.as_tensor(y).cuda()
    dd = torch.as_tensor(d).cuda()
    o1 = torch.empty((4, C, L), dtype=torch.float64, device="cuda")
    o2 = torch.empty_like(o1)
    plan.run(dy, dd, o1)
    plan.run(dy, dd, o2)
    assert torch.equal(o1, o2)
    plan.close()


def test_no_qualified_direction_nan_and_flag():
    y = np.tile(np.arange(64, dtype=np.float64), (2, 1))
    d = oracle.directions(2, 4)
    imfs, st, _ = run_gpu(y, d, 2, 1)
    assert np.isnan(imfs[0]).all()
    assert st.flags & mg.FLAG_NO_QUALIFIED_DIRECTION


def test_coordinate_check():
    y = eeg(2, 500, seed=1)
    d = oracle.directions(2, 8)
    good = torch.arange(500, dtype=torch.int32, device="cuda")
    imfs, st, _ = run_gpu(y, d, 2, 2, x=good)
    bad = good.clone()
    bad[7] = 3
    with pytest.raises(mg.MemdError) as ei:
        run_gpu(y, d, 2, 2, x=bad)
    assert ei.value.status == mg.MEMD_ERR_COORD


def test_precision_mismatch_rejected():
    plan = mg.Plan(2, 100, 4, 2, 1, precision=mg.PREC_F32)
    y = torch.zeros((2, 100), dtype=torch.float64, device="cuda")
    d = torch.zeros((4, 2), dtype=torch.float64, device="cuda")
    o = torch.zeros((2, 2, 100), dtype=torch.float64, device="cuda")
    st = mg.Stats()
    rc = mg.lib().memd_run_f64(plan.handle, None, y.data_ptr(), d.data_ptr(), o.data_ptr(), None, None)
    assert rc == mg.MEMD_ERR_PRECISION
    plan.close()


@pytest.mark.parametrize("C,L,K,maxit", [(8, 2000, 64, 50), (3, 3000, 16, 20), (32, 4096, 24, 30)])
def test_stop_mode_matches_oracle(C, L, K, maxit):
    """Stop criterion (sd, sd2, tol) = (0.075, 0.75, 0.075): the same sift
    count for every IMF, the same number of IMFs, identical extrema sets at
    every pass, IMFs within 1e-10."""
    y = mg.synth_tones(C, L, 1000.0, seed=C) if C == 8 else eeg(C, L, seed=L)
    d = oracle.directions(C, K)
    nimf = 10
    imfs, st, tr = run_gpu(y, d, nimf, maxit, trace=True, stop_mode=mg.STOP_CRITERION)
    oimfs, info = oracle.memd(y, d, nimf, maxit, stop_mode=True, trace=True)
    assert st.n_imfs == info["n_imfs"]
    assert list(st.sifts[: st.n_imfs]) == list(info["sifts"][: info["n_imfs"]])
    assert np.array_equal(tr["count"], info["trace"]["count"])
    assert np.array_equal(tr["hash"], info["trace"]["hash"])
    for i in range(nimf):
        if np.linalg.norm(oimfs[i]) == 0:
            assert np.abs(imfs[i]).max() == 0
        else:
            assert rel_l2(imfs[i], oimfs[i]) < 1e-10, i
    assert np.abs(imfs.sum(axis=0) - y).max() < 1e-9 * np.abs(y).max()


def test_stop_mode_relaunch_and_one_slot():
    y = eeg(4, 1500, seed=2)
    d = oracle.directions(4, 8)
    a, sa, _ = run_gpu(y, d, 6, 20, stop_mode=mg.STOP_CRITERION)
    C, L = y.shape
    plan = mg.Plan(C, L, 8, 6, 20, stop_mode=mg.STOP_CRITERION)
    dy = torch.as_tensor(y).cuda()
    dd = torch.as_tensor(d).cuda()
    out = torch.empty((6, C, L), dtype=torch.float64, device="cuda")
    for _ in range(2):
        s2 = plan.run(dy, dd, out)
        assert np.array_equal(out.cpu().numpy(), a) and s2.n_imfs == sa.n_imfs
    plan.close()
    # a single output slot: no IMF, the residual is the input
    one, s1, _ = run_gpu(y, d, 1, 20, stop_mode=mg.STOP_CRITERION)
    assert np.array_equal(one[0], y) and s1.n_imfs == 0


def test_windowed_solve_bitwise_on_eeg_record():
    """The halo of the windowed tridiagonal solve (48 knots) is far beyond the
    decay of the spline system's inverse: the result is the exact solve's,
    bit for bit, on a full-length record."""
    y = eeg(32, 30504, seed=5)
    d = oracle.directions(32, 32)
    a, _, _ = run_gpu(y, d, 3, 3, solve_window=-1)
    b, _, _ = run_gpu(y, d, 3, 3)
    assert np.array_equal(a, b)


def _as_f32_inputs(y, d):
    y32 = np.ascontiguousarray(y, dtype=np.float32)
    d32 = np.ascontiguousarray(d, dtype=np.float32)
    return y32, d32, y32.astype(np.float64), d32.astype(np.float64)


@pytest.mark.parametrize("C,L,K", [(8, 2000, 64), (32, 8192, 64)])
def test_mixed_extrema_certified_against_fp64(C, L, K):
    """Mixed form (double-float working signal, certified FP32 projection,
    FP32 splines): the first sift's extrema sets equal the FP64 path's on the
    same input, and every IMF stays within 1e-4 relative L2."""
    y = eeg(C, L, seed=21) if C > 8 else mg.synth_tones(C, L, 1000.0, seed=3)
    d = oracle.directions(C, K)
    y32, d32, y64, d64 = _as_f32_inputs(y, d)
    a, sa, ta = run_gpu(y64, d64, 6, 10, trace=True)
    b, sb, tb = run_gpu(y32, d32, 6, 10, precision=mg.PREC_MIXED, trace=True)
    assert np.array_equal(ta["count"][0, 0], tb["count"][0, 0])
    assert np.array_equal(ta["hash"][0, 0], tb["hash"][0, 0])
    for i in range(6):
        assert rel_l2(b[i], a[i]) < 1e-4, i
    assert sb.flags == 0


def test_fp32_path_runs_fast_eval_and_reconstructs():
    y = eeg(16, 5000, seed=4)
    d = oracle.directions(16, 32)
    y32, d32, _, _ = _as_f32_inputs(y, d)
    imfs, st, _ = run_gpu(y32, d32, 5, 6, precision=mg.PREC_F32)
    assert np.isfinite(imfs).all()
    assert np.abs(imfs.astype(np.float64).sum(axis=0) - y32).max() < 1e-3 * np.abs(y32).max()


@pytest.mark.parametrize("seed", [0, 1])
def test_mixed_stop_mode_matches_fp64_sift_counts(seed):
    """Stop mode on the 8-channel tone record (64 directions, thresholds
    0.075 / 0.75 / 0.075, up to 10 IMFs): the mixed form makes the FP64 path's
    decisions -- the same number of IMFs, the same sift count for every IMF,
    the same extrema sets at every pass -- and its IMFs are within 1e-6."""
    import memd_signals

    y = memd_signals.tones(8, 2000, 1000.0, seed=seed)
    d = oracle.directions(8, 64)
    y32, d32, y64, d64 = _as_f32_inputs(y, d)
    a, sa, ta = run_gpu(y64, d64, 11, 200, trace=True, stop_mode=mg.STOP_CRITERION)
    b, sb, tb = run_gpu(y32, d32, 11, 200, precision=mg.PREC_MIXED, trace=True, stop_mode=mg.STOP_CRITERION)
    assert sb.n_imfs == sa.n_imfs >= 1
    assert list(sb.sifts[: sb.n_imfs]) == list(sa.sifts[: sa.n_imfs])
    assert np.array_equal(ta["count"], tb["count"]) and np.array_equal(ta["hash"], tb["hash"])
    for i in range(11):
        if np.linalg.norm(a[i]) > 0:
            assert rel_l2(b[i], a[i]) < 1e-6, i
    assert np.abs(b.astype(np.float64).sum(axis=0) - y32).max() < 1e-4 * np.abs(y32).max()


@pytest.mark.parametrize("C,L,K,chunk", [(8, 2000, 64, 0), (5, 3000, 16, 0), (40, 4000, 24, 0),
                                         (32, 8192, 64, 0), (12, 5000, 40, 16), (128, 10000, 256, 0)])
def test_mixed_impulse_mean_matches_fp64_sets(C, L, K, chunk):
    """Mixed form, fixed mode: the impulse-accumulation mean (default) and the
    direct evaluation of every envelope give the FP64 path's extrema sets at
    every sift; IMFs agree with FP64 to the float32 output rounding."""
    y = eeg(C, L, seed=31) if C > 8 else mg.synth_tones(C, L, 1000.0, seed=5)
    d = oracle.directions(C, K)
    y32, d32, y64, d64 = _as_f32_inputs(y, d)
    nimf = 6
    a, sa, ta = run_gpu(y64, d64, nimf, 10, trace=True)
    b, sb, tb = run_gpu(y32, d32, nimf, 10, precision=mg.PREC_MIXED, trace=True, dir_chunk=chunk)
    c, sc, tc = run_gpu(y32, d32, nimf, 10, precision=mg.PREC_MIXED, trace=True, dir_chunk=chunk, mean_eval=1)
    for t in (tb, tc):
        assert np.array_equal(ta["count"][: nimf - 1, :10], t["count"][: nimf - 1, :10])
        assert np.array_equal(ta["hash"][: nimf - 1, :10], t["hash"][: nimf - 1, :10])
    for i in range(nimf):
        assert rel_l2(b[i], a[i]) < 1e-6, i
        assert rel_l2(b[i], c[i]) < 1e-6, i
    assert sb.flags == 0 and sc.flags == 0


def test_mixed_impulse_mean_nan_when_no_direction_qualifies():
    y = np.tile(np.arange(96, dtype=np.float32), (4, 1))  # monotone: no interior extrema
    d = oracle.directions(4, 8).astype(np.float32)
    b, sb, _ = run_gpu(y, d, 2, 1, precision=mg.PREC_MIXED)
    assert sb.flags & mg.FLAG_NO_QUALIFIED_DIRECTION
    assert np.isnan(b[0]).all()


def test_long_record_mixed_runs_and_matches_fp64():
    """64 channels x 262,144 samples (the long-record length, past the
    reference's int32 indexing at 256 directions): the mixed form runs without
    overflow flags and its first IMFs follow the FP64 path's."""
    C, L, K = 64, 262144, 32
    y = mg.synth_eeg(C, L, 512.0, seed=9).astype(np.float32)
    d = oracle.directions(C, K).astype(np.float32)
    a, sa, ta = run_gpu(y.astype(np.float64), d.astype(np.float64), 3, 2, trace=True)
    b, sb, tb = run_gpu(y, d, 3, 2, precision=mg.PREC_MIXED, trace=True)
    assert sa.flags == 0 and sb.flags == 0
    assert np.array_equal(ta["count"][:2, :2], tb["count"][:2, :2])
    assert np.array_equal(ta["hash"][:2, :2], tb["hash"][:2, :2])
    for i in range(3):
        assert rel_l2(b[i], a[i]) < 1e-6, i
    assert np.abs(b.astype(np.float64).sum(axis=0) - y).max() < 1e-4 * np.abs(y).max()


@pytest.mark.parametrize("precision", [mg.PREC_F64, mg.PREC_MIXED])
def test_two_tone_separation_on_gpu(precision):
    """Known answer: a 60 Hz and a 5 Hz tone in two channels come out as the
    first IMF and the rest, away from the record's ends."""
    L, fs = 2000, 1000.0
    n = np.arange(L) / fs
    hi = np.stack([np.sin(2 * np.pi * 60 * n), 0.7 * np.sin(2 * np.pi * 60 * n + 1.0)])
    lo = np.stack([np.sin(2 * np.pi * 5 * n + 0.3), 1.3 * np.sin(2 * np.pi * 5 * n + 2.0)])
    y = hi + lo
    d = oracle.directions(2, 16)
    if precision == mg.PREC_MIXED:
        y, d = y.astype(np.float32), d.astype(np.float32)
    imfs, st, _ = run_gpu(y, d, 3, 10, precision=precision)
    imfs = imfs.astype(np.float64)
    core = slice(200, L - 200)
    assert np.linalg.norm(imfs[0][:, core] - hi[:, core]) / np.linalg.norm(hi[:, core]) < 0.03
    rest = imfs[1] + imfs[2]
    assert np.linalg.norm(rest[:, core] - lo[:, core]) / np.linalg.norm(lo[:, core]) < 0.03
    assert st.flags == 0
