"""Batched runs: many epochs of uneven length decomposed in one pass
(memd_run_batched_*), checked against one single-record run per epoch."""
import numpy as np
import pytest

import memd_gb300 as mg
import oracle


def test_batched_plan_limits_on_host():
    with pytest.raises(mg.MemdError) as ei:
        mg.Plan(4, 1000, 8, 3, 2, max_epochs=4, boundary=mg.BOUNDARY_MIRROR)
    assert ei.value.status == mg.MEMD_ERR_UNSUPPORTED
    with pytest.raises(mg.MemdError) as ei:
        mg.Plan(4, 1 << 20, 8, 3, 2, max_epochs=512)
    assert ei.value.status == mg.MEMD_ERR_INVALID


def _epochs(C, lengths, seed):
    recs = [mg.synth_eeg(C, L, 256.0, seed=seed + e) for e, L in enumerate(lengths)]
    offs = np.concatenate([[0], np.cumsum([C * L for L in lengths])[:-1]]).astype(np.int64)
    return recs, offs


def _run_batched(recs, lengths, offs, d, nimf, it, prec, **kw):
    torch = pytest.importorskip("torch")
    C = recs[0].shape[0]
    tdt = torch.float64 if prec == mg.PREC_F64 else torch.float32
    plan = mg.Plan(C, max(lengths), d.shape[0], nimf, it, precision=prec, max_epochs=len(lengths), **kw)
    y = torch.as_tensor(np.concatenate([r.ravel() for r in recs]), dtype=tdt, device="cuda")
    out = torch.full((nimf * y.numel(),), float("nan"), dtype=tdt, device="cuda")
    dd = torch.as_tensor(d, dtype=tdt, device="cuda")
    st = plan.run_batched(y, lengths, offs, dd, out)
    o = out.cpu().numpy()
    plan.close()
    return [o[nimf * off: nimf * off + nimf * C * L].reshape(nimf, C, L) for off, L in zip(offs, lengths)], st


def _run_single(rec, d, nimf, it, prec, **kw):
    torch = pytest.importorskip("torch")
    C, L = rec.shape
    tdt = torch.float64 if prec == mg.PREC_F64 else torch.float32
    plan = mg.Plan(C, L, d.shape[0], nimf, it, precision=prec, **kw)
    out = torch.empty((nimf, C, L), dtype=tdt, device="cuda")
    plan.run(torch.as_tensor(rec, dtype=tdt, device="cuda"), torch.as_tensor(d, dtype=tdt, device="cuda"), out)
    o = out.cpu().numpy()
    plan.close()
    return o


LENGTHS = [1000, 37, 512, 2049, 4096, 777, 1024]


@pytest.mark.gpu
@pytest.mark.parametrize("chunk", [0, 5])
def test_batched_f64_equals_single_runs_bitwise(chunk):
    """Epoch boundaries are identity rows of the spline systems and every
    tile, span and bitmask word stays inside one epoch, so each epoch's IMFs
    equal a single-record run of it bit for bit (FP64)."""
    C, K, nimf, it = 6, 16, 4, 4
    recs, offs = _epochs(C, LENGTHS, seed=50)
    d = oracle.directions(C, K)
    got, st = _run_batched(recs, LENGTHS, offs, d, nimf, it, mg.PREC_F64, dir_chunk=chunk)
    for rec, g in zip(recs, got):
        ref = _run_single(rec, d, nimf, it, mg.PREC_F64, dir_chunk=chunk)
        assert np.array_equal(g, ref, equal_nan=True)


@pytest.mark.gpu
@pytest.mark.parametrize("chunk", [0, 5])
def test_batched_not_a_knot_f64_equals_single_runs_bitwise(chunk):
    """Not-a-knot ends per record (the second and second-to-last rows of each
    record in the factorisation, the end extrapolations per record after the
    sweeps): each epoch equals a single-record not-a-knot run bit for bit
    (FP64), including records of fewer than four knots (natural ends)."""
    C, K, nimf, it = 6, 16, 4, 4
    lengths = [1000, 37, 9, 2049, 4096, 777, 1024]
    recs, offs = _epochs(C, lengths, seed=90)
    d = oracle.directions(C, K)
    kw = dict(dir_chunk=chunk, spline_end=mg.SPLINE_NOT_A_KNOT)
    got, st = _run_batched(recs, lengths, offs, d, nimf, it, mg.PREC_F64, **kw)
    assert st.flags in (0, 1)  # 1: an epoch too short for any qualified direction (0/0, as a single run)
    for rec, g in zip(recs, got):
        ref = _run_single(rec, d, nimf, it, mg.PREC_F64, **kw)
        assert np.array_equal(g, ref, equal_nan=True)


@pytest.mark.gpu
def test_batched_not_a_knot_mixed_tracks_fp64():
    C, K, nimf, it = 8, 24, 5, 5
    lengths = [3000, 1500, 4100, 2048, 900]
    recs, offs = _epochs(C, lengths, seed=71)
    d = oracle.directions(C, K).astype(np.float32).astype(np.float64)
    recs32 = [r.astype(np.float32) for r in recs]
    kw = dict(spline_end=mg.SPLINE_NOT_A_KNOT)
    got, st = _run_batched(recs32, lengths, offs, d, nimf, it, mg.PREC_MIXED, **kw)
    assert st.flags == 0
    for rec, g in zip(recs32, got):
        r64 = _run_single(rec.astype(np.float64), d, nimf, it, mg.PREC_F64, **kw)
        single = _run_single(rec, d, nimf, it, mg.PREC_MIXED, **kw)
        for i in range(nimf):
            assert np.linalg.norm(g[i] - r64[i]) <= 1e-6 * np.linalg.norm(r64[i])
            assert np.linalg.norm(g[i] - single[i]) <= 1e-6 * np.linalg.norm(single[i])


@pytest.mark.gpu
@pytest.mark.parametrize("chunk", [0, 5])
def test_batched_f32_equals_single_runs_bitwise(chunk):
    """The FP32 form (the reference's own precision) batched: each epoch's
    IMFs equal a single-record FP32 run bit for bit, natural and not-a-knot
    ends."""
    C, K, nimf, it = 6, 16, 4, 4
    recs, offs = _epochs(C, LENGTHS, seed=60)
    recs = [r.astype(np.float32) for r in recs]
    d = oracle.directions(C, K)
    for spline in (mg.SPLINE_NATURAL, mg.SPLINE_NOT_A_KNOT):
        kw = dict(dir_chunk=chunk, spline_end=spline)
        got, st = _run_batched(recs, LENGTHS, offs, d, nimf, it, mg.PREC_F32, **kw)
        for rec, g in zip(recs, got):
            ref = _run_single(rec, d, nimf, it, mg.PREC_F32, **kw)
            assert np.array_equal(g, ref, equal_nan=True)


@pytest.mark.gpu
def test_batched_mixed_matches_single_runs_and_fp64():
    C, K, nimf, it = 8, 24, 5, 5
    lengths = [3000, 1500, 4100, 2048, 900]
    recs, offs = _epochs(C, lengths, seed=70)
    d = oracle.directions(C, K).astype(np.float32).astype(np.float64)
    recs32 = [r.astype(np.float32) for r in recs]
    got, st = _run_batched(recs32, lengths, offs, d, nimf, it, mg.PREC_MIXED)
    ref64, _ = _run_batched([r.astype(np.float64) for r in recs32], lengths, offs, d, nimf, it, mg.PREC_F64)
    assert st.flags == 0
    for rec, g, r64 in zip(recs32, got, ref64):
        single = _run_single(rec, d, nimf, it, mg.PREC_MIXED)
        for i in range(nimf):
            assert np.linalg.norm(g[i] - single[i]) <= 1e-6 * np.linalg.norm(single[i])
            assert np.linalg.norm(g[i] - r64[i]) <= 1e-6 * np.linalg.norm(r64[i])


@pytest.mark.gpu
def test_batched_mixed_direct_mean_matches_impulse_accumulation():
    """The mixed form's direct mean (every envelope at every sample) in a
    batch: the same IMFs as the impulse-accumulation batch to 1e-6."""
    C, K, nimf, it = 8, 24, 5, 5
    lengths = [3000, 1500, 4100, 2048, 900]
    recs, offs = _epochs(C, lengths, seed=72)
    d = oracle.directions(C, K).astype(np.float32).astype(np.float64)
    recs32 = [r.astype(np.float32) for r in recs]
    a, sa = _run_batched(recs32, lengths, offs, d, nimf, it, mg.PREC_MIXED, mean_eval=1)
    b, sb = _run_batched(recs32, lengths, offs, d, nimf, it, mg.PREC_MIXED)
    assert sa.flags == 0 and sb.flags == 0
    for ga, gb in zip(a, b):
        for i in range(nimf):
            assert np.linalg.norm(ga[i] - gb[i]) <= 1e-6 * np.linalg.norm(gb[i])


@pytest.mark.gpu
def test_batched_api_misuse():
    torch = pytest.importorskip("torch")
    plan = mg.Plan(4, 500, 8, 3, 2, max_epochs=2)
    y = torch.zeros(4 * 500, dtype=torch.float64, device="cuda")
    d = torch.as_tensor(oracle.directions(4, 8), device="cuda")
    out = torch.zeros(3 * 4 * 500, dtype=torch.float64, device="cuda")
    with pytest.raises(mg.MemdError) as ei:
        plan.run(y.view(4, 500), d, out.view(3, 4, 500))
    assert ei.value.status == mg.MEMD_ERR_UNSUPPORTED
    with pytest.raises(mg.MemdError) as ei:
        plan.run_batched(y, [600], [0], d, out)
    assert ei.value.status == mg.MEMD_ERR_INVALID
    with pytest.raises(mg.MemdError) as ei:
        plan.run_batched(y, [100, 100, 100], [0, 400, 800], d, out)
    assert ei.value.status == mg.MEMD_ERR_INVALID
    plan.close()


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [mg.PREC_F64, mg.PREC_F32, mg.PREC_MIXED])
def test_batched_profile_equals_graph_run(prec):
    """The kernel-by-kernel profiled batched run computes what the graph does."""
    torch = pytest.importorskip("torch")
    C, nimf, it = 4, 3, 3
    lengths = [700, 1500, 64]
    recs, offs = _epochs(C, lengths, 77)
    d = oracle.directions(C, 10)
    tdt = torch.float64 if prec == mg.PREC_F64 else torch.float32
    plan = mg.Plan(C, max(lengths), 10, nimf, it, precision=prec, max_epochs=len(lengths))
    y = torch.as_tensor(np.concatenate([r.ravel() for r in recs]), dtype=tdt, device="cuda")
    dd = torch.as_tensor(d, dtype=tdt, device="cuda")
    a = torch.empty((nimf * y.numel(),), dtype=tdt, device="cuda")
    b = torch.empty_like(a)
    plan.run_batched(y, lengths, offs, dd, a)
    pr = plan.profile_batched(y, lengths, offs, dd, b).as_dict()
    plan.close()
    assert torch.equal(a, b)
    assert pr["solve"]["launches"] == 2 * (nimf - 1) * it and pr["eval"]["ms"] > 0


@pytest.mark.gpu
def test_batched_two_layouts_on_a_side_stream_without_sync():
    """Two batched calls with different length sets, back to back on a
    non-blocking stream with no host synchronisation between them: the second
    call's new epoch table must not reach the first call's kernels, so each
    result equals the same call made alone."""
    torch = pytest.importorskip("torch")
    C, K, nimf, it = 4, 8, 3, 3
    la, lb = [900, 1300, 200], [1500, 64, 700, 1100]
    ra, oa = _epochs(C, la, seed=90)
    rb, ob = _epochs(C, lb, seed=95)
    d = oracle.directions(C, K)
    want_a, _ = _run_batched(ra, la, oa, d, nimf, it, mg.PREC_F64)
    want_b, _ = _run_batched(rb, lb, ob, d, nimf, it, mg.PREC_F64)
    plan = mg.Plan(C, 1500, K, nimf, it, precision=mg.PREC_F64, max_epochs=4)
    side = torch.cuda.Stream()
    ya = torch.as_tensor(np.concatenate([r.ravel() for r in ra]), device="cuda")
    yb = torch.as_tensor(np.concatenate([r.ravel() for r in rb]), device="cuda")
    dd = torch.as_tensor(d, device="cuda")
    outa = torch.full((nimf * ya.numel(),), float("nan"), dtype=torch.float64, device="cuda")
    outb = torch.full((nimf * yb.numel(),), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    with torch.cuda.stream(side):
        plan.run_batched(ya, la, oa, dd, outa, stream=side, stats=False)
        plan.run_batched(yb, lb, ob, dd, outb, stream=side, stats=False)
    side.synchronize()
    plan.close()
    ga, gb = outa.cpu().numpy(), outb.cpu().numpy()
    for got, want, offs, lens in ((ga, want_a, oa, la), (gb, want_b, ob, lb)):
        for w, off, L in zip(want, offs, lens):
            assert np.array_equal(got[nimf * off: nimf * off + nimf * C * L].reshape(nimf, C, L), w, equal_nan=True)


def _stop_epochs(C, lengths, seed):
    # tones for some records (few IMFs, short sift loops), EEG-shaped for the others
    recs = []
    for e, L in enumerate(lengths):
        recs.append(mg.synth_tones(C, L, 1000.0, seed=seed + e) if e % 2 else mg.synth_eeg(C, L, 256.0, seed=seed + e))
    offs = np.concatenate([[0], np.cumsum([C * L for L in lengths])[:-1]]).astype(np.int64)
    return recs, offs


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [mg.PREC_F64, mg.PREC_F32, mg.PREC_MIXED])
def test_batched_stop_mode_equals_single_runs(prec):
    """Stop criterion in a batch: every record sifts and stops by its own
    statistics, so each epoch has the IMF and sift counts of its single-record
    stop run and the same IMFs (FP64 and FP32 bit for bit: the arithmetic per
    record is the same; the mixed form to 1e-6), its unused slots zero and
    the residual in the last slot."""
    torch = pytest.importorskip("torch")
    C, K, nimf, it = 6, 16, 8, 40
    lengths = [1500, 2600, 900, 37, 4100, 1024]
    recs, offs = _stop_epochs(C, lengths, seed=300)
    d = oracle.directions(C, K)
    tdt = torch.float64 if prec == mg.PREC_F64 else torch.float32
    if prec != mg.PREC_F64:
        recs = [r.astype(np.float32) for r in recs]
    kw = dict(precision=prec, stop_mode=mg.STOP_CRITERION)
    plan = mg.Plan(C, max(lengths), K, nimf, it, max_epochs=len(lengths), **kw)
    y = torch.as_tensor(np.concatenate([r.ravel() for r in recs]), dtype=tdt, device="cuda")
    out = torch.full((nimf * y.numel(),), float("nan"), dtype=tdt, device="cuda")
    st = plan.run_batched(y, lengths, offs, torch.as_tensor(d, dtype=tdt, device="cuda"), out)
    ni, sf = plan.batched_counts(len(lengths))
    plan.close()
    o = out.cpu().numpy()
    assert st.n_imfs == ni.max()
    for e, (rec, off, L) in enumerate(zip(recs, offs, lengths)):
        got = o[nimf * off: nimf * off + nimf * C * L].reshape(nimf, C, L)
        sp = mg.Plan(C, L, K, nimf, it, **kw)
        ref = torch.empty((nimf, C, L), dtype=tdt, device="cuda")
        ss = sp.run(torch.as_tensor(rec, dtype=tdt, device="cuda"), torch.as_tensor(d, dtype=tdt, device="cuda"), ref)
        sp.close()
        assert ni[e] == ss.n_imfs, e
        assert list(sf[e, : ni[e]]) == list(ss.sifts[: ss.n_imfs]), e
        r = ref.cpu().numpy()
        if prec != mg.PREC_MIXED:
            assert np.array_equal(got, r, equal_nan=True), e
        else:
            # the double-float sweeps' windows start where the batch's knot
            # counts put them, so the last bits may differ from a single run
            for i in range(nimf):
                n = np.linalg.norm(r[i])
                assert np.linalg.norm(got[i] - r[i]) <= 1e-6 * max(n, 1e-30), (e, i)


@pytest.mark.gpu
def test_batched_stop_counts_misuse():
    torch = pytest.importorskip("torch")
    plan = mg.Plan(4, 500, 8, 3, 2, max_epochs=2)  # fixed mode
    with pytest.raises(mg.MemdError) as ei:
        plan.batched_counts(2)
    assert ei.value.status == mg.MEMD_ERR_UNSUPPORTED
    plan.close()
