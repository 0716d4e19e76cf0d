"""The autotuner's host logic (no GPU): shape keys, the coordinate descent
over the launch-shape knobs with a stand-in timer, JSON persistence, and the
C ABI's rejection of launch shapes outside their ranges (checked before any
CUDA call).  The GPU test tunes a small record and checks that the tuned plan
decomposes it exactly as the default plan does."""
import numpy as np
import pytest

import memd_autotune as at
import memd_gb300 as mg


def test_keys_round_lengths_up_to_powers_of_two():
    assert at.shape_key(32, 128, 30504, mg.PREC_MIXED, False, False) == "C32-K128-L32768-mixed-single-fixed"
    assert at.shape_key(32, 64, 8192, mg.PREC_F64, True, False) == "C32-K64-L8192-f64-batched-fixed"
    cfg = mg.default_config(channels=8, length=2000, directions=64, precision=mg.PREC_F64, stop_mode=1)
    assert at.config_key(cfg) == "C8-K64-L2048-f64-single-stop"


def test_coordinate_descent_takes_the_fastest_valid_value_per_knob():
    space = {"a": [0, 1, 2], "b": [0, 5]}
    cost = {(0, 0): 10.0, (1, 0): 8.0, (2, 0): 6.0, (2, 5): 5.0, (0, 5): 1.0}

    def measure(choice):
        k = (choice["a"], choice["b"])
        return cost.get(k, 9.0), k

    # value 2 of knob a is fastest but gives a different result: rejected
    valid = lambda base, res: res != (2, 0) and res != (2, 5)
    best, ms, log = at.coordinate_descent(measure, space, valid)
    assert best == {"a": 1, "b": 0} and ms == 8.0
    assert [t["valid"] for t in log] == [True, True, False, True]


def test_store_and_lookup_round_trip(tmp_path, monkeypatch):
    f = tmp_path / "t.json"
    monkeypatch.setenv("MEMD_TUNING_FILE", str(f))
    cfg = mg.default_config(channels=4, length=1000, directions=8, precision=mg.PREC_MIXED)
    assert at.lookup(cfg) is None
    at.store(at.config_key(cfg), {"solve_segment": 128}, {"ms": 1.0})
    assert at.lookup(cfg) == {"solve_segment": 128}


@pytest.mark.parametrize("bad", [dict(solve_segment=100), dict(solve_segment=2048), dict(solve_min_segment=512),
                                 dict(factor_segment=2), dict(solve_queue=3), dict(mean_ctas=64),
                                 dict(proj_tile_n=40), dict(proj_tile_n=512), dict(solve_layout=3)])
def test_out_of_range_launch_shapes_are_rejected(bad):
    with pytest.raises(mg.MemdError) as ei:
        mg.Plan(4, 1000, 8, 3, 2, precision=mg.PREC_MIXED, tuning=bad)
    assert ei.value.status == mg.MEMD_ERR_INVALID


@pytest.mark.gpu
def test_tuned_plan_decomposes_as_the_default_plan(tmp_path, monkeypatch):
    torch = pytest.importorskip("torch")
    import memd_signals
    import oracle

    monkeypatch.setenv("MEMD_TUNING_FILE", str(tmp_path / "t.json"))
    y = memd_signals.as_float32_record(memd_signals.eeg(8, 3000, 256.0, 3))
    d = oracle.directions(8, 24)
    for prec in (mg.PREC_MIXED, mg.PREC_F64):
        key, choice, ms, ms0, log = at.tune_record(y, d, 4, 4, prec, reps=1)
        assert all(t["ms"] > 0 for t in log) and len(log) > 4
        cfg = mg.default_config(channels=8, length=3000, directions=24, precision=prec)
        assert at.lookup(cfg) == choice
        tdt = torch.float64 if prec == mg.PREC_F64 else torch.float32
        outs = []
        for tun in (None, "auto"):
            plan = mg.Plan(8, 3000, 24, 4, 4, precision=prec, tuning=tun)
            o = torch.empty((4, 8, 3000), dtype=tdt, device="cuda")
            plan.run(torch.as_tensor(y, dtype=tdt, device="cuda"), torch.as_tensor(d, dtype=tdt, device="cuda"), o)
            if tun == "auto":
                assert plan.tuning() == choice
            plan.close()
            outs.append(o.cpu().numpy().astype(np.float64))
        tol = 1e-10 if prec == mg.PREC_F64 else 1e-6
        assert np.linalg.norm(outs[1] - outs[0]) <= tol * np.linalg.norm(outs[0])


@pytest.mark.gpu
def test_work_queue_substitution_gives_the_static_results():
    """The device work queue (persistent sweeps pulling segments by ticket)
    computes exactly what one warp per possible segment computes."""
    torch = pytest.importorskip("torch")
    import oracle

    for prec, C, L, K, kw in ((mg.PREC_F64, 6, 5000, 24, {}), (mg.PREC_MIXED, 40, 4000, 20, {}),
                              (mg.PREC_MIXED, 12, 3000, 40, {"dir_chunk": 16})):
        y = mg.synth_eeg(C, L, 256.0, seed=C)
        d = oracle.directions(C, K)
        tdt = torch.float64 if prec == mg.PREC_F64 else torch.float32
        outs = []
        for q in (2, 1):
            plan = mg.Plan(C, L, K, 4, 4, precision=prec, tuning={"solve_queue": q}, **kw)
            o = torch.empty((4, C, L), dtype=tdt, device="cuda")
            st = plan.run(torch.as_tensor(y, dtype=tdt, device="cuda"), torch.as_tensor(d, dtype=tdt, device="cuda"), o)
            assert st.flags == 0 and plan.tuning()["solve_queue"] == q
            plan.close()
            outs.append(o.cpu().numpy())
        assert np.array_equal(outs[0], outs[1])


@pytest.mark.gpu
def test_in_place_substitution_gives_the_separate_arrays_results():
    """The solution written over the eliminated right-hand side (the halo
    rows a warp reads from the next segment copied aside by the forward
    sweep) computes exactly what separate arrays compute: single records
    (FP64, mixed with direction chunks, the work queue), batched epochs
    (mixed, FP64 with not-a-knot ends)."""
    torch = pytest.importorskip("torch")
    import oracle

    cases = ((mg.PREC_F64, 6, 5000, 24, {}, {}), (mg.PREC_MIXED, 40, 4000, 20, {}, {}),
             (mg.PREC_MIXED, 12, 3000, 40, {"dir_chunk": 16}, {}), (mg.PREC_MIXED, 8, 6000, 16, {}, {"solve_queue": 1}),
             (mg.PREC_F32, 8, 3000, 16, {}, {}))
    for prec, C, L, K, kw, tun in cases:
        y = mg.synth_eeg(C, L, 256.0, seed=C + L)
        d = oracle.directions(C, K)
        tdt = torch.float64 if prec == mg.PREC_F64 else torch.float32
        outs = []
        for lay in (2, 1):
            plan = mg.Plan(C, L, K, 4, 4, precision=prec, tuning=dict(tun, solve_layout=lay), **kw)
            assert plan.tuning()["solve_layout"] == lay
            o = torch.empty((4, C, L), dtype=tdt, device="cuda")
            st = plan.run(torch.as_tensor(y, dtype=tdt, device="cuda"), torch.as_tensor(d, dtype=tdt, device="cuda"), o)
            assert st.flags == 0
            plan.close()
            outs.append(o.cpu().numpy())
        assert np.array_equal(outs[0], outs[1]), (prec, C, L, K)
    C, K = 8, 16
    lengths = np.array([1500, 2600, 900, 4100], dtype=np.int64)
    recs = [mg.synth_eeg(C, int(n), 256.0, seed=200 + i) for i, n in enumerate(lengths)]
    offs = np.concatenate([[0], np.cumsum(C * lengths)[:-1]]).astype(np.int64)
    for prec, kw in ((mg.PREC_MIXED, {}), (mg.PREC_F64, {"spline_end": mg.SPLINE_NOT_A_KNOT})):
        tdt = torch.float64 if prec == mg.PREC_F64 else torch.float32
        y = torch.as_tensor(np.concatenate([r.ravel() for r in recs]), dtype=tdt, device="cuda")
        d = torch.as_tensor(oracle.directions(C, K), dtype=tdt, device="cuda")
        outs = []
        for lay in (2, 1):
            plan = mg.Plan(C, int(lengths.max()), K, 4, 4, precision=prec, max_epochs=4,
                           tuning={"solve_layout": lay}, **kw)
            o = torch.empty(4 * y.numel(), dtype=tdt, device="cuda")
            st = plan.run_batched(y, lengths, offs, d, o)
            assert st.flags == 0
            plan.close()
            outs.append(o.cpu().numpy())
        assert np.array_equal(outs[0], outs[1]), prec


@pytest.mark.gpu
def test_in_place_layout_falls_back_where_it_does_not_apply():
    """Asked for where it cannot run (segments shorter than the substitution's
    halo; one record with not-a-knot ends), the in-place layout gives way to
    separate arrays: the plan reports that layout and computes what the
    default plan computes."""
    torch = pytest.importorskip("torch")
    import oracle

    C, L, K = 8, 3000, 16
    y = torch.as_tensor(mg.synth_eeg(C, L, 256.0, seed=77), dtype=torch.float64, device="cuda")
    d = torch.as_tensor(oracle.directions(C, K), dtype=torch.float64, device="cuda")
    for tun, kw in (({"solve_min_segment": 16}, {}), ({}, {"spline_end": mg.SPLINE_NOT_A_KNOT})):
        outs = []
        for t in (dict(tun), dict(tun, solve_layout=1)):
            plan = mg.Plan(C, L, K, 4, 4, precision=mg.PREC_F64, tuning=t, **kw)
            assert plan.tuning()["solve_layout"] == 2
            o = torch.empty((4, C, L), dtype=torch.float64, device="cuda")
            assert plan.run(y, d, o).flags == 0
            plan.close()
            outs.append(o.cpu().numpy())
        assert np.array_equal(outs[0], outs[1]), (tun, kw)
