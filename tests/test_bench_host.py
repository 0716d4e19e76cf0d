"""Host-side inputs of the benchmark line (no GPU): the committed DRAM-traffic
summary that the roofline's `traffic` field quotes, and the workload
description both arms print."""
import bench


def test_traffic_summary_covers_every_mixed_stage_and_names_its_capture():
    tr = bench.load_profile_traffic()
    for stage in ("eval", "solve", "project", "factor", "compact"):
        e = tr[f"mixed:{stage}"]
        assert e["bytes_per_launch"] > 0, stage
        assert e["launches"] >= 80, stage
        # the capture command: one pass of duration and DRAM counters, clocks untouched
        assert "--clock-control none" in e["source"], stage
        assert "profile_case.py eeg32" in e["source"], stage
        assert "dram__bytes_read.sum" in e["source"] and "dram__bytes_write.sum" in e["source"], stage
    # the mean reads each knot solution once: its traffic sits between the
    # signal read and written once (2 C L 8 bytes) and the whole K C L solution
    # array of one sift at the densest knots
    C, L, K = bench.WL["C"], bench.WL["L"], bench.WL["K"]
    assert 2 * C * L * 8 < tr["mixed:eval"]["bytes_per_launch"] < K * C * L * 8


def test_both_arms_describe_the_same_workload():
    cfg = bench.bench_config(1)
    assert cfg["workload"] == bench.WL["workload"]
    assert (cfg["C"], cfg["L"], cfg["K"]) == (32, 30504, 128)
    assert (cfg["num_imfs"], cfg["max_iter"], cfg["sifts_per_step"]) == (9, 10, 80)
    assert cfg["l2"] == "flushed between steps" and cfg["parallelism"] == "single"
    assert bench.bench_config(8)["parallelism"] == "replicas"
