"""The replicated (N > 1) measurement path on the host: two gloo ranks each
run bench.measure_replicated -- the helper every leg of bench.py times with --
over a real decomposition of their own record (the CPU oracle on a small
seeded record, host-clock step timer).  The step time reported is the slowest
rank's, the units are summed over the ranks, and each rank's IMFs are those of
its own record, as bench.py does over NCCL when every GPU decomposes its own
record."""
import os
import socket
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
C, L, K, NIMF, IT = 4, 1500, 16, 4, 5


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _record(rank):
    sys.path.insert(0, os.path.join(REPO, "memd-gpu_gb300", "py"))
    import memd_signals

    return memd_signals.as_float32_record(memd_signals.eeg(C, L + 500 * rank, 256.0, seed=rank))


def _rank_main(rank, world, port, results):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    sys.path.insert(0, REPO)
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import bench
    import oracle

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        y = _record(rank)  # replicas decompose records of different lengths
        d = oracle.directions(C, K)
        out = {}

        def step():
            out["imfs"], _ = oracle.memd(y, d, NIMF, IT, nthreads=1)

        m = bench.measure_replicated(step, float(C * y.shape[1]), steps=2, warmup=1, timer=bench.WallSteps(),
                                     device="cpu")
        results[rank] = (m, out["imfs"])
    finally:
        dist.destroy_process_group()


def test_two_replicas_decompose_their_own_records_and_reduce_over_ranks():
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle

    port = _free_port()
    with mp.get_context("spawn").Manager() as mgr:
        results = mgr.dict()
        mp.spawn(_rank_main, args=(2, port, results), nprocs=2, join=True)
        got = dict(results)
    local = [got[r][0]["local_ms_per_step"] for r in (0, 1)]
    units = C * (L + L + 500)
    for rank in (0, 1):
        m, imfs = got[rank]
        assert m["ms_per_step"] == max(local)
        assert m["units"] == units
        assert abs(m["value"] - units / (max(local) / 1e3)) <= 1e-9 * m["value"]
        want, _ = oracle.memd(_record(rank), oracle.directions(C, K), NIMF, IT, nthreads=1)
        assert np.array_equal(imfs, want)


def test_single_process_reductions_are_identity():
    sys.path.insert(0, REPO)
    import bench

    assert not dist.is_initialized()
    assert bench.max_over_ranks(7.25, device="cpu") == 7.25
    assert bench.sum_over_ranks(3.0, device="cpu") == 3.0
