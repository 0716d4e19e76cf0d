"""The replicated (N > 1) measurement path on the host: two gloo ranks on the
CPU reduce their step times to the slowest rank's and sum their units of work,
as bench.py does over NCCL when every GPU decomposes its own record."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, results):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    sys.path.insert(0, REPO)
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        step_ms = [12.5, 20.0][rank]          # rank 1 is the slower replica
        units = [1000.0, 3000.0][rank]        # uneven epoch sets per replica
        slowest = bench.max_over_ranks(step_ms, device="cpu")
        total = bench.sum_over_ranks(units, device="cpu")
        results[rank] = (slowest, total, total / (slowest / 1e3))
    finally:
        dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank_and_all_units():
    port = _free_port()
    with mp.get_context("spawn").Manager() as mgr:
        results = mgr.dict()
        mp.spawn(_rank_main, args=(2, port, results), nprocs=2, join=True)
        got = dict(results)
    for rank in (0, 1):
        slowest, total, rate = got[rank]
        assert slowest == 20.0 and total == 4000.0
        assert abs(rate - 4000.0 / 0.020) < 1e-9


def test_single_process_reductions_are_identity():
    sys.path.insert(0, REPO)
    import bench

    assert not dist.is_initialized()
    assert bench.max_over_ranks(7.25, device="cpu") == 7.25
    assert bench.sum_over_ranks(3.0, device="cpu") == 3.0
