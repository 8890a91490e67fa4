"""The benchmark's multi-rank host logic on CPU: two gloo ranks (the same
calls the benchmark makes over NCCL, one rank per GPU, when launched with
torchrun).  Each rank corrects its own replica, so the only cross-rank step
is the max of the per-rank times; the whole-job rate counts every rank's
voxels against that max."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        per_rank_ms = [7.5, 9.25][rank]
        ms = bench.max_over_ranks(per_rank_ms, "cpu")
        rate = bench.whole_job_rate(512 ** 3, world, ms)
        dist.barrier()
        out[rank] = (ms, rate)
    finally:
        dist.destroy_process_group()


def test_two_ranks_take_the_max_time_and_count_all_voxels():
    world, port = 2, _free_port()
    with mp.get_context("spawn").Manager() as m:  # no fork: the pytest process may hold a CUDA context
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == res[1]
    ms, rate = res[0]
    assert ms == 9.25
    assert rate == pytest.approx(2 * 512 ** 3 / 9.25e-3 / 1e9)


def test_single_process_is_the_identity():
    import bench
    assert not dist.is_initialized()
    assert bench.max_over_ranks(3.5, "cpu") == 3.5
    assert bench.whole_job_rate(1000, 1, 1.0) == pytest.approx(1e-3)


def test_reference_arm_on_a_non_zero_rank_does_no_work(monkeypatch):
    import bench
    monkeypatch.setenv("RANK", "1")
    args = bench.parse(["--impl", "reference"])
    assert bench.run_reference(args) is None  # returns before touching a GPU
