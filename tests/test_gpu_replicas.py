"""Replicas: two processes, each correcting its own field, coordinated on
the host the way the benchmark coordinates its ranks (a process group for
the barrier and the max of the per-rank times; gloo here, NCCL across GPUs).
The path does not shard, so no kernel of one rank waits on another: both
run their corrections on the one GPU this test has, independently, and each
result must equal the oracle's, sweep records included; the whole-job rate
counts both ranks' voxels against the slower rank's time."""
import os
import socket

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
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
        from oracle import oracle as O
        from pmsz_anonymous_gb300 import api, fields as F
        shape, eb, seed = (40, 36, 44), 1e-3, 80 + rank  # a different field per rank
        dtype = np.float64 if rank == 0 else np.float32
        f = F.perlin_field(shape, seed, 4, 1 / 16, dtype=dtype)
        fh = F.standin(f, eb, "zfp" if rank == 0 else "sz3", seed)
        ref, _, st, sw, recs = O.correct(f, fh, eb)
        df = torch.from_numpy(f).cuda()
        dfh = torch.from_numpy(fh).cuda()
        dist.barrier()
        start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record()
        r = api.correct(df, dfh, eb)
        stop.record()
        stop.synchronize()
        ms = bench.max_over_ranks(start.elapsed_time(stop), "cpu")
        same = bool(np.array_equal(dfh.cpu().numpy().view(np.uint8), ref.view(np.uint8)))
        out[rank] = (same, r.status == st, r.sweeps == sw, bool(np.array_equal(r.log[:, :5], recs)), ms,
                     bench.whole_job_rate(f.size, world, ms), f.size)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_replicas_each_match_the_oracle(cuda):
    world, port = 2, _free_port()
    with mp.get_context("spawn").Manager() as m:  # no fork after this process has a CUDA context
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        same, status, sweeps, records, ms, rate, n = res[rank]
        assert same and status and sweeps and records, rank
    assert res[0][4] == res[1][4]  # both ranks report the max of the two times
    assert res[0][5] == pytest.approx(world * res[0][6] / (res[0][4] * 1e-3) / 1e9)
