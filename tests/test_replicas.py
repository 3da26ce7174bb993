"""The multi-GPU path is replicas only: N independent copies of the step, a
barrier, the job time = the slowest rank's, value = all ranks' bytes / that
time.  The aggregation runs here on two gloo ranks (CPU)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    dist.barrier()
    local_ms = [40.0, 55.0][rank]  # rank 1 is the slower replica
    ms = bench.replica_max_ms(local_ms, dist, "cpu")
    out[rank] = (ms, bench.job_gbs(16_642_998_272, world, ms / 20))
    dist.destroy_process_group()


def test_two_gloo_replicas_take_the_slowest_time():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        procs = [mp.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=120)
            assert p.exitcode == 0
        assert out[0][0] == out[1][0] == 55.0
        # two replicas of 16.64 GB each in 55 ms / 20 steps
        assert abs(out[0][1] - 2 * 16_642_998_272 / (55.0 / 20 * 1e-3) / 1e9) < 1e-6
