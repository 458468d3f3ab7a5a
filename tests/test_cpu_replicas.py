"""bench.py --gpus N runs N independent replicas (the time-step path has no
cross-GPU exchange): the timed region is the slowest rank's, and the value is
the facet-steps of all ranks over it. Two gloo ranks on the CPU."""
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
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    dist.barrier()
    ms = bench.slowest_rank_ms(100.0 + 50.0 * rank, dist)
    out[rank] = (ms, bench.replica_value(world, 81920, 20, ms))
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    with mp.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [mp.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    assert res[0] == res[1]
    ms, value = res[0]
    assert ms == 150.0
    assert value == pytest.approx(2 * 81920 * 20 / 0.150)


def test_one_process_is_its_own_time():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.slowest_rank_ms(42.0) == 42.0
    assert bench.replica_value(1, 1000, 10, 1000.0) == pytest.approx(10000.0)
