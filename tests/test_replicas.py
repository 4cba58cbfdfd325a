"""The N > 1 path of bench.py on CPU: replicas combined over a world-size-2
gloo group (max of the step times over ranks, whole-job throughput)."""
import os
import socket

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 2.0 + rank          # rank 1 is the slower replica
    dist.barrier()
    out[rank] = bench.combine_replicas(ms, world, 1e9, dist, "cpu")
    dist.destroy_process_group()


def test_replicas_take_the_slowest_rank_and_sum_the_work():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    for r in range(2):
        ms, value = res[r]
        assert ms == 3.0                                # max over ranks
        assert abs(value - 2 * 1e9 / 3e-3 / 1e9) < 1e-9  # both replicas' work over the slowest time


def test_single_rank_needs_no_group():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    ms, value = bench.combine_replicas(4.0, 1, 8e9)
    assert ms == 4.0 and abs(value - 2000.0) < 1e-9
