"""Multi-GPU form of the benchmark: replicas only. Each rank places its own
instance (seeded by its rank) with no data-path collective; the only
exchange is the max-over-ranks time. Run here as two gloo ranks on CPU."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    prob = bench.make_problem("ecp5-2k", rank)          # host-side generator only
    total_ms = 100.0 + 50.0 * rank                      # this rank's timed steps
    max_ms, value = bench.aggregate_ranks(total_ms, 10, dist, "cpu")
    out.put((rank, max_ms, value, int(prob.pin_cell.sum())))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank_and_differ_by_seed():
    pytest.importorskip("torch")
    from texo_gb300 import build
    build.build()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0][1] == res[1][1] == 150.0
    assert res[0][2] == pytest.approx(2 * 10 / 0.150)
    assert res[0][3] != res[1][3]          # the two replicas place different netlists
