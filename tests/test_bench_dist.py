"""bench.py's multi-rank aggregation (replicas: every rank runs the same
steps; value = units of all ranks / the slowest rank's time) on world-size-2
gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    sys.path.insert(0, REPO)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=ws)
    try:
        t_local = [2.0, 5.0][rank]                 # rank 1 is the slow one
        t_max = bench.max_over_ranks(t_local, ws)
        out.put((rank, t_max, bench.whole_job_rate(10, t_max, ws)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_replica_aggregation_takes_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, t_max, rate in res:
        assert t_max == 5.0
        assert rate == pytest.approx(2 * 10 / 5.0)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, REPO)
    import bench
    assert bench.max_over_ranks(3.0, 1) == 3.0
    assert bench.whole_job_rate(5, 2.0, 1) == 2.5
