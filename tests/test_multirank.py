"""The N > 1 path of bench.py (replicas only: every rank steps its own copy of
the workload, no data-path collective), run as world-size-2 gloo ranks on the
CPU: the barrier before the timed region, the MAX over ranks of the timed
region, and the whole-job value world * K / t_max."""
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


def _rank(rank, world, port, ms_by_rank, K, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    import bench
    dist.barrier()
    out[rank] = bench.replica_throughput(ms_by_rank[rank], K, dist, world)
    dist.destroy_process_group()


@pytest.mark.parametrize("ms_by_rank", [(100.0, 250.0), (300.0, 120.0)])
def test_replicas_take_the_slowest_rank(ms_by_rank):
    world, K = 2, 20
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, world, port, ms_by_rank, K, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
        assert all(p.exitcode == 0 for p in procs)
        res = dict(out)
    t = max(ms_by_rank)
    for r in range(world):
        assert res[r][0] == t
        assert res[r][1] == pytest.approx(world * K / (t / 1e3))


def test_single_rank_needs_no_process_group():
    import bench
    t, v = bench.replica_throughput(50.0, 10)
    assert t == 50.0 and v == pytest.approx(200.0)
