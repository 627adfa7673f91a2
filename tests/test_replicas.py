"""Multi-GPU form of the benchmark on CPU: world_size 2 over gloo.  Replicas
solve disjoint molecules, the only collective is the max-over-ranks reduction
of the timed totals, and the whole-job rate counts every rank's molecules."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    seeds = bench.replica_seeds(rank, 8)
    # rank r "took" 100 + 10 r ms plain and 50 + r ms mixed
    ms = bench.reduce_step_times([100.0 + 10 * rank, 50.0 + rank], dist, "cpu")
    names = [tuple(m["species"][0]["shells"][-1][3]) for m in bench.systems_for(rank, 2)]   # geometries
    q.put((rank, seeds, ms, names))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replicas_gloo():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = {}
    for _ in procs:
        r, seeds, ms, names = q.get(timeout=120)
        out[r] = (seeds, ms, names)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert set(out[0][0]).isdisjoint(out[1][0])
    assert out[0][1] == out[1][1] == [110.0, 51.0]     # max over ranks on every rank
    import bench
    assert bench.whole_job_rate(8, 2, 110.0) == pytest.approx(16 / 0.110)
    assert set(out[0][2]).isdisjoint(out[1][2])          # different molecules on the two ranks
