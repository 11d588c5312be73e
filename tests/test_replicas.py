"""bench.py's multi-GPU mode runs independent replicas (the path does not shard): each rank steps
its own seeded plasma and the ranks only agree on timing.  This checks the host-side aggregation
with two gloo ranks on the CPU: the barrier, the max of the per-rank times and the sum of the
per-rank particle counts that make the whole-job value.
"""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench

    d = bench.Dist(world)
    d.barrier()
    t = d.max(1.0 + rank)  # per-rank elapsed time
    n = d.sum(1000.0 * (rank + 1))  # per-rank particle count
    out[rank] = (d.world, d.rank, t, n)
    d.close()


@pytest.mark.timeout(120)
def test_two_gloo_ranks_aggregate_time_and_work():
    ctx = mp.get_context("spawn")
    port = _free_port()
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(100)
            assert p.exitcode == 0
        res = dict(out)
    assert res[0] == (2, 0, 2.0, 3000.0)
    assert res[1] == (2, 1, 2.0, 3000.0)
