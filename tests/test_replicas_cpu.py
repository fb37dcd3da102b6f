"""The multi-GPU path is replicas only (every rank runs its own problems; no
data-path collective).  Its host-side coordination -- process group, barrier,
max-over-ranks timing, sharding of independent units -- runs here as two gloo
ranks on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import bench
    import torch.distributed as dist

    w, r, _ = bench.dist_init()
    bench.barrier(w)
    t = bench.max_over_ranks(w, 10.0 + r)   # the slowest rank sets the step time
    units = bench.shard_units(13, w, r)
    q.put((r, w, t, units))
    dist.destroy_process_group()


def test_two_gloo_replicas_coordinate():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [2, 2]
    assert [r[2] for r in res] == [11.0, 11.0]
    a, b = res[0][3], res[1][3]
    assert not set(a) & set(b) and sorted(a + b) == list(range(13))


def test_shard_units_single_rank_is_everything():
    import bench
    assert bench.shard_units(5, 1, 0) == [0, 1, 2, 3, 4]
