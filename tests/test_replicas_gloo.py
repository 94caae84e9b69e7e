"""The multi-process path of bench.py on CPU: two ranks over gloo.

The path does not shard (one replica per GPU), so the only cross-rank work
is timing: every rank reads its rank and world size from the launcher's
environment, the timed region is bracketed by barriers, and rank 0 reports
the units of all ranks over the slowest rank's time.  Here two processes
with different "times" check that max-over-ranks and the whole-job
aggregate come out the same on every rank.
"""
import os
import socket

import torch.multiprocessing as mp


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    w, r, local = bench.dist_env()
    seconds = bench.max_over_ranks(1.0 + rank, w)  # rank r "took" 1 + r seconds
    bench.barrier(w)
    out[rank] = (w, r, local, seconds, bench.aggregate(3.0, seconds, w))
    dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank_and_all_units():
    world = 2
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        got = dict(out)
    for rank in range(world):
        w, r, local, seconds, units_per_s = got[rank]
        assert (w, r, local) == (world, rank, rank)
        assert seconds == 2.0                       # the slower rank
        assert units_per_s == 3.0 * world / 2.0     # all ranks' units over that time
