"""The multi-GPU bench path's host logic on the CPU, with two ranks as plain
processes (no GPU, no PyTorch).

Scenes are independent, so ranks shard them with no exchange: rank r takes
the scenes s with s mod N == r (bench.shard).  The job-wide numbers are the
max over ranks of the times and the sum of the bodies (bench.combine_ranks
over bench.SocketRanks, the rendezvous the bench uses under a launcher)."""
import multiprocessing as mp
import os
import socket
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NSCENES = 12
WORLD = 2


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(WORLD), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port - 1)})
    sys.path.insert(0, ROOT)
    import bench
    from ornis_gb300 import scenes

    ranks, r, world, local = bench.dist_init(WORLD)
    try:
        assert (r, world, local) == (rank, WORLD, rank)
        bodies, offs, _ = scenes.batched(NSCENES)
        mine, my_offs = bench.shard(bodies, offs, rank, WORLD)
        ndyn = scenes.dynamic_count(mine)
        seconds = 1.5 + rank + 0.1  # rank 1 is the slower one; not a round number
        worst, total = bench.combine_ranks(ranks, worst=[seconds], total=[ndyn, len(my_offs) - 1])
        ranks.barrier()
        q.put((rank, mine, my_offs, worst, total))
    finally:
        ranks.close()


def test_two_ranks_shard_scenes_and_combine_timing():
    from ornis_gb300 import scenes

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(WORLD)]
    for p in procs:
        p.start()
    got = {}
    try:
        for _ in range(WORLD):
            rank, mine, my_offs, worst, total = q.get(timeout=120)
            got[rank] = (mine, my_offs, worst, total)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert all(p.exitcode == 0 for p in procs)

    bodies, offs, _ = scenes.batched(NSCENES)
    # every scene exactly once, on rank s mod N, in order
    for s in range(NSCENES):
        mine, my_offs, _, _ = got[s % WORLD]
        k = s // WORLD
        np.testing.assert_array_equal(mine[my_offs[k]:my_offs[k + 1]], bodies[offs[s]:offs[s + 1]])
    # both ranks see the slowest rank's time (exactly) and the summed counts
    ndyn_all = scenes.dynamic_count(bodies)
    for rank in range(WORLD):
        _, _, worst, total = got[rank]
        assert worst == [1.5 + (WORLD - 1) + 0.1]
        assert total == [float(ndyn_all), float(NSCENES)]


def test_one_rank_needs_no_rendezvous():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.dist_init(1) is None
