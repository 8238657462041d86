"""The multi-rank path on CPU: events sharded across 2 gloo ranks, each rank
clustering its shard (oracle, no GPU), results gathered on rank 0 must equal
one process clustering everything; max-over-ranks timing reduction."""
import os
import socket

import numpy as np
import pytest

import clue_gb300 as C
from clue_gb300 import synthetic as S


def test_shards_cover_every_event_once():
    b = S.uneven_batch(37, seed=3, lo=2000, hi=30000)
    for world in (1, 2, 3, 8):
        ranges = [C.shard_events(b["offsets"], r, world) for r in range(world)]
        assert ranges[0][0] == 0 and ranges[-1][1] == 37
        for (a0, a1), (b0, b1) in zip(ranges, ranges[1:]):
            assert a1 == b0 and a0 <= a1
    pts = [int(b["offsets"][e1] - b["offsets"][e0]) for e0, e1 in (C.shard_events(b["offsets"], r, 2) for r in (0, 1))]
    assert abs(pts[0] - pts[1]) < 0.5 * sum(pts)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import sys
    sys.path[:0] = [os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                    os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "heterogeneous-clue_gb300")]
    import torch.distributed as dist
    import clue_gb300 as C
    import oracle
    from clue_gb300 import synthetic as S
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    b = S.uneven_batch(9, seed=5, lo=2000, hi=20000)
    sh = C.shard_batch(b, rank, world)
    out = oracle.clue2d_batch(sh["offsets"], sh["x"], sh["y"], sh["layer"], sh["weight"], 1.3, 2.0, 2.0)
    gathered = [None] * world
    dist.all_gather_object(gathered, (sh["event_range"], out))
    m = C.dist_max(float(rank + 1))
    if rank == 0:
        q.put((gathered, m))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_match_one_process():
    import torch.multiprocessing as mp
    import oracle
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    gathered, m = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert m == 2.0
    b = S.uneven_batch(9, seed=5, lo=2000, hi=20000)
    want = oracle.clue2d_batch(b["offsets"], b["x"], b["y"], b["layer"], b["weight"], 1.3, 2.0, 2.0)
    got = {k: np.concatenate([o[k] for _, o in sorted(gathered, key=lambda g: g[0][0])]) for k in want}
    for k in want:
        assert np.array_equal(got[k].view(np.int32), want[k].view(np.int32)), k
