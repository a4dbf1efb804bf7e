"""Multi-rank host logic on CPU (gloo, world size 2): events are split into
contiguous hit-balanced ranges with no data exchange, and the union of the
ranks' triplets equals the single-process result."""
import os
import socket

import numpy as np
import pytest

from trax_gb300 import events, sharding


def test_shards_cover_all_events_contiguously():
    rng = np.random.default_rng(0)
    for world in (1, 2, 3, 8):
        h = rng.integers(1, 40000, 1000)
        s = sharding.shard_events(h, world)
        assert s[0][0] == 0 and s[-1][1] == 1000
        assert all(a[1] == b[0] for a, b in zip(s, s[1:]))
        loads = [h[a:b].sum() for a, b in s]
        assert max(loads) <= h.sum() / world + h.max()


def test_more_ranks_than_events():
    s = sharding.shard_events(np.array([5, 7]), 4)
    assert [b - a for a, b in s].count(1) == 2 and s[-1][1] == 2


def _free_port():
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        return so.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    from oracle import oracle
    ranks = sharding.Ranks("gloo")
    b = events.generate(1, n_events=8)
    lo, hi = sharding.shard_events(b.layer_hits.sum(axis=1), world)[rank]
    part = b.subset(range(lo, hi))
    res = oracle.run(part, event_grouping=1)
    trip = set()
    for g, r in enumerate(res):
        p = r["perm"]
        offs = part.event_offsets
        for a, c, d in zip(p[r["trip_h1"]], p[r["trip_h2"]], p[r["trip_h3"]]):
            e = int(part.event[a])
            base = int(b.event_offsets[lo + e]) - int(offs[e])
            trip.add((int(a) + base, int(c) + base, int(d) + base))
    ranks.barrier()
    t_max = ranks.max(float(rank + 1))
    n_all = ranks.sum(float(len(trip)))
    ranks.close()
    q.put((rank, sorted(trip), t_max, n_all))


def test_two_gloo_ranks_reproduce_the_single_process_triplets(oracle_lib):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    union = set()
    for rank, trip, t_max, n_all in out:
        union |= set(map(tuple, trip))
        assert t_max == 2.0
    assert n_all == len(union)
    b = events.generate(1, n_events=8)
    ref = set()
    for r in oracle_lib.run(b, event_grouping=1):
        p = r["perm"]
        ref |= set(zip(p[r["trip_h1"]].tolist(), p[r["trip_h2"]].tolist(), p[r["trip_h3"]].tolist()))
    assert union == ref
