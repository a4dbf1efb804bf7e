"""Launch shapes: block sizes, grid sizes around the shared-memory grid-build
limit, and the autotuner (trax_autotune) with its JSON cache.  Whatever shape
runs, the results must equal the oracle's at the same grid."""
import json

import numpy as np
import pytest

from trax_gb300 import events

from .test_gpu_parity import compare

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(trax_lib):
    c = trax_lib.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("blocks", [(64, 64, 128), (256, 256, 64), (96, 160, 224), (192, 96, 192)])
def test_block_sizes_keep_results(ctx, oracle_lib, blocks):
    batch = events.generate(2, n_events=3)
    ref = oracle_lib.run(batch)[0]
    ctx.upload(batch)
    ctx.set_block_sizes(*blocks)
    try:
        ctx.seed_batch(use_graph=True)
        compare(ctx.results(), ref)
    finally:
        ctx.set_block_sizes(128, 128, 256)


@pytest.mark.parametrize("grid", [(190, 128), (400, 128), (200, 256), (500, 128)])
def test_grid_sizes_around_shared_memory_limit(ctx, oracle_lib, grid):
    # (400, 128) and (200, 256) fill most of the shared-memory counters,
    # (500, 128) has more cells than fit and counts in global memory
    batch = events.generate(2, n_events=3)
    batch.n_z, batch.n_phi = grid
    ref = oracle_lib.run(batch)[0]
    ctx.upload(batch)
    ctx.seed_batch(use_graph=True)
    compare(ctx.results(), ref)


@pytest.mark.parametrize("k", [2, 4])
def test_pairs_per_thread_keep_results(ctx, oracle_lib, k):
    """The prediction count with K pairs per thread (windows staged in shared
    memory, one flat walk per lane) writes the same counts, offsets and kept
    candidates as one pair per thread, at several block sizes and numbers of
    captured candidates."""
    batch = events.generate(2, n_events=12)
    ref = oracle_lib.run(batch)[0]
    ctx.upload(batch)
    try:
        for blocks, slots in [((256, 64, 256), 0), ((128, 128, 128), 16), ((128, 256, 128), 8)]:
            ctx.set_block_sizes(*blocks)
            ctx.set_pairs_per_thread(k)
            ctx.set_candidate_slots(slots)
            assert ctx.pairs_per_thread() == k
            ctx.seed_batch(use_graph=True)
            compare(ctx.results(), ref)
    finally:
        ctx.set_pairs_per_thread(1)
        ctx.set_candidate_slots(0)
        ctx.set_block_sizes(128, 128, 256)


@pytest.mark.parametrize("workload", ["ttbar", "pileup"])
def test_candidate_slots_keep_results(ctx, oracle_lib, trax_lib, workload):
    """Any number of captured candidates per pair (the store pass copies them,
    and walks again the pairs with more) gives the same candidates; the
    automatic choice follows the batch's candidates per pair."""
    import dataclasses
    if workload == "ttbar":
        batch = events.generate(2, n_events=12)
    else:  # many candidates per pair: most pairs have more than 4
        batch = events.generate_workload(dataclasses.replace(events.workload(3), n_events=1, n_vertices=6))
    ref = oracle_lib.run(batch)[0]
    ctx.upload(batch)
    try:
        for k in [4, 8, 16, 32, 0]:
            ctx.set_candidate_slots(k)
            ctx.seed_batch(use_graph=True)
            compare(ctx.results(), ref)
            if k:
                assert ctx.candidate_slots() == k
        st = ctx.stats()
        per_pair = st.n_candidates / max(st.n_pairs, 1)
        want = 4 if per_pair <= 1 else 8 if per_pair <= 2.5 else 16 if per_pair <= 6 else 32
        assert ctx.candidate_slots() == want, (per_pair, ctx.candidate_slots())
        with pytest.raises(trax_lib.TraxError):
            ctx.set_candidate_slots(12)
    finally:
        ctx.set_candidate_slots(0)


def test_invalid_block_sizes_rejected(ctx, trax_lib):
    for bad in [(0, 128, 128), (33, 128, 128), (128, 512, 128), (128, 128, 16)]:
        with pytest.raises(trax_lib.TraxError) as e:
            ctx.set_block_sizes(*bad)
        assert e.value.code == 2


def test_autotune_picks_a_shape_and_caches_it(trax_lib, oracle_lib, tmp_path):
    batch = events.generate(1, n_events=20)
    cache = tmp_path / "tune.json"
    c = trax_lib.Context(0)
    try:
        c.upload(batch)
        res = c.autotune(cache_path=str(cache), search_grid=True, replays=1)
        assert res["from_cache"] == 0 and res["shapes_timed"] > 1
        assert 0 < res["best_ms"] <= res["default_ms"]
        shape = c.launch_config()
        assert (shape["n_z"], shape["n_phi"]) == (res["n_z"], res["n_phi"])
        assert (shape["n_z"] + 1) * (shape["n_phi"] + 1) <= 53248
        # results at the tuned shape equal the oracle's at the tuned grid
        batch.n_z, batch.n_phi = res["n_z"], res["n_phi"]
        ref = oracle_lib.run(batch)[0]
        c.seed_batch(use_graph=True)
        compare(c.results(), ref)
        assert res["pairs_per_thread"] in (1, 2, 4) and c.pairs_per_thread() == res["pairs_per_thread"]
        entries = json.loads(cache.read_text())["entries"]
        assert len(entries) == 1 and entries[0]["n_z"] == res["n_z"] and entries[0]["sm_count"] > 0
        assert entries[0]["pairs_per_thread"] == res["pairs_per_thread"]
        assert res["candidate_slots"] in (0, 4, 8, 16, 32)
        assert entries[0]["candidate_slots"] == res["candidate_slots"]
        assert res["fine_rows"] in (0, 2, 4, 8, 16) and c.fine_rows() == res["fine_rows"]
        assert entries[0]["fine_rows"] == res["fine_rows"]
    finally:
        c.close()
    # a new context with the same workload takes the cached shape without timing
    c = trax_lib.Context(0)
    try:
        c.upload(events.generate(1, n_events=20))
        res2 = c.autotune(cache_path=str(cache), search_grid=True, replays=1)
        assert res2["from_cache"] == 1 and res2["shapes_timed"] == 0
        keys = ("n_z", "n_phi", "pair_threads", "predict_threads", "filter_threads", "pairs_per_thread",
                "candidate_slots", "fine_rows")
        assert [res2[k] for k in keys] == [res[k] for k in keys]
        # a different workload gets its own entry
        c.upload(events.generate(1, n_events=21))
        res3 = c.autotune(cache_path=str(cache), search_grid=False, replays=1)
        assert res3["from_cache"] == 0
        assert len(json.loads(cache.read_text())["entries"]) == 2
    finally:
        c.close()


def test_autotune_cache_entry_without_pairs_per_thread(trax_lib, tmp_path):
    """Cache files written before the pairs-per-thread, candidate-slot and
    fine-grid axes existed still load (as 1, the library's own choice and no
    fine grid)."""
    batch = events.generate(1, n_events=20)
    cache = tmp_path / "tune.json"
    c = trax_lib.Context(0)
    try:
        c.upload(batch)
        c.autotune(cache_path=str(cache), search_grid=False, replays=1)
        doc = json.loads(cache.read_text())
        for e in doc["entries"]:
            e.pop("pairs_per_thread")
            e.pop("candidate_slots")
            e.pop("fine_rows")
        cache.write_text(json.dumps(doc))
        c.set_pairs_per_thread(4)
        c.set_candidate_slots(32)
        c.set_fine_rows(8)
        res = c.autotune(cache_path=str(cache), search_grid=False, replays=1)
        assert res["from_cache"] == 1 and res["pairs_per_thread"] == 1 and c.pairs_per_thread() == 1
        assert res["candidate_slots"] == 0
        assert res["fine_rows"] == 0 and c.fine_rows() == 0
    finally:
        c.close()
