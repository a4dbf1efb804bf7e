"""The prediction count over the fine z grid (trax_set_fine_rows).

With f fine rows per grid row the grid stage also sorts every layer's hits by
a z grid f times finer, and the count pass walks only the fine rows its
window reaches.  It must find the same hits and capture the same candidates
as the walk over the grid, so every array equals the oracle's: at every f,
with few and many candidate slots (the captured candidates of one z row come
in fine order and are sorted into the grid walk's order), through the graph
and the synced path, stage by stage, with shared-memory counters (fine grids
up to 53 248 cells per layer) and global ones.
"""
import dataclasses

import numpy as np
import pytest

from trax_gb300 import events

from .test_gpu_parity import compare, stagewise
from .test_oracle_kats import degenerate_batch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(trax_lib):
    c = trax_lib.Context(0)
    yield c
    c.close()


def _pileup_event():
    return events.generate_workload(dataclasses.replace(events.workload(3), n_events=1, n_vertices=6))


def _ttbar_fine_global():
    # 500 x 128 grid: 8 fine rows make 4001 x 129 cells per layer, counted in global memory
    batch = events.generate(2, n_events=3)
    batch.n_z, batch.n_phi = 500, 128
    return batch


CASES = {
    "config 0": lambda: events.generate(0),
    "config 1": lambda: events.generate(1),
    "ttbar-like": lambda: events.generate(2, n_events=12),
    "ttbar-like, 500 x 128 grid": _ttbar_fine_global,
    "degenerate": degenerate_batch,
    "pileup event": _pileup_event,
}


@pytest.fixture
def reset(ctx):
    yield
    ctx.set_fine_rows(0)
    ctx.set_candidate_slots(0)


@pytest.mark.parametrize("case", list(CASES))
def test_fine_rows_keep_results(ctx, oracle_lib, reset, case):
    batch = CASES[case]()
    ref = oracle_lib.run(batch)[0]
    ctx.upload(batch)
    for f, slots in [(2, 0), (4, 4), (8, 16), (16, 32), (8, 4)]:
        ctx.set_fine_rows(f)
        ctx.set_candidate_slots(slots)
        assert ctx.fine_rows() == f
        for graph in (True, False):
            ctx.seed_batch(use_graph=graph)
            compare(ctx.results(), ref)


def test_fine_rows_stage_by_stage(ctx, oracle_lib, reset):
    batch = events.generate(2, n_events=4)
    ref = oracle_lib.run(batch)[0]
    ctx.set_fine_rows(4)
    compare(stagewise(ctx, batch), ref)
    # a fine grid the grid stage did not build is not walked: the count
    # pass falls back to the grid
    ctx.upload(batch)
    ctx.set_fine_rows(0)
    ctx.grid_build()
    ctx.set_fine_rows(8)
    ctx.pair_gen()
    ctx.triplet_predict()
    ctx.triplet_filter()
    n_links = ctx.connectivity(batch.d_eta_cut)
    if n_links:
        ctx.circle_fit()
        ctx.cellular_automaton()
    compare(ctx.results(), ref)


def test_fine_grid_released_between_graph_replays(ctx, oracle_lib, reset):
    """A graph captured with the fine grid, the grid stage run alone without
    it (which frees the fine grid's memory), then the fine grid again: the
    graph is captured anew instead of replayed over the freed buffers."""
    batch = events.generate(2, n_events=4)
    ref = oracle_lib.run(batch)[0]
    ctx.upload(batch)
    ctx.set_fine_rows(8)
    ctx.seed_batch(use_graph=True)
    compare(ctx.results(), ref)
    ctx.set_fine_rows(0)
    compare(stagewise(ctx, batch), ref)
    ctx.set_fine_rows(8)
    st = ctx.seed_batch(use_graph=True)
    assert st.graph_captures == 1
    compare(ctx.results(), ref)


def test_fine_rows_on_the_full_pileup_workload(ctx, reset):
    """All 16 events of the high-occupancy workload (grid 80 x 256; the
    oracle parity of the grid walk on it is test_pileup_workload_at_full_size):
    every array of the fine walks equals the grid walk's."""
    batch = events.generate(3)
    ctx.upload(batch)
    ctx.seed_batch(use_graph=True)
    base = {k: np.asarray(v).tobytes() for k, v in ctx.results().items()}
    for f in (2, 8, 16):
        ctx.set_fine_rows(f)
        st = ctx.seed_batch(use_graph=True)
        assert st.n_candidates > 5e8
        got = ctx.results()
        bad = [k for k in base if np.asarray(got[k]).tobytes() != base[k]]  # bit for bit, floats included
        assert not bad, (f, bad)


def test_invalid_fine_rows_rejected(ctx, trax_lib, reset):
    for f in (1, 3, 32):
        with pytest.raises(trax_lib.TraxError):
            ctx.set_fine_rows(f)
    assert ctx.fine_rows() == 0
