"""The linking stages on the caller's inputs, through the C ABI.

TrackletCircleFitter::run takes a validIdx list (TrackletCircleFitter.h:25-29)
and CellularAutomaton::run takes basis, follower and pt arrays
(CellularAutomaton.h:43-49); the context computes on what it is given:
trax_circle_fit_on and trax_cellular_automaton_on.  The CA is checked against
the oracle's CA on link sets unlike the chain's own (levels skipped, several
bases per follower, repeated links, ties of |dpt|), whose oracle the CPU
tests pin to the reference's own kernels.
"""
import numpy as np
import pytest

from trax_gb300 import events

pytestmark = pytest.mark.gpu


@pytest.fixture
def ctx(trax_lib):
    with trax_lib.Context(0) as c:
        yield c


@pytest.mark.parametrize("seed", [1, 3, 5])
def test_ca_on_random_link_sets_matches_oracle(ctx, oracle_lib, seed):
    from tests.ca_cases import random_links
    b, f, pt = random_links(seed)
    states, tracks, offsets = ctx.cellular_automaton_on(b, f, pt)
    o = oracle_lib.ca(pt.size, b, f, pt)
    assert np.array_equal(states, o["ca_states"])
    assert np.array_equal(offsets, o["track_offsets"])
    assert np.array_equal(tracks, o["tracks"])


def test_ca_on_chain_links_equals_the_chain(ctx):
    """The chain's own links and pt fed back in give the chain's own CA result."""
    batch = events.generate(1, n_events=20)
    ctx.upload(batch)
    ctx.seed_batch(use_graph=False)
    want = ctx.tracks()
    b, f, _, _ = ctx.links()
    _, pt = ctx.eta_pt()
    got = ctx.cellular_automaton_on(b, f, pt)
    for w, g in zip(want, got):
        assert np.array_equal(w, g)


def test_ca_on_rejects_a_cycle(ctx, trax_lib):
    b = np.array([0, 1, 2], np.uint32)
    f = np.array([1, 2, 0], np.uint32)
    with pytest.raises(trax_lib.TraxError) as e:
        ctx.cellular_automaton_on(b, f, np.ones(3, np.float32))
    assert e.value.code == 2


def test_circle_fit_on_a_caller_list(ctx, oracle_lib):
    """The fit of a caller's subset equals the chain's fit on it, 0 elsewhere."""
    batch = events.generate(1, n_events=10)
    ctx.upload(batch)
    ctx.seed_batch(use_graph=False)
    ref = oracle_lib.run(batch)[0]
    _, pt_chain = ctx.eta_pt()
    conn = ref["connectable"]
    assert np.array_equal(pt_chain[conn].view(np.uint32), ref["pt"][conn].view(np.uint32))
    rng = np.random.default_rng(0)
    sub = np.sort(rng.choice(conn, conn.size // 3, replace=False))
    pt = ctx.circle_fit_on(sub)
    assert np.array_equal(pt[sub].view(np.uint32), pt_chain[sub].view(np.uint32))
    rest = np.setdiff1d(np.arange(pt.size), sub)
    assert np.all(pt[rest] == 0)
    # any triplet may be listed, connectable or not
    pt_all = ctx.circle_fit_on(np.arange(pt.size))
    assert np.array_equal(pt_all[conn].view(np.uint32), pt_chain[conn].view(np.uint32))
