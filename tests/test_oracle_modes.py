"""The oracle's faster modes give its literal results (CPU, no GPU).

Two options make the oracle usable on the largest workloads:
* n_workers host threads inside one event group: every stage loop runs in
  chunks whose outputs are disjoint, so nothing depends on their number;
* links="indexed": connectivity finds each basis's followers through an
  index of the triplets by (first, second) hit instead of the reference's
  linear scan of the follower segment -- the same followers in the same order.
Both are checked against the serial, literal oracle, which the tests in
test_ref_kernels.py pin to the reference's own kernels.
"""
import numpy as np
import pytest

from oracle import oracle
from trax_gb300 import events


def _batches():
    from tests.test_oracle_kats import degenerate_batch
    yield "config 1", events.generate(1)
    yield "config 2, 30 events", events.generate(2, n_events=30)
    yield "degenerate", degenerate_batch()


@pytest.mark.parametrize("which", [0, 1, 2])
def test_threads_and_indexed_links_give_the_literal_results(which):
    name, batch = list(_batches())[which]
    lit = oracle.run(batch)[0]
    for kw in ({"n_workers": 8}, {"links": "indexed"}, {"n_workers": 8, "links": "indexed"}):
        got = oracle.run(batch, **kw)[0]
        for k, v in lit.items():
            if k == "stats_dict":
                continue
            assert np.array_equal(got[k].view(np.uint32), v.view(np.uint32)), (name, kw, k)


def test_links_none_stops_after_the_filter():
    batch = events.generate(1, n_events=10)
    lit = oracle.run(batch)[0]
    got = oracle.run(batch, links="none")[0]
    for k in ("pairs", "cands", "trip_h1", "trip_h2", "trip_h3", "trip_offsets"):
        assert np.array_equal(got[k], lit[k]), k
    assert got["link_basis"].size == 0 and got["tracks"].size == 0
