"""The oracle against the reference's own kernel text (CPU, no GPU).

``oracle/_ref/libtraxref.so`` runs the OpenCL C of the reference's
KERNEL_CLASS blocks -- grid build, the recursive prefix sum, pair generation,
prediction, filter, connectivity, circle fit and cellular automaton -- copied
by ``oracle/ref_extract.py`` and driven by the reference's host-side
sequences (``oracle/ref_driver.cpp``).  These tests compare it with the
oracle, which the GPU path is compared with element by element, so that the
bit-exact claims of the GPU tests rest on the reference's own code.

With one work-item per (event, layer) and per (event, layer pair) the
reference's atomic slot order is the input order, and its arrays must equal
the oracle's element for element.  With more work-items the reference's
arrays come out in another order (grid slots by atomic order, pairs by
work-item), and the sets keyed by hit identity must be equal.

The library is built only where the reference's sources are present; the
tests skip elsewhere.
"""
import dataclasses

import numpy as np
import pytest

from oracle import oracle, ref
from trax_gb300 import events

pytestmark = pytest.mark.skipif(not ref.available(), reason="reference sources absent: oracle/_ref not built")

LINK_ARRAYS = ("link_basis", "link_follower", "connectable", "non_connectable", "ca_states", "ca_best",
               "tracks", "track_offsets")


def assert_identical(batch, r, o):
    """Element-for-element equality of the reference run `r` and the oracle run `o`."""
    perm = o["perm"]
    for col, src, dt in (("hx", batch.x, np.float32), ("hy", batch.y, np.float32), ("hz", batch.z, np.float32),
                         ("hlayer", batch.layer, np.uint32), ("hdet", batch.det_id, np.uint32),
                         ("hhit", batch.hit_id, np.uint32), ("hevt", batch.event, np.uint32)):
        assert np.array_equal(r[col].view(np.uint32), np.asarray(src, dt)[perm].view(np.uint32)), col
    for name in ("grid", "pairs", "pair_offsets", "cand_offsets", "trip_h1", "trip_h2", "trip_h3",
                 "trip_offsets"):
        assert np.array_equal(r[name], o[name]), name
    # candidates: slots the reference never writes (the two rOrigin roundings)
    # hold the appended hit in the reference run and 0xffffffff in the oracle
    rc, oc = r["cands"].reshape(-1, 2), o["cands"].reshape(-1, 2)
    assert rc.shape == oc.shape
    undefined = rc[:, 1] == batch.n_hits
    assert int(undefined.sum()) == r["stats_dict"]["cand_sentinels"]
    assert np.all(oc[undefined, 1] == 0xFFFFFFFF)
    assert np.array_equal(rc[~undefined], oc[~undefined])
    assert r["stats_dict"]["pair_sentinels"] == o["stats_dict"]["pair_dup_slots"]
    assert np.array_equal(r["eta"].view(np.uint32), o["eta"].view(np.uint32))
    if r["stats_dict"]["no_links"]:
        # the reference returns null pointers (TripletConnectivityTight.cpp:127-129)
        for name in LINK_ARRAYS:
            assert name not in r and o[name].size == 0, name
        return
    assert r["stats_dict"]["ca_chain_broken"] == 0
    for name in LINK_ARRAYS:
        assert np.array_equal(r[name], o[name]), name
    c = o["connectable"]
    assert np.array_equal(r["pt"][c].view(np.uint32), o["pt"][c].view(np.uint32))


def both(batch, n_threads=1, local_mem=ref.GTX660_LOCAL_MEM):
    return ref.run(batch, n_threads=n_threads, local_mem=local_mem), oracle.run(batch)[0]


# ------------------------------------------------------------- prefix sum
@pytest.mark.parametrize("wg", [1, 16, 128, 256])
def test_reference_scan_all_ones_kat(wg):
    """KAT #1 (trax_test.cpp:437-479): the reference's scan of n ones gives out[n-1] == n-1."""
    n = 1 << 16
    out = ref.prefix_sum(np.ones(n, np.uint32), wg)
    assert out[n - 1] == n - 1
    assert np.array_equal(out, np.arange(n, dtype=np.uint32))


@pytest.mark.parametrize("n,wg", [(1, 1), (2, 1), (1000, 1), (4097, 64), (100003, 128), (70000, 256)])
def test_reference_scan_matches_numpy_and_oracle(n, wg):
    rng = np.random.default_rng(n)
    data = rng.integers(0, 1 << 20, n, dtype=np.uint32)
    expect = np.zeros(n, np.uint64)
    expect[1:] = np.cumsum(data[:-1], dtype=np.uint64)
    expect = (expect & 0xFFFFFFFF).astype(np.uint32)  # uint32 wrap-around
    got = ref.prefix_sum(data, wg)
    assert np.array_equal(got, expect)
    assert np.array_equal(got, oracle.prefix_sum_blelloch(data, wg))


# ------------------------------------------------- the chain, element for element
@pytest.mark.parametrize("local_mem", [ref.GTX660_LOCAL_MEM, 0])
@pytest.mark.parametrize("config", [0, 1])
def test_configs_0_and_1_identical(config, local_mem):
    """Both local-memory choices of GridBuilder.cpp:17-140 and PairGeneratorBeamspot.cpp:46-88."""
    batch = events.generate(config)
    r, o = both(batch, local_mem=local_mem)
    expect_local = int(local_mem > 4 * (batch.n_z + 1) * (batch.n_phi + 1))
    assert r["stats_dict"]["grid_count_local"] == expect_local
    assert r["stats_dict"]["pair_count_local"] == expect_local
    assert_identical(batch, r, o)


def test_config2_twenty_events_identical():
    """20 ttbar-like events of the benchmark workload (10 layers, 6 layer triplets)."""
    batch = events.generate(2, n_events=20)
    r, o = both(batch)
    assert len(r["link_basis"]) > 10000 and r["stats_dict"]["ca_iterations"] > 2
    assert_identical(batch, r, o)


def test_reference_ttbar_events_identical():
    """The reference's own 10 ttbar events (hits.ttBar.pb, as its loader hands them over)."""
    from tests.test_eventio import ttbar_fixture
    batch = ttbar_fixture()[0]
    r, o = both(batch)
    assert len(r["trip_h1"]) > 100
    assert_identical(batch, r, o)


def test_degenerate_batch_identical():
    """Hits on the edges of the window arithmetic (phi = +-pi, inner hits with y = 0, the y
    axis, 0/0 TIP, duplicated hits, row boundaries, denormals, tiny radii).  Outer hits on
    the x axis are left out: the reference reads about 2^32 cells past its grid there."""
    from tests.test_oracle_kats import degenerate_batch
    batch = degenerate_batch(x_axis_outer_hits=False)
    for local_mem in (ref.GTX660_LOCAL_MEM, 0):
        r, o = both(batch, local_mem=local_mem)
        assert_identical(batch, r, o)


def test_pileup_event_identical():
    """The high-occupancy event shape (grid 80 x 256: larger than the local memory, so the
    no-local-memory kernels), cut to six vertices."""
    w = dataclasses.replace(events.workload(3), n_events=1, n_vertices=6)
    batch = events.generate_workload(w)
    r, o = both(batch)
    assert r["stats_dict"]["grid_count_local"] == 0
    assert_identical(batch, r, o)


def test_empty_layers_identical():
    """Events with empty layers and an event with no hits on the first layer triplet."""
    b = events.generate(1, n_events=3)
    keep = ~(((b.event == 0) & (b.layer == 2)) | ((b.event == 2) & (b.layer == 1)))
    cols = {k: getattr(b, k)[keep] for k in ("x", "y", "z", "layer", "det_id", "hit_id", "event")}
    lh = b.layer_hits.copy()
    lh[0, 1] = 0
    lh[2, 0] = 0
    batch = events._assemble(cols, lh, b)
    r, o = both(batch)
    assert_identical(batch, r, o)


# ------------------------------------------------- more work-items: equal sets
def _canonical(res, orig):
    """Sets keyed by original hit index: pairs, candidates, triplets, links, CA states."""
    pairs = res["pairs"].reshape(-1, 2).astype(np.int64)
    P = orig[pairs]
    cands = res["cands"].reshape(-1, 2).astype(np.int64)
    C = np.stack([P[cands[:, 0], 0], P[cands[:, 0], 1], orig[cands[:, 1]]], axis=1)
    T = np.stack([orig[res["trip_h1"]], orig[res["trip_h2"]], orig[res["trip_h3"]]], axis=1)
    key = [tuple(t) for t in T.tolist()]
    out = {
        "pairs": sorted(map(tuple, P.tolist())),
        "cands": sorted(map(tuple, C.tolist())),
        "triplets": sorted(key),
        "eta": sorted(zip(key, res["eta"].view(np.uint32).tolist())),
    }
    if "link_basis" in res:
        out["links"] = sorted((key[b], key[f]) for b, f in zip(res["link_basis"], res["link_follower"]))
        out["states"] = sorted(zip(key, res["ca_states"].tolist()))
    return out


@pytest.mark.parametrize("n_threads", [32, 256])
def test_work_group_sizes_give_the_same_sets(n_threads):
    """exec.threads changes the reference's array order (atomic slot order in the grid,
    pairs by work-item), not the sets.  det_id carries the input index through the
    grid build; no kernel reads it."""
    b = events.generate(1, n_events=8)
    batch = dataclasses.replace(b, det_id=np.arange(b.n_hits, dtype=np.uint32))
    r = ref.run(batch, n_threads=n_threads)
    o = oracle.run(batch)[0]
    if n_threads == 32:  # fewer work-items than hits per layer: another slot order in the cells
        assert not np.array_equal(r["hdet"], o["perm"])
    cr, co = _canonical(r, r["hdet"].astype(np.int64)), _canonical(o, o["perm"].astype(np.int64))
    assert cr.keys() == co.keys()
    for k in cr:
        assert cr[k] == co[k], k
    assert np.array_equal(r["pair_offsets"], o["pair_offsets"])
    assert np.array_equal(r["trip_offsets"], o["trip_offsets"])


# ------------------------------------------------- the CA alone, any link set
@pytest.mark.parametrize("seed,sort_by_basis,n_threads", [(1, True, 1), (2, False, 1), (3, True, 64),
                                                          (4, False, 256)])
def test_ca_on_random_link_sets_identical(seed, sort_by_basis, n_threads):
    """CellularAutomaton::run on links that skip levels, with many bases per follower,
    repeated links and ties of |dpt|: the reference's kernels and the oracle agree."""
    from tests.ca_cases import random_links
    b, f, pt = random_links(seed, sort_by_basis=sort_by_basis)
    n = pt.size
    r = ref.ca(n, b, f, pt, n_threads=n_threads)
    o = oracle.ca(n, b, f, pt)
    assert r["stats_dict"]["ca_chain_broken"] == 0 and o["stats_dict"]["ca_capped"] == 0
    assert r["stats_dict"]["ca_iterations"] == o["stats_dict"]["ca_iterations"] > 3
    for name in ("ca_states", "ca_best", "tracks", "track_offsets"):
        assert np.array_equal(r[name], o[name]), name
