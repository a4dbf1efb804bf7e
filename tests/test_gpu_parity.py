"""GPU parity: the sm_103a chain, called through the C ABI, against the CPU oracle.

Every stage output is compared exactly (integer arrays element by element,
float arrays bit for bit): the FP32 cut predicates use the same math in the
same operation order on both sides, so exact equality is the bar.
"""
import numpy as np
import pytest

from trax_gb300 import events

pytestmark = pytest.mark.gpu

INT_ARRAYS = ["perm", "grid", "pairs", "pair_offsets", "cands", "cand_offsets", "trip_h1", "trip_h2", "trip_h3",
              "trip_offsets", "link_basis", "link_follower", "connectable", "non_connectable", "ca_states", "tracks",
              "track_offsets"]
FLOAT_ARRAYS = ["eta", "pt"]


def compare(got, ref, names=None):
    bad = []
    for name in names or (INT_ARRAYS + FLOAT_ARRAYS):
        if name not in ref:
            continue
        a, b = np.asarray(got[name]), np.asarray(ref[name])
        if name in FLOAT_ARRAYS:
            a, b = a.view(np.uint32), b.view(np.uint32)
        if a.shape != b.shape:
            bad.append(f"{name}: shape {a.shape} vs oracle {b.shape}")
        elif not np.array_equal(a, b):
            idx = np.nonzero(a != b)[0]
            bad.append(f"{name}: {idx.size} differences, first at {idx[0]}: {a[idx[0]]} vs {b[idx[0]]}")
    assert not bad, "; ".join(bad)


def stagewise(ctx, batch):
    ctx.upload(batch)
    ctx.grid_build()
    ctx.pair_gen()
    ctx.triplet_predict()
    ctx.triplet_filter()
    n_links = ctx.connectivity(batch.d_eta_cut)
    if n_links:
        ctx.circle_fit()
        ctx.cellular_automaton()
    return ctx.results()


@pytest.fixture(scope="module")
def ctx(trax_lib):
    c = trax_lib.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("config", [0, 1])
def test_stagewise_matches_oracle(ctx, oracle_lib, config):
    batch = events.generate(config)
    ref = oracle_lib.run(batch)[0]
    got = stagewise(ctx, batch)
    compare(got, ref)
    assert got["trip_h1"].size > 0


@pytest.mark.parametrize("config,n_events", [(1, 100), (2, 6)])
def test_batched_graph_matches_oracle(ctx, oracle_lib, config, n_events):
    batch = events.generate(config, n_events=n_events)
    ref = oracle_lib.run(batch)[0]
    ctx.upload(batch)
    stats = ctx.seed_batch(use_graph=True)
    got = ctx.results()
    compare(got, ref)
    assert stats.n_triplets == ref["trip_h1"].size
    assert stats.n_links == ref["link_basis"].size
    # a second replay of the captured graph gives the same arrays
    ctx.seed_batch(use_graph=True)
    compare(ctx.results(), ref)


def test_warp_tile_boundaries(ctx, oracle_lib):
    """Pair and candidate counts are scanned per warp of 32 (offsets within
    the warp plus a scan of the warp sums) and the filter flags are packed 32
    to a word: many small batches put the counts on many residues mod 32,
    including partial last words and single-pair batches."""
    residues = {"pairs": set(), "cands": set()}
    for seed in range(12):
        n_events = 1 + seed % 4
        batch = events.generate(0 if seed % 3 == 0 else 1, n_events=n_events, seed=100 + seed)
        ref = oracle_lib.run(batch)[0]
        compare(stagewise(ctx, batch), ref)
        ctx.seed_batch(use_graph=True)
        compare(ctx.results(), ref)
        residues["pairs"].add(int(ref["pairs"].shape[0]) % 32)
        residues["cands"].add(int(ref["cands"].shape[0]) % 32)
    assert len(residues["pairs"]) >= 6 and len(residues["cands"]) >= 6, residues
    # no pairs at all: only the first layer keeps its hits
    batch = events.generate(1, n_events=3, seed=7)
    keep = batch.layer == 1
    lh = batch.layer_hits.copy()
    lh[:, 1:] = 0
    sub = events._assemble({k: getattr(batch, k)[keep] for k in ("x", "y", "z", "layer", "det_id", "hit_id", "event")},
                           lh, batch)
    ref = oracle_lib.run(sub)[0]
    assert ref["pairs"].shape[0] == 0
    compare(stagewise(ctx, sub), ref)
    ctx.seed_batch(use_graph=True)
    compare(ctx.results(), ref)


def test_full_batch_equals_its_events_run_alone(ctx, oracle_lib):
    """At the benchmark's full size (1000 events, 9.7 M hits): every event's
    slice of the batched pairs, candidates, triplets and eta equals the
    oracle's results for that event alone, indices shifted by the event's
    first hit and pair (oracle/batch_slices.py), and every array -- links,
    connectable lists, pt and the CA included, which depend on the events
    grouped together -- equals the oracle run on the whole batch as one
    group.  The triplet offsets are monotone and every segment's triplets are
    sorted by (h2, h1) (non-decreasing: a pair can have several third
    hits)."""
    import os
    from oracle import batch_slices
    batch = events.generate(2)
    ctx.upload(batch)
    ctx.seed_batch(use_graph=True)
    got = ctx.results()
    refs = oracle_lib.run(batch, event_grouping=1, n_workers=os.cpu_count() or 1,
                          arrays=("pairs", "cands", "trip_h1", "trip_h2", "trip_h3", "eta"))
    res = batch_slices.compare(batch, got, refs)
    assert res["events"] == batch.n_events
    assert not res["mismatch"], res["mismatch"]
    # links, connectable lists, pt and the CA depend on the events grouped
    # together: against the oracle on the whole batch as one group
    whole = oracle_lib.run(batch)[0]
    assert batch_slices.compare_whole(got, whole) == []
    to = np.asarray(got["trip_offsets"])
    assert np.all(np.diff(to.astype(np.int64)) >= 0)
    h1, h2 = (np.asarray(got[k]).astype(np.uint64) for k in ("trip_h1", "trip_h2"))
    key = (h2 << np.uint64(32)) | h1
    seg = np.searchsorted(to, np.arange(key.size), side="right")
    same = seg[1:] == seg[:-1]
    assert np.all(key[1:][same] >= key[:-1][same])  # equal keys: one pair, several third hits


def test_batched_synced_matches_graph(ctx, oracle_lib):
    batch = events.generate(2, n_events=4)
    ctx.upload(batch)
    ctx.seed_batch(use_graph=False)
    a = ctx.results()
    ctx.seed_batch(use_graph=True)
    compare(ctx.results(), a)


def test_batched_path_is_deterministic(ctx):
    """The atomic orders inside the kernels (grid slots, queue positions,
    CA levels) decide nothing: a host-synced run and five graph replays of
    the same batch give the same arrays bit for bit, on a ttbar-like batch
    and on a pileup event."""
    import dataclasses
    for batch in (events.generate(2, n_events=40),
                  events.generate_workload(dataclasses.replace(events.workload(3), n_events=2, n_vertices=8))):
        ctx.upload(batch)
        ctx.seed_batch(use_graph=False)
        first = ctx.results()
        assert first["trip_h1"].size > 0
        for _ in range(5):
            ctx.seed_batch(use_graph=True)
            compare(ctx.results(), first)


def test_empty_layers_and_events(ctx, oracle_lib):
    batch = events.generate(1, n_events=5)
    # drop every hit of event 2 and of layer 3 in event 4
    keep = np.ones(batch.n_hits, dtype=bool)
    keep[batch.event == 2] = False
    keep[(batch.event == 4) & (batch.layer == 3)] = False
    lh = batch.layer_hits.copy()
    lh[2, :] = 0
    lh[4, 2] = 0
    sub = events._assemble({k: getattr(batch, k)[keep] for k in ("x", "y", "z", "layer", "det_id", "hit_id", "event")},
                           lh, batch)
    ref = oracle_lib.run(sub)[0]
    ctx.upload(sub)
    ctx.seed_batch(use_graph=True)
    compare(ctx.results(), ref)


def test_degenerate_hits_match_oracle(ctx, oracle_lib):
    """Hits on the edge cases of the window arithmetic (radius 0 from
    sign(0), phi = +-pi, the y axis, 0/0 TIP, duplicates, row boundaries,
    denormal and 1e-20 coordinates): stage by stage and in one graph replay."""
    from tests.test_oracle_kats import degenerate_batch
    b = degenerate_batch()
    ref = oracle_lib.run(b)[0]
    compare(stagewise(ctx, b), ref)
    ctx.upload(b)
    ctx.seed_batch(use_graph=True)
    compare(ctx.results(), ref)


def test_single_event_single_track(ctx, oracle_lib):
    batch = events.generate(0, n_events=1)
    ref = oracle_lib.run(batch)[0]
    got = stagewise(ctx, batch)
    compare(got, ref)


@pytest.mark.parametrize("n", [1, 2, 7, 2047, 2048, 2049, 4095, 4096, 4097, 123457, 4 * 1024 * 1024 + 3])
def test_prefix_sum_random(ctx, n):
    rng = np.random.default_rng(n)
    x = rng.integers(0, 1000, n, dtype=np.uint32)
    got = ctx.prefix_sum(x)
    ref = np.concatenate([[0], np.cumsum(x, dtype=np.uint64)[:-1]]).astype(np.uint32)
    assert np.array_equal(got, ref)


def test_prefix_sum_all_ones_kat(ctx):
    # trax_test.cpp:437-479: scanning 1 Mi ones must leave SIZE-1 in the last slot
    size = 1024 * 1024
    out = ctx.prefix_sum(np.ones(size, dtype=np.uint32))
    assert out[size - 1] == size - 1


def test_prefix_sum_wraps_like_uint32(ctx):
    x = np.full(10, 0x80000000, dtype=np.uint32)
    out = ctx.prefix_sum(x)
    assert out.tolist() == [(k * 0x80000000) & 0xffffffff for k in range(10)]


def test_stage_order_is_enforced(trax_lib):
    with trax_lib.Context(0) as c:
        batch = events.generate(0, n_events=2)
        c.upload(batch)
        with pytest.raises(trax_lib.TraxError) as e:
            c.pair_gen()
        assert e.value.code == 6


def test_invalid_layer_triplets_rejected(trax_lib):
    with trax_lib.Context(0) as c:
        batch = events.generate(0, n_events=1)
        bad = [events.LayerTriplet(2, 3, 4, 0.01, 0.037, 0.05, 0.032, 1.0, 2, 10.0, 2, 4)]
        with pytest.raises(trax_lib.TraxError) as e:
            c.set_layer_triplets(bad, batch.min_pt)
        assert e.value.code == 2


def test_hits_outside_grid_rejected(trax_lib):
    with trax_lib.Context(0) as c:
        batch = events.generate(0, n_events=1)
        batch.z[0] = np.float32(450.0)
        c.upload(batch)
        with pytest.raises(trax_lib.TraxError) as e:
            c.grid_build()
        assert e.value.code == 5


def _kat_batch():
    from tests.test_oracle_kats import load_kat
    kat, cols, t = load_kat()
    n_layers = int(cols["layer"].max())
    lh = np.bincount(cols["layer"] - 1, minlength=n_layers).astype(np.uint32).reshape(1, n_layers)
    w = events.workload(2)
    lts = [events.LayerTriplet(p + 1, p + 2, p + 3, 0.01, 0.037, 0.05, 0.032, 1.0, 2, 10.0, 2, 4)
           for p in range(kat["n_layer_triplets"])]
    proto = events.EventBatch(x=None, y=None, z=None, layer=None, det_id=None, hit_id=None, event=None,
                              event_offsets=None, layer_hits=None, layer_offsets=None,
                              min_r=np.asarray(w.radii[:n_layers], np.float32) - 0.1,
                              max_r=np.asarray(w.radii[:n_layers], np.float32) + 0.1, lts=lts, n_z=20, n_phi=20,
                              min_pt=1.0, d_eta_cut=kat["d_eta_cut"])
    cols = dict(cols, det_id=np.zeros_like(cols["layer"]), hit_id=np.zeros_like(cols["layer"]))
    return kat, events._assemble(cols, lh, proto), t


@pytest.mark.parametrize("shuffle", [False, True])
def test_tight_connectivity_kat_gpu(ctx, oracle_lib, shuffle):
    # TripletConnectivityTest.h:66-94 through trax_set_tracklets + the linking stages
    kat, batch, t = _kat_batch()
    if shuffle:  # unsorted segments: the connectivity scans like the reference
        rng = np.random.default_rng(3)
        t = np.concatenate([t[4 * p:4 * p + 4][rng.permutation(4)] for p in range(4)])
    ref = oracle_lib.link(batch.x, batch.y, batch.z, batch.layer, batch.event, t[:, 0], t[:, 1], t[:, 2], 1,
                          kat["n_layer_triplets"], kat["d_eta_cut"])
    ctx.upload(batch)
    ctx.set_tracklets(t[:, 0], t[:, 1], t[:, 2])
    assert ctx.connectivity(kat["d_eta_cut"]) == 3
    ctx.circle_fit()
    ctx.cellular_automaton()
    got = ctx.results()
    compare(got, ref, ["link_basis", "link_follower", "connectable", "non_connectable", "ca_states", "tracks",
                       "track_offsets", "eta", "pt"])
    if not shuffle:
        assert np.stack([got["link_basis"], got["link_follower"]], 1).tolist() == kat["expected"]["links"]
        assert got["ca_states"].tolist() == kat["expected"]["ca_states"]


def test_config0_golden_gpu(ctx):
    from tests.test_oracle_kats import golden_batch
    b, d = golden_batch()
    got = stagewise(ctx, b)
    for k in ("grid", "perm", "pairs", "cands", "trip_h1", "trip_h2", "trip_h3", "trip_offsets"):
        assert np.array_equal(got[k], d["oracle_" + k]), k


def test_pileup_stress_event_matches_oracle(ctx, oracle_lib):
    """The high-occupancy workload's event shape (vertices of 1000 tracks plus
    noise, 10 layers, 6 layer triplets, grid 80 x 256), cut to three vertices
    so that the oracle finishes in seconds."""
    import dataclasses
    w = dataclasses.replace(events.workload(3), n_events=2, n_vertices=6)
    batch = events.generate_workload(w)
    ref = oracle_lib.run(batch)[0]
    ctx.upload(batch)
    ctx.seed_batch(use_graph=True)
    compare(ctx.results(), ref)


def test_grid_build_hit_arrays_outside_shared_memory(ctx, oracle_lib):
    """The grid build keeps each hit's cell, phi and slot in shared memory
    when the largest layer fits beside the cell counters.  Two ways past it:
    a grid whose counters leave no room (every layer in global scratch), and
    a replay of a graph captured for a smaller largest layer (the layers
    that do not fit fall back one by one)."""
    batch = events.generate(1, n_events=20)
    lh = batch.layer_hits
    # the event whose first two layers together outnumber every single layer
    e = int(np.argmax(lh[:, 0] + lh[:, 1]))
    assert lh[e, 0] + lh[e, 1] > lh.max()
    merged = events.generate(1, n_events=20)
    in_e = merged.event == e
    merged.layer = np.where(in_e & (merged.layer == 2), 1, merged.layer).astype(merged.layer.dtype)
    mlh = merged.layer_hits.copy()
    mlh[e, 0] += mlh[e, 1]
    mlh[e, 1] = 0
    merged = events._assemble({k: getattr(merged, k) for k in ("x", "y", "z", "layer", "det_id", "hit_id", "event")},
                              mlh, merged)
    ref = oracle_lib.run(merged)[0]
    ctx.upload(batch)
    ctx.seed_batch(use_graph=True)
    ctx.upload(merged)
    ctx.seed_batch(use_graph=True)
    compare(ctx.results(), ref)
    # 401 x 129 cells: 207 KB of counters, no room for a layer of 2747 hits
    dense = events.generate(2, n_events=2, seed=4)
    dense.n_z, dense.n_phi = 400, 128
    assert dense.layer_hits.max() * 12 > 227 * 1024 - 256 - 401 * 129 * 4
    ref = oracle_lib.run(dense)[0]
    ctx.upload(dense)
    ctx.seed_batch(use_graph=True)
    compare(ctx.results(), ref)


def test_layer_beyond_16bit_grid_counters(ctx, oracle_lib):
    """The grid build counts in 16-bit halves while every layer has fewer
    than 65 536 hits; a layer of 71 216 hits (on layer 10, which no layer
    triplet uses) takes the 32-bit build with its per-hit arrays in global
    scratch, in the synced path and in a captured graph."""
    b = events.generate(2, n_events=2, seed=4)
    rng = np.random.default_rng(9)
    n_add = 70000
    phi = rng.uniform(-np.pi, np.pi, n_add)
    new = {"x": (78.0 * np.cos(phi)).astype(np.float32), "y": (78.0 * np.sin(phi)).astype(np.float32),
           "z": rng.uniform(-100, 100, n_add).astype(np.float32), "layer": np.full(n_add, 10, np.uint32),
           "det_id": np.zeros(n_add, np.uint32), "hit_id": np.arange(n_add, dtype=np.uint32) + 10 ** 6,
           "event": np.zeros(n_add, np.uint32)}
    end0 = int(b.event_offsets[1])  # event 0 ends with its layer-10 hits
    cols = {k: np.concatenate([getattr(b, k)[:end0], new[k].astype(getattr(b, k).dtype), getattr(b, k)[end0:]])
            for k in new}
    lh = b.layer_hits.copy()
    lh[0, 9] += n_add
    big = events._assemble(cols, lh, b)
    assert big.layer_hits.max() > 0xffff
    ref = oracle_lib.run(big)[0]
    compare(stagewise(ctx, big), ref)
    ctx.seed_batch(use_graph=True)
    compare(ctx.results(), ref)


@pytest.mark.parametrize("config,n_events", [(2, 40), (3, 2)])
def test_track_evaluation_on_the_device(ctx, config, n_events):
    """trax_physics_tracks_device (track extraction, clone removal over the
    components of shared hits, real / fake / distinct tracks on the device)
    equals the host's list-based evaluation of the same CA output, on ttbar-like
    events and on the pileup events, where clones share hits densely."""
    import dataclasses
    from trax_gb300 import physics
    if config == 3:
        batch = events.generate_workload(dataclasses.replace(events.workload(3), n_events=n_events, n_vertices=6))
    else:
        batch = events.generate(config, n_events=n_events)
    ctx.upload(batch)
    ctx.seed_batch(use_graph=True)
    got = ctx.results()
    hid = batch.hit_id[got["perm"]]
    host = physics.track_metrics(got["tracks"], got["track_offsets"], got["trip_h1"], got["trip_h2"],
                                 got["trip_h3"], hid, 1000)
    device = physics.track_metrics_device(ctx, 1000)
    assert device == host
    assert host["total"] > 0 and host["filtered"] < host["total"]


def test_capacity_overflow_recalibrates(ctx, oracle_lib):
    """A batch of the same shape but far denser hits overflows the capacities
    calibrated on the first: the call recalibrates, recaptures and returns the
    exact result (admission never truncates)."""
    sparse = events.generate(1, n_events=20)
    ctx.upload(sparse)
    calibrated = ctx.seed_batch(use_graph=True)
    dense = events.generate(1, n_events=20)
    rng = np.random.default_rng(5)
    r = np.hypot(dense.x, dense.y)
    phi = rng.uniform(-0.3, 0.3, r.size)  # every hit into one narrow phi wedge
    dense.x = (r * np.cos(phi)).astype(np.float32)
    dense.y = (r * np.sin(phi)).astype(np.float32)
    ref = oracle_lib.run(dense)[0]
    ctx.upload(dense)
    st = ctx.seed_batch(use_graph=True)
    assert st.n_pairs > 2 * calibrated.n_pairs  # beyond the calibrated headroom
    compare(ctx.results(), ref)


def test_pileup_workload_at_full_size(ctx, oracle_lib):
    """The high-occupancy workload at full size (16 events x 20 vertices x 1000
    tracks, about 125 000 hits per event, grid 80 x 256; 176 M pairs, 735 M
    candidates) in one CUDA-graph replay: every array equals the oracle run on
    the whole batch as one group (its connectivity through an index of the
    triplets -- the same result as the reference's scan, which is quadratic
    in segments of 290 000 triplets), on all host cores; the triplet offsets
    are monotone and every segment's triplets sorted by (h2, h1)."""
    import os
    from oracle import batch_slices
    batch = events.generate(3)
    ctx.upload(batch)
    st = ctx.seed_batch(use_graph=True)
    assert st.graph_captures == 1 and st.n_candidates > 5e8
    got = ctx.results()
    whole = oracle_lib.run(batch, n_workers=os.cpu_count() or 1, links="indexed")[0]
    assert batch_slices.compare_whole(got, whole) == []
    assert np.array_equal(got["grid"], whole["grid"]) and np.array_equal(got["perm"], whole["perm"])
    to = np.asarray(got["trip_offsets"])
    assert np.all(np.diff(to.astype(np.int64)) >= 0)
    h1, h2 = (np.asarray(got[k]).astype(np.uint64) for k in ("trip_h1", "trip_h2"))
    key = (h2 << np.uint64(32)) | h1
    seg = np.searchsorted(to, np.arange(key.size), side="right")
    same = seg[1:] == seg[:-1]
    assert np.all(key[1:][same] >= key[:-1][same])
