"""The CPU oracle against the reference's own known answers and invariants.

The reference's build cannot run here (its OpenCL wrapper submodule is empty,
no OpenCL runtime), so the oracle is pinned by what the reference's tests and
checks state: the prefix-sum self-check of trax_test, the tight
connectivity fixture of TripletConnectivityTest, the grid verification of
GridBuilder::verifyGrid, plus closed-form properties of each stage.
"""
import json
import os

import numpy as np
import pytest

from trax_gb300 import events

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_prefix_sum_all_ones_kat(oracle_lib):
    # trax_test.cpp:437-479: scan 1 Mi ones for every work-group size, out[SIZE-1] == SIZE-1
    size = 1024 * 1024
    ones = np.ones(size, dtype=np.uint32)
    wg = 1
    while wg <= 256:
        out = oracle_lib.prefix_sum_blelloch(ones, wg)
        assert out[size - 1] == size - 1, wg
        wg <<= 1


@pytest.mark.parametrize("n,wg", [(1, 1), (2, 1), (7, 4), (255, 64), (256, 128), (257, 128), (100003, 256),
                                  (1 << 20, 32)])
def test_prefix_sum_matches_exclusive_scan(oracle_lib, n, wg):
    rng = np.random.default_rng(n)
    x = rng.integers(0, 1 << 31, n, dtype=np.uint32)  # wraps, like uint in OpenCL
    out = oracle_lib.prefix_sum_blelloch(x, wg)
    ref = np.concatenate([[0], np.cumsum(x.astype(np.uint64))[:-1]]).astype(np.uint64) & 0xffffffff
    assert np.array_equal(out.astype(np.uint64), ref)


def load_kat():
    with open(os.path.join(GOLD, "connectivity_kat.json")) as f:
        kat = json.load(f)
    hits = kat["hits"]
    cols = {k: np.array([h[k] for h in hits], dtype=np.float32) for k in ("x", "y", "z")}
    cols["layer"] = np.array([h["layer"] for h in hits], dtype=np.uint32)
    cols["event"] = np.zeros(len(hits), dtype=np.uint32)
    t = np.array(kat["triplets"], dtype=np.uint32)
    return kat, cols, t


def test_tight_connectivity_kat_oracle(oracle_lib):
    # TripletConnectivityTest.h:66-94 + :233-258: the chain links into one track of 4 triplets
    kat, cols, t = load_kat()
    r = oracle_lib.link(cols["x"], cols["y"], cols["z"], cols["layer"], cols["event"], t[:, 0], t[:, 1], t[:, 2],
                        1, kat["n_layer_triplets"], kat["d_eta_cut"])
    links = np.stack([r["link_basis"], r["link_follower"]], axis=1).tolist()
    assert links == kat["expected"]["links"]
    assert r["ca_states"].tolist() == kat["expected"]["ca_states"]
    off = r["track_offsets"]
    tracks = [r["tracks"][off[i]:off[i + 1]].tolist() for i in range(len(off) - 1) if off[i + 1] > off[i]]
    assert kat["expected"]["chain_track"] in tracks
    assert sum(len(x) >= 3 for x in tracks) == 1  # the host keeps tracks of >= 3 triplets


def golden_batch():
    d = np.load(os.path.join(GOLD, "config0_golden.npz"))
    w = events.workload(0)
    b = events.EventBatch(x=d["x"], y=d["y"], z=d["z"], layer=d["layer"], det_id=d["det_id"], hit_id=d["hit_id"],
                          event=d["event"], event_offsets=d["event_offsets"], layer_hits=d["layer_hits"],
                          layer_offsets=d["layer_offsets"], min_r=d["min_r"], max_r=d["max_r"], lts=w.lts,
                          n_z=w.n_z, n_phi=w.n_phi, min_pt=w.min_pt, d_eta_cut=w.d_eta_cut, workload=w)
    return b, d


def test_config0_golden_fixture(oracle_lib):
    b, d = golden_batch()
    r = oracle_lib.run(b)[0]
    for k in ("grid", "perm", "pairs", "cands", "trip_h1", "trip_h2", "trip_h3", "trip_offsets"):
        assert np.array_equal(r[k], d["oracle_" + k]), k


@pytest.fixture(scope="module")
def config1(oracle_lib):
    b = events.generate(1, n_events=30)
    return b, oracle_lib.run(b)[0]


def test_grid_verification(config1):
    # GridBuilder::verifyGrid (GridBuilder.cpp:188-225): every hit of a cell lies in its z/phi bounds and layer
    b, r = config1
    C = (b.n_z + 1) * (b.n_phi + 1)
    sz = np.float32(600.0) / np.float32(b.n_z)
    sp = np.float32(np.float32(np.pi) * 2) / np.float32(b.n_phi)
    perm = r["perm"]
    x, y, z, lay = b.x[perm], b.y[perm], b.z[perm], b.layer[perm]
    phi = np.arctan2(y.astype(np.float64), x.astype(np.float64))
    grid = r["grid"].reshape(b.n_events, b.n_layers, C)
    for e in range(b.n_events):
        for l in range(b.n_layers):
            g = grid[e, l]
            for zc in range(b.n_z):
                for pc in range(b.n_phi):
                    c = zc * (b.n_phi + 1) + pc
                    lo, hi = g[c], g[c + 1]
                    if hi <= lo:
                        continue
                    sl = slice(lo, hi)
                    assert np.all(lay[sl] == l + 1)
                    assert np.all(z[sl] >= -300 + zc * sz - 1e-3) and np.all(z[sl] <= -300 + (zc + 1) * sz + 1e-3)
                    assert np.all(phi[sl] >= -np.pi + pc * sp - 1e-5) and np.all(phi[sl] <= -np.pi + (pc + 1) * sp + 1e-5)
    # cell order is stable: inside a cell the hits keep their input order
    for e in range(b.n_events):
        for l in range(b.n_layers):
            g = grid[e, l]
            for c in range(C - 1):
                seg = perm[g[c]:g[c + 1]]
                assert np.all(np.diff(seg.astype(np.int64)) > 0)


def test_stage_invariants(config1):
    b, r = config1
    perm = r["perm"]
    layer = b.layer[perm]
    event = b.event[perm]
    lts = b.lts
    pairs = r["pairs"].reshape(-1, 2)
    ok = pairs[:, 0] != 0xffffffff
    pl = layer[pairs[ok, 1]] - 1  # outer hit layer -> layer triplet via layer2
    # pairs: inner on layer1, outer on layer2 of their layer triplet, same event
    lt_of = {lt.layer2: i for i, lt in enumerate(lts)}
    for (inner, outer) in pairs[ok][:5000]:
        p = lt_of[layer[outer]]
        assert layer[inner] == lts[p].layer1 and event[inner] == event[outer]
    assert pl.size == ok.sum()
    # candidates: third hit on layer3 of the pair's layer triplet
    cands = r["cands"].reshape(-1, 2)
    good = cands[:, 1] != 0xffffffff
    for (pi, h3) in cands[good][:5000]:
        inner = pairs[pi, 0]
        p = layer[inner] - 1
        assert layer[h3] == lts[p].layer3 and event[h3] == event[inner]
    # triplets are candidates (as hit triples), in candidate order
    tri = np.stack([r["trip_h1"], r["trip_h2"], r["trip_h3"]], axis=1)
    cand_hits = np.stack([pairs[cands[good, 0], 0], pairs[cands[good, 0], 1], cands[good, 1]], axis=1)
    ci = 0
    for t in tri:
        while ci < len(cand_hits) and not np.array_equal(cand_hits[ci], t):
            ci += 1
        assert ci < len(cand_hits)
        ci += 1
    # links share two hits and pass the eta cut
    bb, ff, eta = r["link_basis"], r["link_follower"], r["eta"]
    assert np.all(tri[ff, 0] == tri[bb, 1]) and np.all(tri[ff, 1] == tri[bb, 2])
    assert np.all(np.abs(eta[bb] - eta[ff]) < np.float32(b.d_eta_cut))


def test_ca_states_are_longest_chains(config1):
    # the CA forward phase converges to the longest chain of links ending at each triplet
    b, r = config1
    n = r["trip_h1"].size
    best = np.ones(n, dtype=np.int64)
    order = np.argsort(r["link_follower"], kind="stable")
    changed = True
    while changed:  # Bellman-Ford style relaxation, independent of the oracle's scheme
        changed = False
        for p in order:
            bb, ff = r["link_basis"][p], r["link_follower"][p]
            if best[bb] + 1 > best[ff]:
                best[ff] = best[bb] + 1
                changed = True
    assert np.array_equal(best, r["ca_states"].astype(np.int64))
    # every track walks best bases with strictly decreasing state
    off, tr, st = r["track_offsets"], r["tracks"], r["ca_states"]
    for i in range(n):
        seg = tr[off[i]:off[i + 1]]
        if seg.size:
            assert seg[0] == i and seg.size == st[i]
            assert np.all(np.diff(st[seg].astype(np.int64)) == -1)


def test_event_grouping_only_moves_boundary_quirks(oracle_lib):
    # per-event groups and one big group give the same triplets (keyed by input hit index)
    b = events.generate(1, n_events=6)
    one = oracle_lib.run(b)[0]
    per = oracle_lib.run(b, event_grouping=1)

    def keyed(r):
        p = r["perm"]
        return set(zip(p[r["trip_h1"]].tolist(), p[r["trip_h2"]].tolist(), p[r["trip_h3"]].tolist()))

    assert keyed(one) == set().union(*[keyed(r) for r in per])


def test_config0_finds_most_muons(oracle_lib):
    b = events.generate(0)
    r = oracle_lib.run(b)[0]
    perm = r["perm"]
    tid = b.hit_id[perm]
    ev = b.event[perm]
    found = set()
    for a, c, d in zip(r["trip_h1"], r["trip_h2"], r["trip_h3"]):
        if tid[a] and tid[a] == tid[c] == tid[d]:
            found.add((int(ev[a]), int(tid[a])))
    # a track is findable when all three layers have its hit
    lay = b.layer
    findable = {(int(e), int(t)) for e, t in set(zip(b.event.tolist(), b.hit_id.tolist())) if t
                and len({int(l) for l in lay[(b.event == e) & (b.hit_id == t)]}) == 3}
    assert len(found & findable) >= 0.9 * len(findable)


def degenerate_batch(x_axis_outer_hits: bool = True):
    """Two config-1 events with hits moved onto the edge cases of the
    reference's window arithmetic: outer hits on the x axis (sign(y) = 0 gives
    radius 0 and NaN/inf windows, PairGeneratorBeamspot.h:111-112), phi = +pi
    and -pi exactly (the overflow phi column, TripletThetaPhiPredictor.h:193),
    the y axis, an outer hit at the inner hit's transverse point (0/0 in the
    prediction's TIP), a duplicated third-layer hit, z on the first row and on
    a row boundary, a denormal y, and outer radii of 1e-20 and 1e-3.

    x_axis_outer_hits=False leaves out the hits on the x axis of the layers
    that are outer layers of a pair (2 and 3): their infinite phi windows make
    the reference read grid cells about 2^32 past the layer, where its result
    is undefined (the oracle and the GPU clamp to the layer's last cell)."""
    b = events.generate(1, n_events=2)
    x, y, z = b.x.copy(), b.y.copy(), b.z.copy()
    f = np.float32

    def idx(e, l, k):
        return int(np.nonzero((b.event == e) & (b.layer == l))[0][k])

    def rad(i):
        return f(np.hypot(x[i], y[i]))

    sz = f(f(300) - f(-300)) / f(b.n_z)
    for e in (0, 1):
        if x_axis_outer_hits:
            i = idx(e, 2, 0); x[i], y[i] = rad(i), f(0.0)
            i = idx(e, 2, 1); x[i], y[i] = -rad(i), f(-0.0)
        for l in (1, 3):
            if x_axis_outer_hits or l == 1:
                i = idx(e, l, 2); x[i], y[i] = -rad(i), f(0.0)
            i = idx(e, l, 3); x[i], y[i] = f(0.0), rad(i)
        i, j = idx(e, 2, 4), idx(e, 1, 4); x[i], y[i] = x[j], y[j]
        i, j = idx(e, 3, 5), idx(e, 3, 6); x[i], y[i], z[i] = x[j], y[j], z[j]
        i = idx(e, 1, 7); z[i] = f(-300.0)
        for k, l in ((8, 1), (9, 2), (10, 3)):
            i = idx(e, l, k); z[i] = f(-300.0) + f(b.n_z // 2) * sz
        i = idx(e, 1, 11); x[i], y[i] = -rad(i), f(-1e-30)
        i = idx(e, 2, 6); x[i], y[i] = f(1e-20), f(1e-20)
        i = idx(e, 2, 7); x[i], y[i] = f(1e-3), f(-1e-3)
    cols = {k: getattr(b, k) for k in ("layer", "det_id", "hit_id", "event")}
    cols.update(x=x, y=y, z=z)
    return events._assemble(cols, b.layer_hits, b)


def test_oracle_on_degenerate_hits(oracle_lib):
    b = degenerate_batch()
    r = oracle_lib.run(b)[0]
    # phi = +pi lands in the overflow column nP, which the prediction's row
    # end includes and the pair window's does not (Q8)
    f = np.float32
    sp = (f(np.pi) - f(-np.pi)) / f(b.n_phi)
    phi = np.arctan2(f(0.0), -np.hypot(b.x[:1], b.y[:1]).astype(np.float32))[0]
    assert phi == f(np.pi) and np.floor((phi - f(-np.pi)) / sp) == b.n_phi
    C = (b.n_z + 1) * (b.n_phi + 1)
    grid = r["grid"].reshape(b.n_events, b.n_layers, C).astype(np.int64)
    ends = np.concatenate([grid[..., 1:], grid[..., -1:]], axis=-1)
    overflow = (ends - grid).reshape(b.n_events, b.n_layers, b.n_z + 1, b.n_phi + 1)[..., b.n_phi]
    assert overflow[:, 0].sum() >= 2 and overflow[:, 2].sum() >= 2
    # every hit is placed once and the chain runs to the tracks
    assert np.array_equal(np.sort(r["perm"]), np.arange(b.n_hits))
    assert r["stats_dict"]["triplets"] > 0 and r["stats_dict"]["links"] > 0
