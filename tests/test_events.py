"""Seeded synthetic workloads: determinism, layout and sizes."""
import numpy as np

from trax_gb300 import events


def test_generation_is_deterministic():
    a = events.generate(1, n_events=5)
    b = events.generate(1, n_events=5)
    for k in ("x", "y", "z", "layer", "hit_id", "event", "layer_hits"):
        assert np.array_equal(getattr(a, k), getattr(b, k))


def test_supplements_describe_the_hit_order():
    b = events.generate(2, n_events=7)
    pos = 0
    for e in range(b.n_events):
        assert b.event_offsets[e] == pos
        for l in range(b.n_layers):
            n = b.layer_hits[e, l]
            s = pos + b.layer_offsets[e, l]
            assert np.all(b.layer[s:s + n] == l + 1) and np.all(b.event[s:s + n] == e)
        pos += int(b.layer_hits[e].sum())
    assert pos == b.n_hits


def test_hits_lie_on_their_layers():
    b = events.generate(2, n_events=3)
    r = np.hypot(b.x.astype(np.float64), b.y.astype(np.float64))
    lay = b.layer - 1
    assert np.all(r >= b.min_r[lay] - 0.01) and np.all(r <= b.max_r[lay] + 0.01)
    assert np.all(np.abs(b.z) < 110.0)


def test_workload_sizes():
    w = events.workload(2)
    assert w.n_events == 1000 and len(w.radii) == 10 and len(w.lts) == 6
    b = events.generate(2, n_events=40)
    per = b.layer_hits.sum(axis=1)
    assert per.min() >= 500 and per.max() <= 45000
    assert events.workload(3).n_vertices == 20 and events.workload(3).n_z == 80


def test_layer_triplet_cuts_follow_the_reference_rows():
    lts = events.workload(2).lts
    assert [(t.layer1, t.layer2, t.layer3) for t in lts] == [(k, k + 1, k + 2) for k in range(1, 7)]
    assert lts[0].sigma_z == np.float32(0.037) and lts[1].sigma_phi == np.float32(0.102)
    assert lts[3].tip_cut == 3.5 and lts[5].z0 == 10.0


def test_subset_renumbers_events():
    b = events.generate(1, n_events=6)
    s = b.subset([4, 1])
    assert s.n_events == 2 and np.array_equal(np.unique(s.event), [0, 1])
    assert s.n_hits == int(b.layer_hits[4].sum() + b.layer_hits[1].sum())
