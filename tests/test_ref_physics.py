"""Our track evaluation against the reference's own code (CPU, no GPU).

``trax_physics_tracks`` (the host restatement of TripletBuilder.cpp:840-1066,
which ``trax_physics_tracks_device`` is tested against on the GPU) is
compared with the reference's functions themselves: extractTracks,
cloneRemoval, splitRealFakeTracks and findUniqueRealTracks, copied from
TripletBuilder.cpp by ``oracle/ref_extract.py`` and compiled against plain
arrays.  The five counts printTracks reports must be equal.
"""
import dataclasses

import numpy as np
import pytest

from oracle import oracle, ref
from trax_gb300 import events

pytestmark = pytest.mark.skipif(not ref.available(), reason="reference sources absent: oracle/_ref not built")

COUNTS = ("total", "filtered", "valid", "valid_unique", "fakes")


@pytest.fixture(scope="module")
def ours():
    from trax_gb300 import build, physics
    build.build()
    return physics


def both(physics, tracks, track_offsets, h1, h2, h3, hit_id):
    mine = physics.track_metrics(tracks, track_offsets, h1, h2, h3, hit_id, 1)
    theirs = ref.track_metrics(tracks, track_offsets, h1, h2, h3, hit_id)
    return {k: mine[k] for k in COUNTS}, theirs


def test_hand_counted_case(ours):
    h1, h2, h3 = [0, 1, 2, 3, 4], [1, 2, 3, 4, 5], [2, 3, 4, 5, 6]
    mine, theirs = both(ours, [1, 0, 4, 3, 2], [0, 0, 2, 2, 2, 5], h1, h2, h3, np.full(7, 7, np.uint32))
    assert mine == theirs == {"total": 1, "filtered": 1, "valid": 1, "valid_unique": 1, "fakes": 0}


def _ca_case(batch):
    o = oracle.run(batch, n_workers=4, links="indexed")[0]
    return o["tracks"], o["track_offsets"], o["trip_h1"], o["trip_h2"], o["trip_h3"], batch.hit_id[o["perm"]]


@pytest.mark.parametrize("case", ["config 2, 6 events, seed 7", "config 2, 20 events", "pileup event",
                                  "reference ttbar"])
def test_oracle_ca_output(ours, case):
    """The CA output of the oracle on workloads with six layer triplets (tracks
    need three triplets or more; config 1 has two).  Both clone removals are
    quadratic in the tracks (20 events: about 20 000 tracks, 4 s each)."""
    if case == "config 2, 6 events, seed 7":
        batch = events.generate(2, n_events=6, seed=7)
    elif case == "config 2, 20 events":
        batch = events.generate(2, n_events=20)
    elif case == "pileup event":
        batch = events.generate_workload(dataclasses.replace(events.workload(3), n_events=1, n_vertices=6))
    else:
        from tests.test_eventio import ttbar_fixture
        batch = ttbar_fixture()[0]
    mine, theirs = both(ours, *_ca_case(batch))
    assert theirs["total"] > 10, theirs
    assert mine == theirs


@pytest.mark.parametrize("seed", [1, 2, 3, 4, 5])
def test_random_track_sets(ours, seed):
    """Tracks that share many hits (clone removal keeps, replaces and drops),
    tracks of equal length, short CA chains and fakes."""
    rng = np.random.default_rng(seed)
    n_hits, n_sim = 400, 12
    hit_id = rng.integers(0, n_sim, n_hits).astype(np.uint32)
    n_t = 600
    # triplets over a small hit pool so that tracks overlap
    h1 = rng.integers(0, n_hits, n_t)
    h2 = rng.integers(0, n_hits, n_t)
    h3 = rng.integers(0, n_hits, n_t)
    # a third of the triplets lie on one simulated track each
    for t in range(0, n_t, 3):
        same = np.nonzero(hit_id == hit_id[h1[t]])[0]
        h2[t], h3[t] = rng.choice(same, 2)
    tracks, offsets = [], [0]
    for _ in range(n_t):
        length = int(rng.choice([0, 1, 2, 3, 4, 5, 6], p=[0.3, 0.1, 0.1, 0.2, 0.15, 0.1, 0.05]))
        tracks += list(rng.integers(0, n_t, length))
        offsets.append(len(tracks))
    mine, theirs = both(ours, np.array(tracks, np.uint32), np.array(offsets, np.uint32), h1, h2, h3, hit_id)
    assert theirs["total"] > 50 and theirs["filtered"] < theirs["total"], theirs
    assert mine == theirs
