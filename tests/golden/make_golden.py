"""Writes the golden fixtures of tests/golden/ (run from the repository root).

connectivity_kat.json
    The four-layer "tight" connectivity fixture of the reference's own tests
    (src/algorithms/test/TripletConnectivityTest.h:66-94,
    addFourLayerForwardTight, expected counts at :233-258), restated for the
    tight-connectivity + cellular-automaton path: triplet k of layer triplet p
    has its hits on layers p+1, p+2, p+3, so the reference's hit 27 -- used on
    two different layers by the fixture -- is renamed 127 in the last layer
    triplet.  The chain (1,4,6) -> (4,6,16) -> (6,16,30) -> (16,30,36) must link
    into one 4-triplet track; the expected connectivity 3 of its last triplet
    is CA state 4, every other triplet has state 1 (connectivity 0).  Hits of
    the chain lie on one straight line from the origin (equal eta); the other
    hits are spread in phi and z.

config0_golden.npz
    The seeded 10-event, 3-layer muon workload (inputs) and the CPU oracle's
    pairs, candidates, triplets and grid for it.  Inputs are stored, so the
    check does not depend on the random generator of the installed numpy.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

# TripletConnectivityTest.h:66-94 (the reference's hit 27 of the last block renamed 127)
SEGMENTS = [
    [(1, 4, 6), (1, 3, 5), (2, 3, 8), (2, 4, 7)],
    [(4, 6, 16), (9, 12, 17), (9, 13, 18), (9, 14, 19)],
    [(6, 16, 30), (15, 22, 29), (15, 24, 29), (15, 25, 27)],
    [(16, 30, 36), (28, 32, 37), (26, 33, 38), (127, 34, 39)],
]
CHAIN = [(1, 4, 6), (4, 6, 16), (6, 16, 30), (16, 30, 36)]
RADII = [4.4, 7.3, 10.2, 25.5, 33.9, 41.8]


def connectivity_kat():
    layer_of = {}
    for p, seg in enumerate(SEGMENTS):
        for trip in seg:
            for k, hid in enumerate(trip):
                lay = p + 1 + k
                assert layer_of.get(hid, lay) == lay, (hid, lay)
                layer_of[hid] = lay
    chain_hits = {h for t in CHAIN for h in t}
    ids = sorted(layer_of, key=lambda h: (layer_of[h], h))
    index = {h: i for i, h in enumerate(ids)}
    hits = []
    for h in ids:
        r = RADII[layer_of[h] - 1]
        if h in chain_hits:
            phi, cot = 0.3, 0.5
        else:
            phi, cot = 0.3 + 0.47 * h, 0.11 * (h % 9) - 0.4
        hits.append({"id": h, "layer": layer_of[h], "x": float(np.float32(r * np.cos(phi))),
                     "y": float(np.float32(r * np.sin(phi))), "z": float(np.float32(r * cot))})
    triplets = [[index[a], index[b], index[c]] for seg in SEGMENTS for (a, b, c) in seg]
    chain_idx = [triplets.index([index[a], index[b], index[c]]) for (a, b, c) in CHAIN]
    states = [1] * len(triplets)
    for k, t in enumerate(chain_idx):
        states[t] = k + 1
    return {
        "source": "src/algorithms/test/TripletConnectivityTest.h:66-94 (addFourLayerForwardTight)",
        "n_layer_triplets": len(SEGMENTS),
        "d_eta_cut": 0.0256,
        "hits": hits,
        "triplets": triplets,
        "expected": {
            "links": [[chain_idx[k], chain_idx[k + 1]] for k in range(len(chain_idx) - 1)],
            "ca_states": states,
            "chain_track": list(reversed(chain_idx)),
        },
    }


def config0():
    from oracle import oracle
    from trax_gb300 import events
    b = events.generate(0)
    r = oracle.run(b)[0]
    out = {k: getattr(b, k) for k in ("x", "y", "z", "layer", "det_id", "hit_id", "event", "event_offsets",
                                      "layer_hits", "layer_offsets", "min_r", "max_r")}
    for k in ("grid", "perm", "pairs", "cands", "trip_h1", "trip_h2", "trip_h3", "trip_offsets"):
        out["oracle_" + k] = r[k]
    return out


def main():
    with open(os.path.join(HERE, "connectivity_kat.json"), "w") as f:
        json.dump(connectivity_kat(), f, indent=1)
    np.savez_compressed(os.path.join(HERE, "config0_golden.npz"), **config0())
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    main()
