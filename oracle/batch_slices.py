"""Every event's slice of a batched run against the oracle run on that event
alone.  TEST INFRASTRUCTURE: the GPU tests and the benchmark's parity check
use it as the checker.

Pair generation, prediction, filter and eta work within one event, so the
batched chain's pairs, candidates, triplets and eta of event e equal the
oracle's for e run as its own event group, once indices are shifted:

* hit indices by the event's first hit (grid order keeps events contiguous);
* pair indices (in candidates) by the event's first pair.

Two rules of the reference bound the slices:

* the triplet offsets' last entry is nT - 1, not nT (filterOffsetStore,
  TripletThetaPhiFilter.h:240-256), so the last event's triplets run to the
  end of the arrays;
* links, and so the connectable lists, pt and the CA, depend on the events
  grouped together: filterOffsetStore records where each (event, layer
  triplet) segment starts and the monotonize kernel fills empty segments
  with the previous start (TripletThetaPhiFilter.h:221-280), so when an
  event's trailing layer triplets have no triplets, its last non-empty
  segment reads as empty in a group and its triplets get no followers --
  run alone, the last-triplet rule gives that segment an end instead.  The
  reference's own kernels (oracle/_ref) show the same.  Those arrays are
  compared with the oracle run on the whole batch as one group instead.
"""
from __future__ import annotations

from typing import Dict, List

import numpy as np

SENTINEL = np.uint32(0xFFFFFFFF)


def compare(batch, got: Dict[str, np.ndarray], refs: List[Dict[str, np.ndarray]]) -> Dict[str, object]:
    """`got`: the batched run's arrays (trax_gb300.capi.Context.results());
    `refs`: oracle.run(batch, event_grouping=1) -- one dict per event.
    Returns {"events": n, "mismatch": {array: [events]}}."""
    n_lt = len(batch.lts)
    E = batch.n_events
    assert len(refs) == E
    po, co, to = (np.asarray(got[k]).astype(np.int64) for k in ("pair_offsets", "cand_offsets", "trip_offsets"))
    pairs = np.asarray(got["pairs"]).reshape(-1, 2)
    cands = np.asarray(got["cands"]).reshape(-1, 2)
    h = [np.asarray(got[k]) for k in ("trip_h1", "trip_h2", "trip_h3")]
    n_trip = h[0].size
    eta = np.asarray(got["eta"]).view(np.uint32)
    mism: Dict[str, List[int]] = {}

    def bad(name, e):
        mism.setdefault(name, []).append(int(e))

    for e in range(E):
        r = refs[e]
        off = np.int64(batch.event_offsets[e])
        pa, pb = po[e * n_lt], po[(e + 1) * n_lt]
        p = pairs[pa:pb].astype(np.int64)
        p = np.where(p != SENTINEL, p - off, p)
        if not np.array_equal(p.reshape(-1), r["pairs"].astype(np.int64)):
            bad("pairs", e)
        ca, cb = co[e * n_lt], co[(e + 1) * n_lt]
        c = cands[ca:cb].astype(np.int64)
        c[:, 0] -= pa
        c[:, 1] = np.where(c[:, 1] != SENTINEL, c[:, 1] - off, c[:, 1])
        if not np.array_equal(c.reshape(-1), r["cands"].astype(np.int64)):
            bad("cands", e)
        ta = to[e * n_lt]
        tb = to[(e + 1) * n_lt] if e + 1 < E else n_trip
        for k, col in zip(("trip_h1", "trip_h2", "trip_h3"), h):
            if not np.array_equal(col[ta:tb].astype(np.int64) - off, r[k].astype(np.int64)):
                bad(k, e)
        if not np.array_equal(eta[ta:tb], r["eta"].view(np.uint32)):
            bad("eta", e)
    return {"events": E, "mismatch": mism}


LINKING = ("link_basis", "link_follower", "connectable", "non_connectable", "ca_states", "ca_best", "tracks",
           "track_offsets")


def compare_whole(got: Dict[str, np.ndarray], whole: Dict[str, np.ndarray]) -> List[str]:
    """Arrays of the batched run that differ from the oracle run on the whole
    batch as one group (every array, element for element; pt on the
    connectable triplets, bit patterns)."""
    out = []
    for k in ("pairs", "pair_offsets", "cands", "cand_offsets", "trip_h1", "trip_h2", "trip_h3",
              "trip_offsets") + LINKING:
        if k in got and k in whole and not np.array_equal(np.asarray(got[k]), np.asarray(whole[k])):
            out.append(k)
    if "eta" in got and not np.array_equal(np.asarray(got["eta"]).view(np.uint32), whole["eta"].view(np.uint32)):
        out.append("eta")
    if "pt" in got and whole.get("connectable") is not None and whole["connectable"].size:
        c = whole["connectable"]
        if not np.array_equal(np.asarray(got["pt"])[c].view(np.uint32), whole["pt"][c].view(np.uint32)):
            out.append("pt")
    return out
