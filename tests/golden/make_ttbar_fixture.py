"""Writes tests/golden/ttbar10_loaded.npz (run from the repository root, in a
checkout that has the reference project beside it; pass its path as the
first argument).

The reference ships ten real ttbar events (plotting/data/physics/hits.ttBar.pb,
a PEventContainer).  This script reads them with trax_gb300's own event-file
reader and loader (HitCollection::addEvent, HitCollection.cpp:21-180) at the
settings of the reference's configs/ttBar.reco.conf: the four layer triplets
of layerTriplets.xml (the fourth on layers 4, 5, 8), minPt 1.0 GeV, only the
hits of tracks, grid 50 x 8, and layer radii from configs/radiusDictionary.dat
and configs/detectorRadius.dat.  It stores the loaded hit collection (what
the loader hands to the seeding chain), the findable tracks, and the oracle's
triplet count and physics records on it, so that the GPU tests can run the
reference's own events on a machine without the reference.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

LT_FIELDS = ("layer1", "layer2", "layer3", "dtheta_cut", "sigma_z", "dphi_cut", "sigma_phi", "tip_cut",
             "pair_spread_z", "z0", "pair_spread_phi", "n_candidates")


def ttbar_layer_triplets():
    from trax_gb300 import events
    lts = events.layer_triplets([1, 2, 3, 4])
    t = lts[3]
    lts[3] = events.LayerTriplet(4, 5, 8, t.dtheta_cut, t.sigma_z, t.dphi_cut, t.sigma_phi, t.tip_cut,
                                 t.pair_spread_z, t.z0, t.pair_spread_phi, t.n_candidates)
    return lts


def main(ref_root):
    from oracle import oracle
    from trax_gb300 import eventio, physics
    f = eventio.EventFile(os.path.join(ref_root, "plotting/data/physics/hits.ttBar.pb"))
    lts = ttbar_layer_triplets()
    mn, mx = eventio.geometry_from_files(os.path.join(ref_root, "configs/radiusDictionary.dat"),
                                         os.path.join(ref_root, "configs/detectorRadius.dat"), 13)
    batch, fid, fev = f.load(lts, 1.0, only_tracks=True, n_z=50, n_phi=8, min_r=mn[:8], max_r=mx[:8])
    r = oracle.run(batch)[0]
    hid = batch.hit_id[r["perm"]]
    recs = physics.triplet_records(r["trip_h1"], r["trip_h2"], r["trip_h3"], r["trip_offsets"], batch.n_events,
                                   len(lts), hid, fid, fev)
    out = os.path.join(HERE, "ttbar10_loaded.npz")
    np.savez_compressed(
        out, x=batch.x, y=batch.y, z=batch.z, layer=batch.layer.astype(np.uint8), det_id=batch.det_id,
        hit_id=batch.hit_id, event=batch.event.astype(np.uint8), layer_hits=batch.layer_hits,
        min_r=batch.min_r, max_r=batch.max_r, findable_id=fid, findable_event=fev,
        lts=np.array([[float(getattr(t, k)) for k in LT_FIELDS] for t in lts], np.float64),
        oracle_triplets=np.array(r["stats_dict"]["triplets"]),
        oracle_efficiency=np.array([q["efficiency"] for q in recs], np.float64),
        oracle_fake_rate=np.array([q["fake_rate"] for q in recs], np.float64))
    print(out, os.path.getsize(out), "bytes;", batch.n_hits, "hits,", r["stats_dict"]["triplets"], "triplets")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(os.path.dirname(REPO), "reference"))
