"""Physics bookkeeping of seeding results (trax_physics_triplets, counted on the
host or, for a context's triplets, on the device; trax_physics_tracks): triplet efficiency, fake and clone rates per layer
triplet as the reference's PhysicsRecord, and the track-level evaluation of
its triplet builder."""
from __future__ import annotations

import ctypes
from typing import Dict, List

import numpy as np

from . import capi


class PhysicsRecordC(ctypes.Structure):
    _fields_ = [("layer_triplet", ctypes.c_uint32), ("n", ctypes.c_uint64)] + [
        (k, ctypes.c_double) for k in ("efficiency", "efficiency_dev", "fake_rate", "fake_rate_dev", "clone_rate",
                                       "clone_rate_dev")]


class TrackMetricsC(ctypes.Structure):
    _fields_ = [(k, ctypes.c_uint64) for k in ("total", "filtered", "valid", "valid_unique", "fakes")] + [
        (k, ctypes.c_double) for k in ("fake_rate", "clone_rate", "efficiency")]


def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def triplet_records(h1, h2, h3, offsets, n_events: int, n_lt: int, hit_track_id, findable_id,
                    findable_event) -> List[Dict[str, float]]:
    """Per layer triplet, then the total: n, efficiency, fake and clone rates (means and deviations)."""
    L = capi.load()
    arrs = [_u32(a) for a in (h1, h2, h3, offsets, hit_track_id, findable_id, findable_event)]
    out = (PhysicsRecordC * (n_lt + 1))()
    rc = L.trax_physics_triplets(arrs[0].ctypes.data, arrs[1].ctypes.data, arrs[2].ctypes.data,
                                 arrs[3].ctypes.data, n_events, n_lt, arrs[4].ctypes.data, arrs[5].ctypes.data,
                                 arrs[6].ctypes.data, arrs[5].size, out)
    if rc != capi.TRAX_OK:
        raise capi.TraxError(rc, "trax_physics_triplets failed")
    return [{f[0]: getattr(r, f[0]) for f in PhysicsRecordC._fields_} for r in out]


def triplet_records_device(ctx: "capi.Context", findable_id, findable_event) -> List[Dict[str, float]]:
    """The same records for the context's current triplets, counted on the device
    (trax_physics_triplets_device)."""
    fid, fev = _u32(findable_id), _u32(findable_event)
    out = (PhysicsRecordC * (ctx.n_lt + 1))()
    ctx._check(ctx._L.trax_physics_triplets_device(ctx._h, fid.ctypes.data if fid.size else None,
                                                   fev.ctypes.data if fev.size else None, fid.size, out))
    return [{f[0]: getattr(r, f[0]) for f in PhysicsRecordC._fields_} for r in out]


def csv(records: List[Dict[str, float]]) -> str:
    """The reference's physics csv layout (layerTriplet n eff effVar fr frVar cr crVar)."""
    lines = ["layerTriplet n eff effVar fr frVar cr crVar"]
    for r in records:
        lines.append(f"{r['layer_triplet']} {r['n']} {r['efficiency']:.6g} {r['efficiency_dev']:.6g} "
                     f"{r['fake_rate']:.6g} {r['fake_rate_dev']:.6g} {r['clone_rate']:.6g} {r['clone_rate_dev']:.6g}")
    return "\n".join(lines) + "\n"


def track_metrics(tracks, track_offsets, h1, h2, h3, hit_track_id, total_tracks: int) -> Dict[str, float]:
    L = capi.load()
    arrs = [_u32(a) for a in (tracks, track_offsets, h1, h2, h3, hit_track_id)]
    out = TrackMetricsC()
    n_t = arrs[1].size - 1
    rc = L.trax_physics_tracks(arrs[0].ctypes.data if arrs[0].size else None, arrs[1].ctypes.data, max(n_t, 0),
                               arrs[2].ctypes.data if arrs[2].size else None,
                               arrs[3].ctypes.data if arrs[3].size else None,
                               arrs[4].ctypes.data if arrs[4].size else None, arrs[5].ctypes.data, total_tracks,
                               ctypes.byref(out))
    if rc != capi.TRAX_OK:
        raise capi.TraxError(rc, "trax_physics_tracks failed")
    return {f[0]: getattr(out, f[0]) for f in TrackMetricsC._fields_}


def track_metrics_device(ctx: "capi.Context", total_tracks: int) -> Dict[str, float]:
    """track_metrics for the context's current CA output, evaluated on the device
    (trax_physics_tracks_device)."""
    out = TrackMetricsC()
    ctx._check(ctx._L.trax_physics_tracks_device(ctx._h, total_tracks, ctypes.byref(out)))
    return {f[0]: getattr(out, f[0]) for f in TrackMetricsC._fields_}
