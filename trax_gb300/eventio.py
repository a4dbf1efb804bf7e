"""Event files (PEventContainer) and the reference's event loader, through the
C ABI (trax_events_read / trax_events_raw / trax_events_load, and
trax_events_upload with the layer bucketing on the device): the hits of a
file become an EventBatch like the synthetic workloads', or the hits of a
context directly, plus the findable tracks the physics metrics count
against."""
from __future__ import annotations

import ctypes
import dataclasses
import os
from typing import Dict, List, Optional

import numpy as np

from . import capi, events


class LoadedSizesC(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("n_hits", "n_events", "n_layers", "n_findable")]


def _p(a):
    return None if a is None else a.ctypes.data


def geometry_from_files(radius_dictionary: str, detector_radius: str, n_layers: int = 13):
    """(min_r, max_r) per layer from the detector tables (trax_geometry_from_files)."""
    L = capi.load()
    mn = np.zeros(n_layers, np.float32)
    mx = np.zeros(n_layers, np.float32)
    rc = L.trax_geometry_from_files(os.fsencode(radius_dictionary), os.fsencode(detector_radius), n_layers,
                                    mn.ctypes.data, mx.ctypes.data)
    if rc != capi.TRAX_OK:
        raise capi.TraxError(rc, "cannot read the detector tables")
    return mn, mx


class EventFile:
    """An opened PEventContainer file (parsed on the host)."""

    def __init__(self, path: str):
        self._L = capi.load()
        h = ctypes.c_void_p()
        n = ctypes.c_uint64()
        rc = self._L.trax_events_read(os.fsencode(path), ctypes.byref(h), ctypes.byref(n))
        if rc != capi.TRAX_OK:
            raise capi.TraxError(rc, f"cannot read event file {path}")
        self._h = h
        self.n_events = int(n.value)

    def close(self):
        if getattr(self, "_h", None):
            self._L.trax_events_free(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def raw(self, e: int) -> Dict[str, np.ndarray]:
        """The hits of event e as stored in the file."""
        n = ctypes.c_uint64()
        self._check(self._L.trax_events_raw(self._h, e, ctypes.byref(n), *([None] * 8)))
        k = int(n.value)
        out = {"xyz": np.zeros((k, 3), np.float32), "layer": np.zeros(k, np.uint64),
               "det_id": np.zeros(k, np.uint64), "hit_id": np.zeros(k, np.uint64),
               "sim_track_id": np.zeros(k, np.uint64), "sim_pt": np.zeros(k, np.float32),
               "det_type": np.zeros(k, np.int32), "run_lumi_event": np.zeros(3, np.uint64)}
        self._check(self._L.trax_events_raw(self._h, e, ctypes.byref(n), *[_p(out[key]) for key in (
            "xyz", "layer", "det_id", "hit_id", "sim_track_id", "sim_pt", "det_type", "run_lumi_event")]))
        return out

    def load(self, lts: List[events.LayerTriplet], min_pt: float, first: int = 0, count: Optional[int] = None,
             num_tracks: int = -1, only_tracks: bool = False, n_z: int = 50, n_phi: int = 8,
             min_r: Optional[np.ndarray] = None, max_r: Optional[np.ndarray] = None):
        """HitCollection::addEvent over events [first, first + count): (EventBatch,
        findable track ids [n], their events [n]).  Radii default to the hits'
        own min/max radius per layer."""
        count = self.n_events - first if count is None else count
        lt = (capi.LayerTripletC * len(lts))(*[capi.LayerTripletC(
            t.layer1, t.layer2, t.layer3, t.dtheta_cut, t.sigma_z, t.dphi_cut, t.sigma_phi, t.tip_cut,
            t.pair_spread_z, t.z0, t.pair_spread_phi, t.n_candidates) for t in lts])
        sz = LoadedSizesC()
        args = [self._h, first, count, lt, len(lts), ctypes.c_float(min_pt), num_tracks, int(only_tracks),
                ctypes.byref(sz)]
        self._check(self._L.trax_events_load(*args, *([None] * 12)))
        H, E, L, F = (int(getattr(sz, k)) for k in ("n_hits", "n_events", "n_layers", "n_findable"))
        cols = {k: np.zeros(H, np.float32) for k in ("x", "y", "z")}
        cols.update({k: np.zeros(H, np.uint32) for k in ("layer", "det_id", "hit_id", "event")})
        ev_off = np.zeros(E, np.uint32)
        lay_hits = np.zeros((E, L), np.uint32)
        lay_off = np.zeros((E, L), np.uint32)
        fid = np.zeros(F, np.uint32)
        fev = np.zeros(F, np.uint32)
        self._check(self._L.trax_events_load(*args, *[_p(a) for a in (
            cols["x"], cols["y"], cols["z"], cols["layer"], cols["det_id"], cols["hit_id"], cols["event"],
            ev_off, lay_hits, lay_off, fid, fev)]))
        r = np.hypot(cols["x"].astype(np.float64), cols["y"].astype(np.float64))
        if min_r is None or max_r is None:
            min_r = np.array([r[cols["layer"] == l].min() if np.any(cols["layer"] == l) else 0.0
                              for l in range(1, L + 1)], np.float32)
            max_r = np.array([r[cols["layer"] == l].max() if np.any(cols["layer"] == l) else 0.0
                              for l in range(1, L + 1)], np.float32)
        batch = events.EventBatch(
            x=cols["x"], y=cols["y"], z=cols["z"], layer=cols["layer"], det_id=cols["det_id"],
            hit_id=cols["hit_id"], event=cols["event"], event_offsets=ev_off, layer_hits=lay_hits,
            layer_offsets=lay_off, min_r=np.asarray(min_r, np.float32), max_r=np.asarray(max_r, np.float32),
            lts=list(lts), n_z=n_z, n_phi=n_phi, min_pt=min_pt, d_eta_cut=events.D_ETA_CUT)
        return batch, fid, fev

    def upload(self, ctx: "capi.Context", lts: List[events.LayerTriplet], min_pt: float, first: int = 0,
               count: Optional[int] = None, num_tracks: int = -1, only_tracks: bool = False):
        """The loader with its layer bucketing on the device (trax_events_upload):
        the context's hits become those of `load` without a host-side copy of
        the reordered columns.  The context's layer triplets, geometry and grid
        are set by the caller.  Returns (sizes, findable track ids, their
        events)."""
        count = self.n_events - first if count is None else count
        lt = (capi.LayerTripletC * len(lts))(*[capi.LayerTripletC(
            t.layer1, t.layer2, t.layer3, t.dtheta_cut, t.sigma_z, t.dphi_cut, t.sigma_phi, t.tip_cut,
            t.pair_spread_z, t.z0, t.pair_spread_phi, t.n_candidates) for t in lts])
        sz = LoadedSizesC()
        cap = 1 << 20
        fid = np.zeros(cap, np.uint32)
        fev = np.zeros(cap, np.uint32)
        ctx._check(self._L.trax_events_upload(ctx._h, self._h, first, count, lt, len(lts), ctypes.c_float(min_pt),
                                               num_tracks, int(only_tracks), ctypes.byref(sz), _p(fid), _p(fev),
                                               cap))
        H, E, L, F = (int(getattr(sz, k)) for k in ("n_hits", "n_events", "n_layers", "n_findable"))
        ctx.n_events, ctx.n_layers, ctx.n_hits = E, L, H
        if F > cap:
            raise capi.TraxError(capi.TRAX_ERR_CAPACITY, f"{F} findable tracks, more than {cap}")
        return {"n_hits": H, "n_events": E, "n_layers": L, "n_findable": F}, fid[:F].copy(), fev[:F].copy()

    def _check(self, rc):
        if rc != capi.TRAX_OK:
            raise capi.TraxError(rc, "event file access failed")
