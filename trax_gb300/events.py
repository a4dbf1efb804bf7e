"""Seeded synthetic barrel events for the triplet-seeding path.

The reference's own event files (protobuf containers of simulated CMS
events) are not distributed with it, so every workload here is generated:
helical tracks from a beamspot, intersected exactly (float64) with barrel
layers, smeared, stored as float32 hits, plus uniform noise hits.

A barrel layer is a set of modules placed at radius ``r`` +- ``stagger``
(uniform per hit), ``|z| < half_length``.  The geometry supplement (minimum and
maximum layer radius, the reference's ``GeometrySupplement``) is the module
envelope ``r -+ stagger``, as the reference takes it from its module radius
tables (TripletBuilder.cpp:145-184).

Hit order inside a layer is a seeded shuffle, hits are bucketed by event and
layer as ``HitCollection::addEvent`` does (HitCollection.cpp:120-163), and the
supplements (event offsets, per-layer counts and offsets) describe that order.

Workloads (sizes, distributions and cuts; the layer-triplet cut columns that a
workload does not name come from the reference's configs/layerTriplets.xml
row of the same index, falling back to its first row):

  config 0  10 events x 10 muons, pixel layers 4.4/7.3/10.2 cm, LT (1,2,3),
            grid 20x20, pT log-uniform 1-10 GeV, |eta| < 1, seed 0
  config 1  100 events x 200 tracks + 20% noise, 4 layers, LTs (1,2,3)
            (2,3,4), grid 40x100, pT 0.5 + Exp(1) GeV, |eta| < 1.5, seed 1
  config 2  1000 events, tracks ~ Poisson(lambda), lambda ~ U[300, 3000],
            10 layers, LTs (k,k+1,k+2) k=1..6, pT = 0.7 u^-1/2 (pT^-3 above
            0.7 GeV), |eta| < 2.5, seed 2
  config 3  16 events x 20 vertices x 1000 tracks + 5% noise, config-2
            geometry, grid 80x256, seed 3
  config 4  config-2 events with hidden per-layer misalignments
            (dr, dz ~ N(0, 50 um), dphi ~ N(0, 20 urad)), seed 4
"""
from __future__ import annotations

import dataclasses
import math
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

# configs/layerTriplets.xml rows: dThetaCut, sigmaZ, dPhiCut, sigmaPhi, tipCut,
# pairSpreadZ, z0, pairSpreadPhi, nCandidates
XML_ROWS = [
    (0.01, 0.037, 0.075, 0.032, 0.5, 2, 10.0, 2, 4),
    (0.2, 0.207, 0.2, 0.102, 0.5, 2, 10.0, 2, 16),
    (0.4, 0.207, 0.4, 0.102, 1.0, 3, 15.0, 2, 64),
    (0.5, 0.207, 0.4, 0.102, 3.5, 4, 30.0, 2, 128),
]

PIXEL_RADII = (4.4, 7.3, 10.2)
BARREL10_RADII = (4.4, 7.3, 10.2, 25.5, 33.9, 41.8, 49.8, 60.8, 69.2, 78.0)
D_ETA_CUT = 0.0256  # TripletBuilder.cpp:793


def half_length(r: float) -> float:
    """Barrel half-length: pixel 26.7 cm, strips 65 cm (r < 50), 110 cm (r >= 50)."""
    if r < 20.0:
        return 26.7
    if r < 50.0:
        return 65.0
    return 110.0


@dataclasses.dataclass
class LayerTriplet:
    layer1: int
    layer2: int
    layer3: int
    dtheta_cut: float
    sigma_z: float
    dphi_cut: float
    sigma_phi: float
    tip_cut: float
    pair_spread_z: int
    z0: float
    pair_spread_phi: int
    n_candidates: int


def layer_triplets(first_layers: Sequence[int], dtheta=None, dphi=None, tip=None) -> List[LayerTriplet]:
    out = []
    for idx, l1 in enumerate(first_layers):
        row = XML_ROWS[idx] if idx < len(XML_ROWS) else XML_ROWS[0]
        d_t, s_z, d_p, s_p, t_c, psz, z0, psp, nc = row
        out.append(LayerTriplet(l1, l1 + 1, l1 + 2,
                                dtheta if dtheta is not None else d_t, s_z,
                                dphi if dphi is not None else d_p, s_p,
                                tip if tip is not None else t_c, psz, float(int(z0)), psp, nc))
    return out


@dataclasses.dataclass
class Workload:
    name: str
    seed: int
    n_events: int
    radii: Tuple[float, ...]
    lts: List[LayerTriplet]
    n_z: int
    n_phi: int
    min_pt: float
    tracks: str = "fixed"          # fixed | poisson_uniform_lambda
    n_tracks: int = 10
    lambda_range: Tuple[float, float] = (300.0, 3000.0)
    n_vertices: int = 1
    pt_dist: str = "loguniform"    # loguniform | exp | powerlaw3
    pt_range: Tuple[float, float] = (1.0, 10.0)
    eta_max: float = 1.0
    b_field: float = 3.8
    sigma_rphi: float = 0.0015     # 15 um
    sigma_z: float = 0.0020        # 20 um
    efficiency: float = 0.99
    noise_fraction: float = 0.0
    stagger: float = 0.1           # module radius spread, cm
    vertex_sigma_z: float = 5.3
    vertex_sigma_xy: float = 0.001
    d_eta_cut: float = D_ETA_CUT
    misalign: bool = False


def workload(config: int, n_events: Optional[int] = None) -> Workload:
    """The five workloads; ``n_events`` shrinks one for a bounded sample."""
    if config == 0:
        w = Workload("muons-10x10-3layer", 0, 10, PIXEL_RADII,
                     layer_triplets([1], dtheta=0.01, dphi=0.05, tip=1.0), 20, 20, 1.0,
                     n_tracks=10, pt_dist="loguniform", pt_range=(1.0, 10.0), eta_max=1.0)
    elif config == 1:
        w = Workload("multimuon-100x200-4layer", 1, 100, PIXEL_RADII + (25.5,),
                     layer_triplets([1, 2], dtheta=0.01, dphi=0.05, tip=1.0), 40, 100, 0.5,
                     n_tracks=200, pt_dist="exp", pt_range=(0.5, 0.0), eta_max=1.5,
                     noise_fraction=0.2)
    elif config in (2, 4):
        # the alignment workload adds the layer triplets (7,8,9) and (8,9,10):
        # with only the first six, layers 9 and 10 are in no triplet and
        # their shifts have no gradient.  The ttbar-like workload's grid,
        # 250 x 48, is trax_autotune's choice for it on a GB300 (a search
        # over 35 grids: 200 x 64, 300 x 48 and 150 x 64 within 1 %); every
        # implementation timed on this workload runs that grid.
        nz, nphi = (250, 48) if config == 2 else (50, 128)
        w = Workload("ttbarlike-1000-uneven-10layer" if config == 2 else "alignment-1000-10layer",
                     config, 1000, BARREL10_RADII,
                     layer_triplets([1, 2, 3, 4, 5, 6] if config == 2 else [1, 2, 3, 4, 5, 6, 7, 8]),
                     nz, nphi, 0.7, tracks="poisson_uniform_lambda", pt_dist="powerlaw3",
                     pt_range=(0.7, 0.0), eta_max=2.5, misalign=(config == 4))
    elif config == 3:
        w = Workload("pileup-16x20x1000-10layer", 3, 16, BARREL10_RADII,
                     layer_triplets([1, 2, 3, 4, 5, 6]), 80, 256, 0.7, n_tracks=1000,
                     n_vertices=20, pt_dist="powerlaw3", pt_range=(0.7, 0.0), eta_max=2.5,
                     noise_fraction=0.05)
    else:
        raise ValueError(f"unknown config {config}")
    if config == 4:
        # A radial shift moves a track's predicted z on the next layer by
        # cot(theta) * dr (up to 0.03 cm for 50 um at |eta| = 2.5), close to
        # the prediction window's sigma_z = 0.037 cm: windows that tight keep
        # triplets by their misalignment-made z residual and bias the fitted
        # shifts by several um.  The alignment workload opens the z windows
        # four times.
        w = dataclasses.replace(w, lts=[dataclasses.replace(lt, sigma_z=4.0 * lt.sigma_z) for lt in w.lts])
    if n_events is not None:
        w = dataclasses.replace(w, n_events=int(n_events))
    return w


@dataclasses.dataclass
class EventBatch:
    """Hits in the reference's HitCollection layout plus supplements and config."""
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    layer: np.ndarray       # uint32, 1-based
    det_id: np.ndarray
    hit_id: np.ndarray      # simulated track id (0 for noise), the reference's HitId column
    event: np.ndarray       # uint32, 0-based
    event_offsets: np.ndarray
    layer_hits: np.ndarray  # [E, L]
    layer_offsets: np.ndarray
    min_r: np.ndarray       # [L] float32
    max_r: np.ndarray
    lts: List[LayerTriplet]
    n_z: int
    n_phi: int
    min_pt: float
    d_eta_cut: float
    workload: Optional[Workload] = None
    track_pt: Optional[List[np.ndarray]] = None        # per event, per track id-1
    misalignment: Optional[np.ndarray] = None           # [L, 3] (dr, dz, dphi)

    @property
    def n_events(self) -> int:
        return int(self.event_offsets.shape[0])

    @property
    def n_layers(self) -> int:
        return int(self.min_r.shape[0])

    @property
    def n_hits(self) -> int:
        return int(self.x.shape[0])

    def lt_columns(self) -> Dict[str, np.ndarray]:
        cols = {}
        for f in dataclasses.fields(LayerTriplet):
            vals = [getattr(lt, f.name) for lt in self.lts]
            dt = np.uint32 if f.type in ("int", int) else np.float32
            cols[f.name] = np.ascontiguousarray(np.array(vals, dtype=dt))
        return cols

    def subset(self, events: Sequence[int]) -> "EventBatch":
        """A batch made of the listed events (renumbered 0..k-1)."""
        parts = {k: [] for k in ("x", "y", "z", "layer", "det_id", "hit_id", "event")}
        lh = []
        for new_e, e in enumerate(events):
            a = int(self.event_offsets[e])
            b = a + int(self.layer_hits[e].sum())
            for k in parts:
                v = getattr(self, k)[a:b]
                if k == "event":
                    v = np.full(b - a, new_e, dtype=np.uint32)
                parts[k].append(v)
            lh.append(self.layer_hits[e])
        layer_hits = np.array(lh, dtype=np.uint32).reshape(len(events), self.n_layers)
        out = _assemble({k: np.concatenate(v) if v else np.zeros(0, np.uint32) for k, v in parts.items()},
                        layer_hits, self)
        out.misalignment = self.misalignment
        if self.track_pt is not None:
            out.track_pt = [self.track_pt[e] for e in events]
        return out


def _assemble(cols, layer_hits, like: "EventBatch") -> "EventBatch":
    E = layer_hits.shape[0]
    tot = layer_hits.sum(axis=1).astype(np.uint64)
    event_offsets = np.zeros(E, dtype=np.uint32)
    if E > 1:
        event_offsets[1:] = np.cumsum(tot)[:-1].astype(np.uint32)
    layer_offsets = np.zeros_like(layer_hits)
    if layer_hits.shape[1] > 1:
        layer_offsets[:, 1:] = np.cumsum(layer_hits, axis=1)[:, :-1]
    return EventBatch(
        x=np.ascontiguousarray(cols["x"], dtype=np.float32),
        y=np.ascontiguousarray(cols["y"], dtype=np.float32),
        z=np.ascontiguousarray(cols["z"], dtype=np.float32),
        layer=np.ascontiguousarray(cols["layer"], dtype=np.uint32),
        det_id=np.ascontiguousarray(cols["det_id"], dtype=np.uint32),
        hit_id=np.ascontiguousarray(cols["hit_id"], dtype=np.uint32),
        event=np.ascontiguousarray(cols["event"], dtype=np.uint32),
        event_offsets=event_offsets,
        layer_hits=np.ascontiguousarray(layer_hits, dtype=np.uint32),
        layer_offsets=np.ascontiguousarray(layer_offsets, dtype=np.uint32),
        min_r=like.min_r, max_r=like.max_r, lts=like.lts, n_z=like.n_z, n_phi=like.n_phi,
        min_pt=like.min_pt, d_eta_cut=like.d_eta_cut, workload=like.workload)


def _sample_pt(rng, w: Workload, n: int) -> np.ndarray:
    if w.pt_dist == "loguniform":
        lo, hi = w.pt_range
        return np.exp(rng.uniform(math.log(lo), math.log(hi), n))
    if w.pt_dist == "exp":
        return w.pt_range[0] + rng.exponential(1.0, n)
    if w.pt_dist == "powerlaw3":
        u = 1.0 - rng.uniform(0.0, 1.0, n)  # (0, 1]
        return w.pt_range[0] * u ** -0.5
    raise ValueError(w.pt_dist)


def _helix_hits(vx, vy, vz, pt, eta, phi0, q, radius, b_field):
    """Exact helix / cylinder(radius) intersection on the outgoing half turn.

    Returns (x, y, z, ok) in float64.  R = pT / (0.299792458 B) m.
    """
    R = pt / (0.299792458 * b_field) * 100.0  # cm
    # centre of curvature: a positive charge in +Bz turns clockwise
    cx = vx + q * R * np.sin(phi0)
    cy = vy - q * R * np.cos(phi0)
    d = np.hypot(cx, cy)
    psi = np.arctan2(cy, cx)
    arg = (radius * radius - d * d - R * R) / (2.0 * R * d)
    ok = np.abs(arg) <= 1.0
    arg = np.clip(arg, -1.0, 1.0)
    dth = np.arccos(arg)
    th0 = np.arctan2(vy - cy, vx - cx)
    # position angle theta(alpha) = th0 - q alpha; solutions theta = psi +- dth
    two_pi = 2.0 * np.pi
    a1 = np.mod((th0 - (psi + dth)) * q, two_pi)
    a2 = np.mod((th0 - (psi - dth)) * q, two_pi)
    alpha = np.minimum(a1, a2)
    ok &= alpha < np.pi
    th = th0 - q * alpha
    x = cx + R * np.cos(th)
    y = cy + R * np.sin(th)
    z = vz + R * alpha * np.sinh(eta)
    return x, y, z, ok


def generate(config: int, n_events: Optional[int] = None, seed: Optional[int] = None) -> EventBatch:
    """Generate the workload `config` (0-4), optionally only its first events."""
    return generate_workload(workload(config, n_events), seed)


def generate_workload(w: Workload, seed: Optional[int] = None) -> EventBatch:
    """Generate the events of a workload description."""
    rng = np.random.Generator(np.random.PCG64(w.seed if seed is None else seed))
    L = len(w.radii)
    radii = np.array(w.radii)
    misalign = None
    if w.misalign:
        misalign = np.stack([rng.normal(0.0, 0.005, L), rng.normal(0.0, 0.005, L),
                             rng.normal(0.0, 20e-6, L)], axis=1)
    cols = {k: [] for k in ("x", "y", "z", "layer", "det_id", "hit_id", "event")}
    layer_hits = np.zeros((w.n_events, L), dtype=np.uint32)
    track_pt = []
    for e in range(w.n_events):
        if w.tracks == "fixed":
            n_tr_per_vtx = [w.n_tracks] * w.n_vertices
        else:
            lam = rng.uniform(*w.lambda_range)
            n_tr_per_vtx = [int(rng.poisson(lam))]
        vz_v = rng.normal(0.0, w.vertex_sigma_z, w.n_vertices)
        vx_v = rng.normal(0.0, w.vertex_sigma_xy, w.n_vertices)
        vy_v = rng.normal(0.0, w.vertex_sigma_xy, w.n_vertices)
        ntr = int(sum(n_tr_per_vtx))
        vidx = np.repeat(np.arange(len(n_tr_per_vtx)), n_tr_per_vtx)
        pt = _sample_pt(rng, w, ntr)
        eta = rng.uniform(-w.eta_max, w.eta_max, ntr)
        phi0 = rng.uniform(-np.pi, np.pi, ntr)
        q = np.where(rng.uniform(0.0, 1.0, ntr) < 0.5, -1.0, 1.0)
        track_pt.append(pt.astype(np.float32))
        ev_x, ev_y, ev_z, ev_l, ev_id = [], [], [], [], []
        n_signal = np.zeros(L, dtype=np.int64)
        for li in range(L):
            r_hit = radii[li] + rng.uniform(-w.stagger, w.stagger, ntr)
            if misalign is not None:
                r_hit = r_hit + misalign[li, 0]
            x, y, z, ok = _helix_hits(vx_v[vidx], vy_v[vidx], vz_v[vidx], pt, eta, phi0, q, r_hit, w.b_field)
            hl = half_length(radii[li])
            ok &= np.abs(z) < hl
            ok &= rng.uniform(0.0, 1.0, ntr) < w.efficiency
            # smearing: r-phi along the tangent, z along the axis
            rphi = rng.normal(0.0, w.sigma_rphi, ntr)
            dz = rng.normal(0.0, w.sigma_z, ntr)
            ph = np.arctan2(y, x)
            x = x - np.sin(ph) * rphi
            y = y + np.cos(ph) * rphi
            z = z + dz
            if misalign is not None:
                # measured with nominal geometry: undo the hidden shifts
                rr = np.hypot(x, y) - misalign[li, 0]
                ph2 = np.arctan2(y, x) - misalign[li, 2]
                x, y = rr * np.cos(ph2), rr * np.sin(ph2)
                z = z - misalign[li, 1]
            ids = np.nonzero(ok)[0]
            ev_x.append(x[ids]); ev_y.append(y[ids]); ev_z.append(z[ids])
            ev_id.append(ids + 1)
            ev_l.append(np.full(ids.size, li + 1))
            n_signal[li] = ids.size
        for li in range(L):
            n_noise = int(round(w.noise_fraction * n_signal[li]))
            if n_noise:
                hl = half_length(radii[li])
                rr = radii[li] + rng.uniform(-w.stagger, w.stagger, n_noise)
                ph = rng.uniform(-np.pi, np.pi, n_noise)
                ev_x.append(rr * np.cos(ph)); ev_y.append(rr * np.sin(ph))
                ev_z.append(rng.uniform(-hl + 0.01, hl - 0.01, n_noise))
                ev_id.append(np.zeros(n_noise, dtype=np.int64))
                ev_l.append(np.full(n_noise, li + 1))
        x = np.concatenate(ev_x); y = np.concatenate(ev_y); z = np.concatenate(ev_z)
        lay = np.concatenate(ev_l); tid = np.concatenate(ev_id)
        # bucket by layer, seeded shuffle inside a layer
        key = lay * 4.0 + rng.uniform(0.0, 1.0, lay.size)
        order = np.argsort(key, kind="stable")
        x, y, z, lay, tid = x[order], y[order], z[order], lay[order], tid[order]
        x32 = x.astype(np.float32); y32 = y.astype(np.float32); z32 = z.astype(np.float32)
        mod = np.floor((np.arctan2(y, x) + np.pi) / (2.0 * np.pi) * 64.0).astype(np.int64) % 64
        cols["x"].append(x32); cols["y"].append(y32); cols["z"].append(z32)
        cols["layer"].append(lay.astype(np.uint32))
        cols["det_id"].append((lay * 100000 + mod).astype(np.uint32))
        cols["hit_id"].append(tid.astype(np.uint32))
        cols["event"].append(np.full(lay.size, e, dtype=np.uint32))
        layer_hits[e] = np.bincount(lay - 1, minlength=L)[:L]
    proto = EventBatch(x=None, y=None, z=None, layer=None, det_id=None, hit_id=None, event=None,
                       event_offsets=None, layer_hits=None, layer_offsets=None,
                       min_r=np.array(radii - w.stagger, dtype=np.float32),
                       max_r=np.array(radii + w.stagger, dtype=np.float32),
                       lts=w.lts, n_z=w.n_z, n_phi=w.n_phi, min_pt=w.min_pt,
                       d_eta_cut=w.d_eta_cut, workload=w)
    batch = _assemble({k: np.concatenate(v) for k, v in cols.items()}, layer_hits, proto)
    batch.track_pt = track_pt
    batch.misalignment = misalign
    return batch
