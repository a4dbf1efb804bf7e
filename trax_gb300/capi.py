"""ctypes binding of the C ABI in include/trax/trax.h (libtrax_gb300.so).

This is the Python view of the same entry points a C, C++ or cgo caller
binds.  The library must have been built (``trax_gb300.build.build()`` or
``__graft_entry__.build()``); loading fails loudly otherwise -- there is no
fallback implementation.
"""
from __future__ import annotations

import ctypes
import dataclasses
import os
import threading
import weakref
from typing import Dict, Optional

import numpy as np

from . import build as _build

TRAX_OK = 0
ERRORS = {1: "TRAX_ERR_CUDA", 2: "TRAX_ERR_ARG", 3: "TRAX_ERR_CAPACITY", 4: "TRAX_ERR_TIMEOUT",
          5: "TRAX_ERR_DEVICE_ASSERT", 6: "TRAX_ERR_STATE"}

EXPORTED = [
    "trax_create", "trax_destroy", "trax_last_error", "trax_version", "trax_set_layer_triplets",
    "trax_set_geometry", "trax_set_grid", "trax_upload_hits", "trax_grid_build", "trax_set_tracklets",
    "trax_pair_gen", "trax_prefix_sum_noalloc",
    "trax_triplet_predict", "trax_triplet_filter", "trax_connectivity", "trax_circle_fit",
    "trax_cellular_automaton", "trax_prefix_sum", "trax_seed_batch", "trax_get_stats", "trax_get_pairs",
    "trax_get_timings", "trax_get_candidates", "trax_get_triplets", "trax_get_triplet_eta_pt", "trax_get_links",
    "trax_get_tracks", "trax_get_grid", "trax_get_hit_perm", "trax_set_block_sizes", "trax_get_launch_config",
    "trax_autotune", "trax_fit_prepare", "trax_fit_forward", "trax_fit_backward", "trax_fit_get_rows",
    "trax_apply_alignment", "trax_events_read", "trax_events_free", "trax_events_raw", "trax_events_load",
    "trax_events_upload", "trax_physics_triplets_device", "trax_physics_tracks_device",
    "trax_physics_triplets", "trax_physics_tracks", "trax_geometry_from_files", "trax_host_alloc",
    "trax_host_free", "trax_set_wait_limit", "trax_debug_skip_publish", "trax_noalloc_set_wait",
    "trax_circle_fit_on", "trax_get_pt", "trax_cellular_automaton_on", "trax_set_pairs_per_thread",
    "trax_get_pairs_per_thread", "trax_math_eval", "trax_set_candidate_slots", "trax_get_candidate_slots",
    "trax_set_fine_rows", "trax_get_fine_rows",
]


class TraxError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class LayerTripletC(ctypes.Structure):
    _fields_ = [("layer1", ctypes.c_uint32), ("layer2", ctypes.c_uint32), ("layer3", ctypes.c_uint32),
                ("dtheta_cut", ctypes.c_float), ("sigma_z", ctypes.c_float), ("dphi_cut", ctypes.c_float),
                ("sigma_phi", ctypes.c_float), ("tip_cut", ctypes.c_float),
                ("pair_spread_z", ctypes.c_uint32), ("z0", ctypes.c_float),
                ("pair_spread_phi", ctypes.c_uint32), ("n_candidates", ctypes.c_uint32)]


class HitsSoaC(ctypes.Structure):
    _fields_ = [("x", ctypes.c_void_p), ("y", ctypes.c_void_p), ("z", ctypes.c_void_p),
                ("layer", ctypes.c_void_p), ("det_id", ctypes.c_void_p), ("hit_id", ctypes.c_void_p),
                ("event", ctypes.c_void_p)]


class BatchOptsC(ctypes.Structure):
    _fields_ = [("use_graph", ctypes.c_int), ("run_linking", ctypes.c_int), ("d_eta_cut", ctypes.c_float)]


class BatchStatsC(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in (
        "n_hits", "n_pairs", "n_candidates", "n_triplets", "n_links", "n_connectable", "n_non_connectable",
        "n_track_entries", "n_pair_sentinels", "n_candidate_sentinels", "kernel_launches")] + [
        ("device_ms", ctypes.c_double), ("graph_captures", ctypes.c_uint64)]


class FitOptsC(ctypes.Structure):
    _fields_ = [("sigma_z", ctypes.c_float), ("sigma_tip", ctypes.c_float * 16), ("truth_only", ctypes.c_int)]


class TuneOptsC(ctypes.Structure):
    _fields_ = [("search_grid", ctypes.c_int), ("run_linking", ctypes.c_int), ("replays", ctypes.c_int)]


class TuneResultC(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint32) for n in (
        "n_z", "n_phi", "pair_threads", "predict_threads", "filter_threads", "from_cache", "shapes_timed",
        "pairs_per_thread", "candidate_slots", "fine_rows", "reserved")] + [
        ("best_ms", ctypes.c_double), ("default_ms", ctypes.c_double)]


_lock = threading.Lock()
_lib = None


def library_path() -> str:
    """The product library, or with TRAX_GB300_BOUNDS_CHECK=1 in the
    environment its bounds-checked debug build."""
    if os.environ.get("TRAX_GB300_BOUNDS_CHECK") == "1":
        return _build.CHECKED_LIB_PATH
    return _build.LIB_PATH


def load() -> ctypes.CDLL:
    """Load libtrax_gb300.so (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: build it with __graft_entry__.build() (there is no CPU fallback)")
        L = ctypes.CDLL(path)
        vp, u32, u64, i32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
        pu64 = ctypes.POINTER(ctypes.c_uint64)
        sig = {
            "trax_create": ([ctypes.POINTER(vp), i32], i32),
            "trax_destroy": ([vp], None),
            "trax_last_error": ([vp], ctypes.c_char_p),
            "trax_version": ([], ctypes.c_char_p),
            "trax_set_layer_triplets": ([vp, vp, i32, ctypes.c_float], i32),
            "trax_set_geometry": ([vp, vp, vp, i32], i32),
            "trax_set_grid": ([vp, u32, u32], i32),
            "trax_upload_hits": ([vp, vp, u32, vp, vp, vp, u32, u32], i32),
            "trax_grid_build": ([vp], i32),
            "trax_set_tracklets": ([vp, vp, vp, vp, u64], i32),
            "trax_pair_gen": ([vp, pu64], i32),
            "trax_triplet_predict": ([vp, pu64], i32),
            "trax_triplet_filter": ([vp, pu64], i32),
            "trax_connectivity": ([vp, ctypes.c_float, pu64], i32),
            "trax_circle_fit": ([vp], i32),
            "trax_cellular_automaton": ([vp, pu64], i32),
            "trax_prefix_sum": ([vp, vp, u64], i32),
            "trax_set_pairs_per_thread": ([vp, u32], i32),
            "trax_get_pairs_per_thread": ([vp, vp], i32),
            "trax_set_candidate_slots": ([vp, u32], i32),
            "trax_get_candidate_slots": ([vp, vp], i32),
            "trax_set_fine_rows": ([vp, u32], i32),
            "trax_get_fine_rows": ([vp, vp], i32),
            "trax_set_wait_limit": ([vp, u32], i32),
            "trax_circle_fit_on": ([vp, vp, u64], i32),
            "trax_get_pt": ([vp, vp], i32),
            "trax_cellular_automaton_on": ([vp, vp, vp, u64, vp, u64, pu64], i32),
            "trax_debug_skip_publish": ([vp, u32], i32),
            "trax_noalloc_set_wait": ([u32, u32], i32),
            "trax_math_eval": ([i32, i32, vp, vp, vp, u64], i32),
            "trax_seed_batch": ([vp, vp, vp], i32),
            "trax_get_stats": ([vp, vp], i32),
            "trax_get_timings": ([vp, vp, vp], i32),
            "trax_get_pairs": ([vp, vp, vp], i32),
            "trax_get_candidates": ([vp, vp, vp], i32),
            "trax_get_triplets": ([vp, vp, vp, vp, vp], i32),
            "trax_get_triplet_eta_pt": ([vp, vp, vp], i32),
            "trax_get_links": ([vp, vp, vp, vp, vp], i32),
            "trax_get_tracks": ([vp, vp, vp, vp], i32),
            "trax_get_grid": ([vp, vp, pu64], i32),
            "trax_get_hit_perm": ([vp, vp], i32),
            "trax_set_block_sizes": ([vp, u32, u32, u32], i32),
            "trax_get_launch_config": ([vp, vp], i32),
            "trax_autotune": ([vp, ctypes.c_char_p, vp, vp], i32),
            "trax_fit_prepare": ([vp, vp, pu64], i32),
            "trax_fit_forward": ([vp, vp, vp, vp], i32),
            "trax_fit_backward": ([vp, vp, vp, vp, vp, vp], i32),
            "trax_fit_get_rows": ([vp, vp, vp], i32),
            "trax_apply_alignment": ([vp, vp], i32),
            "trax_events_read": ([ctypes.c_char_p, ctypes.POINTER(vp), pu64], i32),
            "trax_events_free": ([vp], None),
            "trax_events_raw": ([vp, u64, pu64, vp, vp, vp, vp, vp, vp, vp, vp], i32),
            "trax_events_load": ([vp, u64, u64, vp, i32, ctypes.c_float, i32, i32, vp] + [vp] * 12, i32),
            "trax_events_upload": ([vp, vp, u64, u64, vp, i32, ctypes.c_float, i32, i32, vp, vp, vp, u64], i32),
            "trax_physics_triplets": ([vp, vp, vp, vp, u32, u32, vp, vp, vp, u64, vp], i32),
            "trax_physics_triplets_device": ([vp, vp, vp, u64, vp], i32),
            "trax_physics_tracks_device": ([vp, u64, vp], i32),
            "trax_physics_tracks": ([vp, vp, u64, vp, vp, vp, vp, u64, vp], i32),
            "trax_geometry_from_files": ([ctypes.c_char_p, ctypes.c_char_p, u32, vp, vp], i32),
            "trax_host_alloc": ([ctypes.c_size_t], vp),
            "trax_host_free": ([vp], None),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
        return L


MATH_CODES = {"atan2": 0, "acos": 1, "atan": 2, "asinh": 3, "log": 4, "div": 5, "sqrt": 6, "floor": 7,
              "f2u_sat": 8, "f2i_sat": 9, "cuda_atan2f": 10, "cuda_acosf": 11, "cuda_atanf": 12,
              "cuda_asinhf": 13, "cuda_logf": 14}


def math_eval(fn: str, a: np.ndarray, b: Optional[np.ndarray] = None, device: int = 0) -> np.ndarray:
    """trax_math_eval: the library's math (or CUDA's own, "cuda_*") on the
    device; f2u_sat / f2i_sat results come back as the integers' bits in a
    float32 array."""
    L = load()
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = None if b is None else np.ascontiguousarray(b, dtype=np.float32)
    out = np.zeros_like(a)
    rc = L.trax_math_eval(device, MATH_CODES[fn], _p(a), _p(b), _p(out), a.size)
    if rc != 0:
        raise TraxError(rc, f"trax_math_eval({fn}) failed")
    return out


def pinned_empty(shape, dtype) -> np.ndarray:
    """A numpy array in page-locked host memory (trax_host_alloc), freed with the array."""
    L = load()
    dt = np.dtype(dtype)
    n = int(np.prod(shape)) * dt.itemsize
    ptr = L.trax_host_alloc(max(n, 1))
    if not ptr:
        raise MemoryError(f"trax_host_alloc({n}) failed")
    buf = (ctypes.c_char * max(n, 1)).from_address(ptr)
    arr = np.frombuffer(buf, dtype=dt, count=int(np.prod(shape))).reshape(shape)
    weakref.finalize(buf, L.trax_host_free, ptr)
    return arr


def _p(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data


@dataclasses.dataclass
class BatchStats:
    n_hits: int
    n_pairs: int
    n_candidates: int
    n_triplets: int
    n_links: int
    n_connectable: int
    n_non_connectable: int
    n_track_entries: int
    n_pair_sentinels: int
    n_candidate_sentinels: int
    kernel_launches: int
    device_ms: float
    graph_captures: int = 0


class Context:
    """One trax_ctx: a CUDA stream and the device buffers of one batch."""

    def __init__(self, device: int = 0):
        self._L = load()
        h = ctypes.c_void_p()
        rc = self._L.trax_create(ctypes.byref(h), device)
        if rc != TRAX_OK:
            raise TraxError(rc, "trax_create failed (no usable CUDA device?)")
        self._h = h
        self._keep = []
        self.n_lt = 0
        self.n_events = 0
        self.n_layers = 0
        self.n_hits = 0
        self.n_z = 0
        self.n_phi = 0
        self.n_fit = 0

    # ------------------------------------------------------------ plumbing
    def _check(self, rc: int):
        if rc != TRAX_OK:
            raise TraxError(rc, self._L.trax_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._L.trax_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -------------------------------------------------------- configuration
    def set_layer_triplets(self, lts, min_pt: float):
        arr = (LayerTripletC * len(lts))()
        for i, lt in enumerate(lts):
            for f in LayerTripletC._fields_:
                setattr(arr[i], f[0], getattr(lt, f[0]))
        self._check(self._L.trax_set_layer_triplets(self._h, ctypes.cast(arr, ctypes.c_void_p), len(lts), min_pt))
        self.n_lt = len(lts)

    def set_geometry(self, min_r: np.ndarray, max_r: np.ndarray):
        a = np.ascontiguousarray(min_r, dtype=np.float32)
        b = np.ascontiguousarray(max_r, dtype=np.float32)
        self._check(self._L.trax_set_geometry(self._h, _p(a), _p(b), a.size))

    def set_grid(self, n_z: int, n_phi: int):
        self._check(self._L.trax_set_grid(self._h, n_z, n_phi))
        self.n_z, self.n_phi = n_z, n_phi

    def upload(self, batch):
        """Configuration and hits of an EventBatch (trax_gb300.events)."""
        self.set_layer_triplets(batch.lts, batch.min_pt)
        self.set_geometry(batch.min_r, batch.max_r)
        self.set_grid(batch.n_z, batch.n_phi)
        self.upload_hits(batch)

    def upload_hits(self, batch):
        cols = [np.ascontiguousarray(getattr(batch, k), dtype=dt) for k, dt in (
            ("x", np.float32), ("y", np.float32), ("z", np.float32), ("layer", np.uint32),
            ("det_id", np.uint32), ("hit_id", np.uint32), ("event", np.uint32))]
        soa = HitsSoaC(*[_p(c) for c in cols])
        eo = np.ascontiguousarray(batch.event_offsets, dtype=np.uint32)
        lh = np.ascontiguousarray(batch.layer_hits.reshape(-1), dtype=np.uint32)
        lo = np.ascontiguousarray(batch.layer_offsets.reshape(-1), dtype=np.uint32)
        self._check(self._L.trax_upload_hits(self._h, ctypes.byref(soa), batch.n_hits, _p(eo), _p(lh), _p(lo),
                                             batch.n_events, batch.n_layers))
        self.n_events, self.n_layers, self.n_hits = batch.n_events, batch.n_layers, batch.n_hits

    # --------------------------------------------------------------- stages
    def grid_build(self):
        self._check(self._L.trax_grid_build(self._h))

    def set_tracklets(self, h1: np.ndarray, h2: np.ndarray, h3: np.ndarray):
        """Caller triplets over the uploaded hits (input order) for the linking stages."""
        a, b, c = (np.ascontiguousarray(v, dtype=np.uint32) for v in (h1, h2, h3))
        self._check(self._L.trax_set_tracklets(self._h, _p(a), _p(b), _p(c), a.size))

    def _count(self, fn, *args) -> int:
        n = ctypes.c_uint64()
        self._check(fn(self._h, *args, ctypes.byref(n)))
        return int(n.value)

    def pair_gen(self) -> int:
        return self._count(self._L.trax_pair_gen)

    def triplet_predict(self) -> int:
        return self._count(self._L.trax_triplet_predict)

    def triplet_filter(self) -> int:
        return self._count(self._L.trax_triplet_filter)

    def connectivity(self, d_eta_cut: float) -> int:
        return self._count(self._L.trax_connectivity, ctypes.c_float(d_eta_cut))

    def circle_fit(self):
        self._check(self._L.trax_circle_fit(self._h))

    def cellular_automaton(self) -> int:
        return self._count(self._L.trax_cellular_automaton)

    def circle_fit_on(self, valid_idx) -> np.ndarray:
        """TrackletCircleFitter::run on the caller's index list; returns pt of every triplet."""
        idx = np.ascontiguousarray(valid_idx, dtype=np.uint32)
        self._check(self._L.trax_circle_fit_on(self._h, _p(idx) if idx.size else None, idx.size))
        n = self.stats().n_triplets
        pt = np.zeros(max(n, 1), dtype=np.float32)
        self._check(self._L.trax_get_pt(self._h, _p(pt)))
        return pt[:n]

    def cellular_automaton_on(self, basis, follower, pt):
        """CellularAutomaton::run on the caller's links and pt; returns (states, tracks, track offsets)."""
        b = np.ascontiguousarray(basis, dtype=np.uint32)
        f = np.ascontiguousarray(follower, dtype=np.uint32)
        p = np.ascontiguousarray(pt, dtype=np.float32)
        n = ctypes.c_uint64()
        self._check(self._L.trax_cellular_automaton_on(self._h, _p(b), _p(f), b.size, _p(p), p.size,
                                                        ctypes.byref(n)))
        return self.tracks()

    def seed_batch(self, use_graph: bool = True, run_linking: bool = True, d_eta_cut: float = 0.0256) -> BatchStats:
        opts = BatchOptsC(int(use_graph), int(run_linking), d_eta_cut)
        st = BatchStatsC()
        self._check(self._L.trax_seed_batch(self._h, ctypes.byref(opts), ctypes.byref(st)))
        return BatchStats(*[getattr(st, f[0]) for f in BatchStatsC._fields_])

    def set_block_sizes(self, pair_threads: int, predict_threads: int, filter_threads: int):
        self._check(self._L.trax_set_block_sizes(self._h, pair_threads, predict_threads, filter_threads))

    def set_pairs_per_thread(self, k: int):
        """Pairs per thread of the prediction's count pass (1, 2 or 4)."""
        self._check(self._L.trax_set_pairs_per_thread(self._h, k))

    def set_candidate_slots(self, k: int):
        """Candidates captured per pair by the prediction count (4, 8, 16, 32; 0: automatic)."""
        self._check(self._L.trax_set_candidate_slots(self._h, k))

    def candidate_slots(self) -> int:
        """The number of captured candidates per pair in effect."""
        k = ctypes.c_uint32()
        self._check(self._L.trax_get_candidate_slots(self._h, ctypes.byref(k)))
        return int(k.value)

    def set_fine_rows(self, f: int):
        """Rows of the prediction count's fine z grid per grid row (0: none, 2, 4, 8, 16)."""
        self._check(self._L.trax_set_fine_rows(self._h, f))

    def fine_rows(self) -> int:
        k = ctypes.c_uint32()
        self._check(self._L.trax_get_fine_rows(self._h, ctypes.byref(k)))
        return int(k.value)

    def pairs_per_thread(self) -> int:
        k = ctypes.c_uint32()
        self._check(self._L.trax_get_pairs_per_thread(self._h, ctypes.byref(k)))
        return int(k.value)

    def launch_config(self) -> Dict[str, int]:
        """Current grid and block sizes: n_z, n_phi, pair/predict/filter threads."""
        a = np.zeros(5, dtype=np.uint32)
        self._check(self._L.trax_get_launch_config(self._h, _p(a)))
        return dict(zip(("n_z", "n_phi", "pair_threads", "predict_threads", "filter_threads"), a.tolist()))

    def autotune(self, cache_path: Optional[str] = None, search_grid: bool = True, run_linking: bool = True,
                 replays: int = 3) -> Dict[str, float]:
        """trax_autotune: time graph replays over grid and block sizes, keep the fastest."""
        opts = TuneOptsC(int(search_grid), int(run_linking), int(replays))
        res = TuneResultC()
        path = None if cache_path is None else os.fsencode(cache_path)
        self._check(self._L.trax_autotune(self._h, path, ctypes.byref(opts), ctypes.byref(res)))
        out = {f[0]: getattr(res, f[0]) for f in TuneResultC._fields_}
        self.n_z, self.n_phi = out["n_z"], out["n_phi"]
        return out

    # ------------------------------------------------ differentiable fit
    def fit_prepare(self, sigma_z: float = 0.0, sigma_tip=None, truth_only: bool = False) -> int:
        """trax_fit_prepare: freeze the fit rows of the current triplets; returns their number."""
        o = FitOptsC()
        o.sigma_z = sigma_z
        for k, v in enumerate(sigma_tip or []):
            o.sigma_tip[k] = v
        o.truth_only = int(truth_only)
        n = ctypes.c_uint64()
        self._check(self._L.trax_fit_prepare(self._h, ctypes.byref(o), ctypes.byref(n)))
        self.n_fit = int(n.value)
        return self.n_fit

    def fit_forward(self, align: np.ndarray, params: bool = False):
        """(chi2, params [n_fit, 4] or None) at align [n_layers, 3] = (dr, dz, dphi)."""
        a = np.ascontiguousarray(align, dtype=np.float64).ravel()
        chi2 = ctypes.c_double()
        p = np.zeros((max(self.n_fit, 1), 4), dtype=np.float32) if params else None
        self._check(self._L.trax_fit_forward(self._h, _p(a), ctypes.byref(chi2), _p(p)))
        return chi2.value, (p[:self.n_fit] if params else None)

    def fit_backward(self, align: np.ndarray, hits: bool = False, squares: bool = False):
        """(chi2, d chi2/d align [n_layers, 3], d chi2/d hits [n_hits, 3] or None), plus the
        approximate Gauss-Newton diagonal [n_layers, 3] when `squares`."""
        a = np.ascontiguousarray(align, dtype=np.float64).ravel()
        chi2 = ctypes.c_double()
        g = np.zeros_like(a)
        g2 = np.zeros_like(a) if squares else None
        gh = np.zeros((max(self.n_hits, 1), 3), dtype=np.float32) if hits else None
        self._check(self._L.trax_fit_backward(self._h, _p(a), ctypes.byref(chi2), _p(g), _p(g2), _p(gh)))
        out = (chi2.value, g.reshape(-1, 3), (gh[:self.n_hits] if hits else None))
        return out + (g2.reshape(-1, 3),) if squares else out

    def apply_alignment(self, align: np.ndarray):
        """trax_apply_alignment: correct the uploaded hits in place (rerun the chain afterwards)."""
        a = np.ascontiguousarray(align, dtype=np.float64).ravel()
        self._check(self._L.trax_apply_alignment(self._h, _p(a)))

    def fit_rows(self):
        """(triplet index of every fit row, sigma_tip per layer triplet)."""
        r = np.zeros(max(self.n_fit, 1), dtype=np.uint32)
        s = np.zeros(16, dtype=np.float32)
        self._check(self._L.trax_fit_get_rows(self._h, _p(r), _p(s)))
        return r[:self.n_fit], s[:self.n_lt]

    def stats(self) -> BatchStats:
        st = BatchStatsC()
        self._check(self._L.trax_get_stats(self._h, ctypes.byref(st)))
        return BatchStats(*[getattr(st, f[0]) for f in BatchStatsC._fields_])

    STAGES = ["grid", "pairs", "predict", "filter", "connectivity", "circle_fit", "ca"]
    KERNELS = ["grid_build", "pair_count", "pair_store", "predict_count", "predict_store", "filter",
               "filter_store", "connectivity_count", "connectivity_store"]

    def timings(self):
        """(stage ms, kernel ms) of the last run, from CUDA events; -1 = not run."""
        s = np.zeros(len(self.STAGES), dtype=np.float32)
        k = np.zeros(len(self.KERNELS), dtype=np.float32)
        self._check(self._L.trax_get_timings(self._h, _p(s), _p(k)))
        return dict(zip(self.STAGES, s.tolist())), dict(zip(self.KERNELS, k.tolist()))

    def set_wait_limit(self, polls: int = 0, skip_publish_tile: int = 0xFFFFFFFF):
        """Bounded-wait settings of this context's scans: polls per look-back wait
        (0: the default) and a tile that publishes nothing (a test fault; 0xffffffff: none)."""
        self._check(self._L.trax_set_wait_limit(self._h, polls))
        self._check(self._L.trax_debug_skip_publish(self._h, skip_publish_tile))

    def prefix_sum(self, data: np.ndarray) -> np.ndarray:
        a = np.ascontiguousarray(data, dtype=np.uint32).copy()
        self._check(self._L.trax_prefix_sum(self._h, _p(a), a.size))
        return a

    # -------------------------------------------------------------- results
    def _n_offsets(self) -> int:
        return self.n_events * self.n_lt + 1

    def pairs(self):
        s = self.stats()
        p = np.zeros((max(s.n_pairs, 1), 2), dtype=np.uint32)
        o = np.zeros(self._n_offsets(), dtype=np.uint32)
        self._check(self._L.trax_get_pairs(self._h, _p(p), _p(o)))
        return p[:s.n_pairs], o

    def candidates(self):
        s = self.stats()
        c = np.zeros((max(s.n_candidates, 1), 2), dtype=np.uint32)
        o = np.zeros(self._n_offsets(), dtype=np.uint32)
        self._check(self._L.trax_get_candidates(self._h, _p(c), _p(o)))
        return c[:s.n_candidates], o

    def triplets(self, out=None):
        """(h1, h2, h3, offsets); `out` = four caller arrays large enough (e.g. pinned) to fill instead."""
        s = self.stats()
        n = max(s.n_triplets, 1)
        if out is not None:
            h1, h2, h3, o = out
        else:
            h1, h2, h3 = (np.zeros(n, dtype=np.uint32) for _ in range(3))
            o = np.zeros(self._n_offsets(), dtype=np.uint32)
        self._check(self._L.trax_get_triplets(self._h, _p(h1), _p(h2), _p(h3), _p(o)))
        k = s.n_triplets
        return h1[:k], h2[:k], h3[:k], o

    def eta_pt(self):
        s = self.stats()
        n = max(s.n_triplets, 1)
        eta, pt = np.zeros(n, dtype=np.float32), np.zeros(n, dtype=np.float32)
        self._check(self._L.trax_get_triplet_eta_pt(self._h, _p(eta), _p(pt)))
        return eta[:s.n_triplets], pt[:s.n_triplets]

    def links(self):
        s = self.stats()
        b = np.zeros(max(s.n_links, 1), dtype=np.uint32)
        f = np.zeros(max(s.n_links, 1), dtype=np.uint32)
        c = np.zeros(max(s.n_connectable, 1), dtype=np.uint32)
        nc = np.zeros(max(s.n_non_connectable, 1), dtype=np.uint32)
        self._check(self._L.trax_get_links(self._h, _p(b), _p(f), _p(c), _p(nc)))
        return b[:s.n_links], f[:s.n_links], c[:s.n_connectable], nc[:s.n_non_connectable]

    def tracks(self, out=None):
        """(states, tracks, track offsets); `out` = three caller arrays large enough to fill instead."""
        s = self.stats()
        if out is not None:
            states, tr, off = out
        else:
            states = np.zeros(max(s.n_triplets, 1), dtype=np.uint32)
            tr = np.zeros(max(s.n_track_entries, 1), dtype=np.uint32)
            off = np.zeros(s.n_triplets + 1, dtype=np.uint32)
        self._check(self._L.trax_get_tracks(self._h, _p(states), _p(tr), _p(off)))
        if s.n_links == 0:
            return states[:0], tr[:0], off[:0]
        return states[:s.n_triplets], tr[:s.n_track_entries], off

    def grid(self) -> np.ndarray:
        n = ctypes.c_uint64()
        self._check(self._L.trax_get_grid(self._h, None, ctypes.byref(n)))
        g = np.zeros(max(n.value, 1), dtype=np.uint32)
        self._check(self._L.trax_get_grid(self._h, _p(g), ctypes.byref(n)))
        return g[:n.value]

    def hit_perm(self) -> np.ndarray:
        p = np.zeros(max(self.n_hits, 1), dtype=np.uint32)
        self._check(self._L.trax_get_hit_perm(self._h, _p(p)))
        return p[:self.n_hits]

    def results(self) -> Dict[str, np.ndarray]:
        """All stage outputs in the oracle's naming."""
        try:
            out = {"perm": self.hit_perm(), "grid": self.grid()}
        except TraxError:  # tracklets given directly: no grid was built
            out = {"perm": self.hit_perm(), "grid": np.zeros(0, np.uint32)}
        p, po = self.pairs()
        out["pairs"], out["pair_offsets"] = p.reshape(-1), po
        c, co = self.candidates()
        out["cands"], out["cand_offsets"] = c.reshape(-1), co
        h1, h2, h3, to = self.triplets()
        out.update(trip_h1=h1, trip_h2=h2, trip_h3=h3, trip_offsets=to)
        s = self.stats()
        if True:
            eta, pt = self.eta_pt()
            # without links the reference stops before the circle fit
            out["eta"], out["pt"] = eta, (pt if s.n_links else pt[:0])
            b, f, cn, nc = self.links()
            out.update(link_basis=b, link_follower=f, connectable=cn, non_connectable=nc)
            st, tr, toff = self.tracks()
            out.update(ca_states=st, tracks=tr, track_offsets=toff)
        return out
