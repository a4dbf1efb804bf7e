"""Python access to the CPU oracle (trax_oracle.cpp).  TEST INFRASTRUCTURE.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, as the checker.  The product path (the CUDA
library behind include/trax/trax.h) never touches it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading
from typing import Dict, List, Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(HERE, "lib")
LIB_PATH = os.path.join(LIB_DIR, "liboracle.so")
SOURCES = [os.path.join(HERE, "trax_oracle.cpp")]
DEPS = SOURCES + [os.path.join(HERE, "trax_oracle.h"),
                  os.path.join(HERE, "..", "trax_gb300", "csrc", "trax_math.h"),
                  os.path.join(HERE, "..", "trax_gb300", "csrc", "trax_math_coeffs.h")]

# -ffp-contract=off: no fused multiply-add (the default on aarch64 is to fuse);
# the float arithmetic must follow the source statement by statement.
CXXFLAGS = ["-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
            "-Wall", "-pthread"]

STATS = ["pairs", "cands", "triplets", "links", "connectable", "non_connectable", "pair_dup_slots",
         "cand_undefined_slots", "cand_truncated", "ca_iterations", "track_entries",
         "pair_tests_lo", "pair_tests_hi", "predict_tests_lo", "predict_tests_hi", "no_links",
         "ca_capped"]

FLOAT_ARRAYS = {"eta", "pt"}
ARRAYS = ["perm", "grid", "pairs", "pair_offsets", "cands", "cand_offsets", "trip_h1", "trip_h2",
          "trip_h3", "trip_offsets", "eta", "link_basis", "link_follower", "connectable",
          "non_connectable", "pt", "ca_states", "ca_best", "tracks", "track_offsets", "stats"]

_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    os.makedirs(LIB_DIR, exist_ok=True)
    newest = max(os.path.getmtime(p) for p in DEPS)
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < newest:
        tmp = LIB_PATH + f".tmp{os.getpid()}"
        subprocess.check_call(["g++"] + CXXFLAGS + ["-o", tmp] + SOURCES)
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


class _Input(ctypes.Structure):
    _fields_ = [
        ("n_hits", ctypes.c_uint32),
        ("x", ctypes.c_void_p), ("y", ctypes.c_void_p), ("z", ctypes.c_void_p),
        ("layer", ctypes.c_void_p), ("det_id", ctypes.c_void_p), ("hit_id", ctypes.c_void_p),
        ("event", ctypes.c_void_p),
        ("n_events", ctypes.c_uint32), ("n_layers", ctypes.c_uint32),
        ("event_offsets", ctypes.c_void_p), ("layer_hits", ctypes.c_void_p),
        ("layer_offsets", ctypes.c_void_p),
        ("n_z", ctypes.c_uint32), ("n_phi", ctypes.c_uint32),
        ("n_lt", ctypes.c_uint32),
        ("lt_layer1", ctypes.c_void_p), ("lt_layer2", ctypes.c_void_p), ("lt_layer3", ctypes.c_void_p),
        ("lt_dtheta_cut", ctypes.c_void_p), ("lt_sigma_z", ctypes.c_void_p),
        ("lt_dphi_cut", ctypes.c_void_p), ("lt_sigma_phi", ctypes.c_void_p),
        ("lt_tip_cut", ctypes.c_void_p), ("lt_pair_spread_z", ctypes.c_void_p),
        ("lt_z0", ctypes.c_void_p), ("lt_pair_spread_phi", ctypes.c_void_p),
        ("lt_n_candidates", ctypes.c_void_p),
        ("min_pt", ctypes.c_float),
        ("min_r", ctypes.c_void_p), ("max_r", ctypes.c_void_p),
        ("d_eta_cut", ctypes.c_float),
        ("n_threads", ctypes.c_uint32), ("event_grouping", ctypes.c_uint32),
        ("n_workers", ctypes.c_uint32), ("links_mode", ctypes.c_uint32),
    ]

LINKS_MODES = {"scan": 0, "indexed": 1, "none": 2}


def lib():
    global _lib
    with _lock:
        if _lib is None:
            path = LIB_PATH if os.path.exists(LIB_PATH) else build()
            L = ctypes.CDLL(path)
            L.oracle_run.argtypes = [ctypes.POINTER(_Input), ctypes.POINTER(ctypes.c_void_p)]
            L.oracle_run.restype = ctypes.c_int
            L.oracle_free.argtypes = [ctypes.c_void_p]
            L.oracle_last_error.restype = ctypes.c_char_p
            L.oracle_n_groups.argtypes = [ctypes.c_void_p]
            L.oracle_n_groups.restype = ctypes.c_uint32
            L.oracle_size.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_char_p]
            L.oracle_size.restype = ctypes.c_int64
            L.oracle_copy.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_char_p, ctypes.c_void_p]
            L.oracle_copy.restype = ctypes.c_int
            L.oracle_prefix_sum_blelloch.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32]
            L.oracle_math_eval.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_uint64]
            L.oracle_min_radius_curvature.argtypes = [ctypes.c_float]
            L.oracle_min_radius_curvature.restype = ctypes.c_float
            L.oracle_dphi_check.argtypes = [ctypes.c_uint64] + [ctypes.c_void_p] * 7
            L.oracle_dphi_check.restype = None
            _lib = L
        return _lib


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


class OracleError(RuntimeError):
    pass


def make_input(batch, n_threads: int = 0, event_grouping: int = 0, n_workers: int = 1, links: str = "scan"):
    """The oracle_input struct for an EventBatch, and the arrays it points into
    (keep them alive while the struct is used)."""
    keep = []

    def arr(a, dt):
        a = np.ascontiguousarray(a, dtype=dt)
        if a.size == 0:
            a = np.zeros(1, dtype=dt)
        keep.append(a)
        return _ptr(a)

    cols = batch.lt_columns()
    inp = _Input()
    inp.n_hits = batch.n_hits
    inp.x, inp.y, inp.z = arr(batch.x, np.float32), arr(batch.y, np.float32), arr(batch.z, np.float32)
    inp.layer, inp.det_id = arr(batch.layer, np.uint32), arr(batch.det_id, np.uint32)
    inp.hit_id, inp.event = arr(batch.hit_id, np.uint32), arr(batch.event, np.uint32)
    inp.n_events, inp.n_layers = batch.n_events, batch.n_layers
    inp.event_offsets = arr(batch.event_offsets, np.uint32)
    inp.layer_hits = arr(batch.layer_hits.reshape(-1), np.uint32)
    inp.layer_offsets = arr(batch.layer_offsets.reshape(-1), np.uint32)
    inp.n_z, inp.n_phi = batch.n_z, batch.n_phi
    inp.n_lt = len(batch.lts)
    inp.lt_layer1, inp.lt_layer2, inp.lt_layer3 = (arr(cols["layer1"], np.uint32), arr(cols["layer2"], np.uint32),
                                                   arr(cols["layer3"], np.uint32))
    inp.lt_dtheta_cut = arr(cols["dtheta_cut"], np.float32)
    inp.lt_sigma_z = arr(cols["sigma_z"], np.float32)
    inp.lt_dphi_cut = arr(cols["dphi_cut"], np.float32)
    inp.lt_sigma_phi = arr(cols["sigma_phi"], np.float32)
    inp.lt_tip_cut = arr(cols["tip_cut"], np.float32)
    inp.lt_pair_spread_z = arr(cols["pair_spread_z"], np.uint32)
    inp.lt_z0 = arr(cols["z0"], np.float32)
    inp.lt_pair_spread_phi = arr(cols["pair_spread_phi"], np.uint32)
    inp.lt_n_candidates = arr(cols["n_candidates"], np.uint32)
    inp.min_pt = batch.min_pt
    inp.min_r, inp.max_r = arr(batch.min_r, np.float32), arr(batch.max_r, np.float32)
    inp.d_eta_cut = batch.d_eta_cut
    inp.n_threads, inp.event_grouping, inp.n_workers = n_threads, event_grouping, n_workers
    inp.links_mode = LINKS_MODES[links]
    return inp, keep


def run(batch, n_threads: int = 0, event_grouping: int = 0, n_workers: int = 1,
        arrays: Optional[Sequence[str]] = None, links: str = "scan") -> List[Dict[str, np.ndarray]]:
    """Run the oracle over an EventBatch; one dict of arrays per event group (only
    `arrays` and the stats when given, e.g. ("stats",) for timing runs).
    links: "scan" (the reference's connectivity scan), "indexed" (the same
    result through an index, for very large events) or "none" (no linking).
    n_workers host threads run groups in parallel or, with one group, work
    inside it; the results do not depend on their number."""
    L = lib()
    inp, keep = make_input(batch, n_threads, event_grouping, n_workers, links)
    h = ctypes.c_void_p()
    rc = L.oracle_run(ctypes.byref(inp), ctypes.byref(h))
    if rc != 0:
        raise OracleError(L.oracle_last_error().decode())
    try:
        out = []
        for g in range(L.oracle_n_groups(h)):
            d = {}
            for name in (ARRAYS if arrays is None else [a for a in ARRAYS if a in arrays or a == "stats"]):
                n = L.oracle_size(h, g, name.encode())
                if n < 0:
                    continue
                dt = np.float32 if name in FLOAT_ARRAYS else np.uint32
                a = np.zeros(max(n, 1), dtype=dt)
                L.oracle_copy(h, g, name.encode(), _ptr(a))
                d[name] = a[:n]
            d["stats_dict"] = {k: int(v) for k, v in zip(STATS, d["stats"])}
            out.append(d)
        return out
    finally:
        L.oracle_free(h)


class _LinkInput(ctypes.Structure):
    _fields_ = [("n_hits", ctypes.c_uint32), ("x", ctypes.c_void_p), ("y", ctypes.c_void_p),
                ("z", ctypes.c_void_p), ("layer", ctypes.c_void_p), ("event", ctypes.c_void_p),
                ("n_events", ctypes.c_uint32), ("n_lt", ctypes.c_uint32), ("n_triplets", ctypes.c_uint32),
                ("h1", ctypes.c_void_p), ("h2", ctypes.c_void_p), ("h3", ctypes.c_void_p),
                ("d_eta_cut", ctypes.c_float)]


def link(x, y, z, layer, event, h1, h2, h3, n_events: int, n_lt: int, d_eta_cut: float) -> Dict[str, np.ndarray]:
    """Connectivity, circle fit and CA on given triplets over hits taken as they are."""
    L = lib()
    if not hasattr(L, "_link_ready"):
        L.oracle_link.argtypes = [ctypes.POINTER(_LinkInput), ctypes.POINTER(ctypes.c_void_p)]
        L.oracle_link.restype = ctypes.c_int
        L._link_ready = True
    keep = []

    def arr(a, dt):
        a = np.ascontiguousarray(a, dtype=dt)
        if a.size == 0:
            a = np.zeros(1, dtype=dt)
        keep.append(a)
        return _ptr(a)

    inp = _LinkInput(len(x), arr(x, np.float32), arr(y, np.float32), arr(z, np.float32),
                     arr(layer, np.uint32), arr(event, np.uint32), n_events, n_lt, len(h1),
                     arr(h1, np.uint32), arr(h2, np.uint32), arr(h3, np.uint32), d_eta_cut)
    h = ctypes.c_void_p()
    if L.oracle_link(ctypes.byref(inp), ctypes.byref(h)) != 0:
        raise OracleError(L.oracle_last_error().decode())
    try:
        d = {}
        for name in ARRAYS:
            n = L.oracle_size(h, 0, name.encode())
            if n < 0:
                continue
            dt = np.float32 if name in FLOAT_ARRAYS else np.uint32
            a = np.zeros(max(n, 1), dtype=dt)
            L.oracle_copy(h, 0, name.encode(), _ptr(a))
            d[name] = a[:n]
        return d
    finally:
        L.oracle_free(h)


def ca(n_triplets: int, basis, follower, pt) -> Dict[str, np.ndarray]:
    """CellularAutomaton::run alone on given links and pt."""
    L = lib()
    if not hasattr(L, "_ca_ready"):
        L.oracle_ca.argtypes = [ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p,
                                ctypes.POINTER(ctypes.c_void_p)]
        L.oracle_ca.restype = ctypes.c_int
        L._ca_ready = True
    b = np.ascontiguousarray(basis, dtype=np.uint32)
    f = np.ascontiguousarray(follower, dtype=np.uint32)
    p = np.ascontiguousarray(pt, dtype=np.float32)
    h = ctypes.c_void_p()
    if L.oracle_ca(n_triplets, _ptr(b), _ptr(f), b.size, _ptr(p), ctypes.byref(h)) != 0:
        raise OracleError(L.oracle_last_error().decode())
    try:
        d = {}
        for name in ("ca_states", "ca_best", "tracks", "track_offsets", "stats"):
            n = L.oracle_size(h, 0, name.encode())
            a = np.zeros(max(n, 1), dtype=np.uint32)
            L.oracle_copy(h, 0, name.encode(), _ptr(a))
            d[name] = a[:n]
        d["stats_dict"] = {k: int(v) for k, v in zip(STATS, d["stats"])}
        return d
    finally:
        L.oracle_free(h)


def prefix_sum_blelloch(data: np.ndarray, wg: int) -> np.ndarray:
    a = np.ascontiguousarray(data, dtype=np.uint32).copy()
    lib().oracle_prefix_sum_blelloch(_ptr(a), a.size, wg)
    return a


MATH_CODES = {"atan2": 0, "acos": 1, "atan": 2, "asinh": 3, "log": 4, "div": 5, "sqrt": 6, "floor": 7,
              "f2u_sat": 8, "f2i_sat": 9}


def math_eval(fn: str, a: np.ndarray, b: Optional[np.ndarray] = None) -> np.ndarray:
    """trax_math.h's `fn` on the CPU; f2u_sat / f2i_sat results come back as the
    integers' bits in a float32 array (view them as uint32 / int32)."""
    code = MATH_CODES[fn]
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = np.ascontiguousarray(b if b is not None else a, dtype=np.float32)
    out = np.zeros_like(a)
    lib().oracle_math_eval(code, _ptr(a), _ptr(b), _ptr(out), a.size)
    return out


def dphi_check(ux, uy, vx, vy, cut):
    """(atan2 evaluation of the dphi cut, the kernels' cross/dot decision: 1, 0 or -1 undecided)."""
    cols = [np.ascontiguousarray(a, dtype=np.float32) for a in (ux, uy, vx, vy, cut)]
    n = cols[0].size
    exact, decided = np.zeros(n, np.int32), np.zeros(n, np.int32)
    lib().oracle_dphi_check(n, *[_ptr(a) for a in cols], _ptr(exact), _ptr(decided))
    return exact, decided


def min_radius_curvature(min_pt: float) -> float:
    return float(lib().oracle_min_radius_curvature(min_pt))
