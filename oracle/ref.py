"""Python access to oracle/_ref/libtraxref.so: the reference's own OpenCL kernel
text run on the CPU (ref_extract.py, ref_shim.h, ref_driver.cpp).

TEST INFRASTRUCTURE ONLY, like the rest of ``oracle/``.  The library exists
only where the reference's sources were available when it was generated;
``available()`` says whether it can be loaded, and the tests that use it skip
otherwise.
"""
from __future__ import annotations

import ctypes
import os
import threading
from typing import Dict, Optional

import numpy as np

from oracle import oracle, ref_extract

STATS = ["pair_sentinels", "cand_sentinels", "ca_iterations", "no_links", "ca_chain_broken",
         "grid_count_local", "grid_store_variant", "pair_count_local"]
FLOAT_ARRAYS = {"hx", "hy", "hz", "eta", "pt"}
ARRAYS = ["hx", "hy", "hz", "hlayer", "hdet", "hhit", "hevt", "grid", "pairs", "pair_offsets", "cands",
          "cand_offsets", "trip_h1", "trip_h2", "trip_h3", "trip_offsets", "eta", "link_basis", "link_follower",
          "connectable", "non_connectable", "pt", "ca_states", "ca_best", "tracks", "track_offsets", "stats"]

# A GTX 660's local memory (the reference's published GPU); 0 selects the
# no-local-memory kernel variants.
GTX660_LOCAL_MEM = 48 * 1024
# The local memory an OpenCL CPU device reports (32 KB on Intel's runtime).
CPU_LOCAL_MEM = 32 * 1024

_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    return ref_extract.build(force)


def available() -> bool:
    try:
        return lib() is not None
    except OSError:
        return False


def lib():
    global _lib
    with _lock:
        if _lib is None:
            path = ref_extract.LIB_PATH
            if not os.path.exists(path):
                path = ref_extract.build()
            if not path:
                return None
            L = ctypes.CDLL(path)
            L.ref_run.argtypes = [ctypes.POINTER(oracle._Input), ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                  ctypes.POINTER(ctypes.c_void_p)]
            L.ref_run.restype = ctypes.c_int
            L.ref_last_error.restype = ctypes.c_char_p
            L.ref_size.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
            L.ref_size.restype = ctypes.c_int64
            L.ref_copy.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p]
            L.ref_copy.restype = ctypes.c_int
            L.ref_free.argtypes = [ctypes.c_void_p]
            L.ref_prefix_sum.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32]
            L.ref_track_metrics.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_uint64] + \
                [ctypes.c_void_p] * 5
            L.ref_track_metrics.restype = None
            L.ref_ca.argtypes = [ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p,
                                 ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(ctypes.c_void_p)]
            L.ref_ca.restype = ctypes.c_int
            L.ref_run_events.argtypes = [ctypes.POINTER(oracle._Input), ctypes.c_uint32, ctypes.c_uint32,
                                         ctypes.c_uint32, ctypes.c_void_p]
            L.ref_run_events.restype = ctypes.c_int
            _lib = L
        return _lib


def run(batch, n_threads: int = 1, local_mem: int = GTX660_LOCAL_MEM, max_ca_iterations: int = 1000
        ) -> Dict[str, np.ndarray]:
    """Runs the reference's kernels over all events of `batch` as one event group
    with exec.threads = n_threads.  Arrays as in oracle.run, plus the grid-ordered
    hit columns (hx, hy, hz, hlayer, hdet, hhit, hevt) in place of a permutation."""
    L = lib()
    if L is None:
        raise RuntimeError("the reference kernel library is not built (reference sources absent)")
    inp, keep = oracle.make_input(batch)
    h = ctypes.c_void_p()
    if L.ref_run(ctypes.byref(inp), n_threads, local_mem, max_ca_iterations, ctypes.byref(h)) != 0:
        raise RuntimeError(L.ref_last_error().decode())
    try:
        out: Dict[str, np.ndarray] = {}
        for name in ARRAYS:
            n = L.ref_size(h, name.encode())
            if n < 0:
                continue
            dt = np.float32 if name in FLOAT_ARRAYS else np.uint32
            a = np.zeros(max(n, 1), dtype=dt)
            L.ref_copy(h, name.encode(), a.ctypes.data)
            out[name] = a[:n]
        out["stats_dict"] = {k: int(v) for k, v in zip(STATS, out["stats"])}
        return out
    finally:
        L.ref_free(h)


def ca(n_triplets: int, basis, follower, pt, n_threads: int = 1, max_ca_iterations: int = 100000
       ) -> Dict[str, np.ndarray]:
    """The reference's CA kernels alone on given links and pt."""
    L = lib()
    b = np.ascontiguousarray(basis, dtype=np.uint32)
    f = np.ascontiguousarray(follower, dtype=np.uint32)
    p = np.ascontiguousarray(pt, dtype=np.float32)
    h = ctypes.c_void_p()
    if L.ref_ca(n_triplets, b.ctypes.data, f.ctypes.data, b.size, p.ctypes.data, n_threads, max_ca_iterations,
                ctypes.byref(h)) != 0:
        raise RuntimeError(L.ref_last_error().decode())
    try:
        out: Dict[str, np.ndarray] = {}
        for name in ("ca_states", "ca_best", "tracks", "track_offsets", "stats"):
            n = L.ref_size(h, name.encode())
            a = np.zeros(max(n, 1), dtype=np.uint32)
            L.ref_copy(h, name.encode(), a.ctypes.data)
            out[name] = a[:n]
        out["stats_dict"] = {k: int(v) for k, v in zip(STATS, out["stats"])}
        return out
    finally:
        L.ref_free(h)


def run_events(batch, workers: int, n_threads: int = 1, local_mem: int = CPU_LOCAL_MEM) -> np.ndarray:
    """The reference's kernels over every event of `batch`, each event its own
    group, on `workers` host threads; returns the triplet count of each event."""
    L = lib()
    inp, keep = oracle.make_input(batch)
    out = np.zeros(batch.n_events, dtype=np.uint64)
    if L.ref_run_events(ctypes.byref(inp), n_threads, local_mem, workers, out.ctypes.data) != 0:
        raise RuntimeError(L.ref_last_error().decode())
    return out


def track_metrics(tracks, track_offsets, h1, h2, h3, hit_track_id) -> dict:
    """The reference's own track evaluation (TripletBuilder.cpp: extractTracks,
    cloneRemoval, splitRealFakeTracks, findUniqueRealTracks) on a CA output:
    the counts printTracks reports."""
    L = lib()
    cols = [np.ascontiguousarray(a, dtype=np.uint32) for a in (tracks, track_offsets, h1, h2, h3, hit_track_id)]
    cols = [c if c.size else np.zeros(1, np.uint32) for c in cols]
    out = np.zeros(5, np.uint64)
    n_entries, n_offsets = np.asarray(tracks).size, np.asarray(track_offsets).size
    L.ref_track_metrics(cols[0].ctypes.data, n_entries, cols[1].ctypes.data, n_offsets, cols[2].ctypes.data,
                        cols[3].ctypes.data, cols[4].ctypes.data, cols[5].ctypes.data, out.ctypes.data)
    return dict(zip(("total", "filtered", "valid", "valid_unique", "fakes"), (int(v) for v in out)))


def prefix_sum(data: np.ndarray, wg: int) -> np.ndarray:
    """The reference's recursive scan kernels (PrefixSum.h:58-248) over `data`."""
    a = np.ascontiguousarray(data, dtype=np.uint32).copy()
    lib().ref_prefix_sum(a.ctypes.data, a.size, wg)
    return a
