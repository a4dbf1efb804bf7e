"""Builds libtrax_gb300.so (sm_103a) in-tree with nvcc.

Every translation unit is compiled in parallel for exactly one target,
``-gencode arch=compute_103a,code=sm_103a``.  The float flags are part of the
contract with the CPU oracle: no fused multiply-add (``-fmad=false``),
IEEE division and square root, no flush-to-zero, and the host-side compiler
without FP contraction either.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "lib")
OBJ_DIR = os.path.join(LIB_DIR, "obj")
LIB_NAME = "libtrax_gb300.so"
LIB_PATH = os.path.join(LIB_DIR, LIB_NAME)
# the bounds-checked debug build (-DTRAX_BOUNDS_CHECK): every data-dependent
# hit index checked on the device, a bad one failing the call
CHECKED_OBJ_DIR = os.path.join(LIB_DIR, "obj_checked")
CHECKED_LIB_PATH = os.path.join(LIB_DIR, "libtrax_gb300_checked.so")

SOURCES = ["k_scan.cu", "k_grid.cu", "k_pairs.cu", "k_triplets.cu", "k_link.cu", "capi.cu", "tune.cu", "k_fit.cu", "host_events.cpp", "k_events.cu", "k_tracks.cu", "k_math.cu"]
HEADERS = ["trax_device.cuh", "trax_kernels.h", "trax_math.h", "trax_math_coeffs.h", "trax_stages.cuh",
           "trax_lookback.cuh", "trax_events.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17",
    "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
    "-I", CSRC, "-I", os.path.join(REPO, "include"),
]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps_mtime() -> float:
    paths = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    paths.append(os.path.join(REPO, "include", "trax", "trax.h"))
    paths.append(os.path.abspath(__file__))
    return max(os.path.getmtime(p) for p in paths)


def _compile(src: str, extra, obj_dir: str = OBJ_DIR) -> str:
    obj = os.path.join(obj_dir, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc()] + NVCC_FLAGS + list(extra) + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose_ptxas: bool = False, checked: bool = False) -> str:
    """Compile all kernels and the C ABI into trax_gb300/lib/libtrax_gb300.so
    (checked: the bounds-checked debug build, libtrax_gb300_checked.so)."""
    obj_dir = CHECKED_OBJ_DIR if checked else OBJ_DIR
    lib_path = CHECKED_LIB_PATH if checked else LIB_PATH
    os.makedirs(obj_dir, exist_ok=True)
    if not force and os.path.exists(lib_path) and os.path.getmtime(lib_path) >= _deps_mtime():
        return lib_path
    extra = (["-Xptxas", "-v"] if verbose_ptxas else []) + (["-DTRAX_BOUNDS_CHECK"] if checked else [])
    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra, obj_dir), SOURCES))
    tmp = lib_path + f".tmp{os.getpid()}"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib_path)
    return lib_path


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="--ptxas" in sys.argv, checked="--checked" in sys.argv))
