"""Runtime records in the reference's csv layout (RuntimeRecords::csvDump,
RuntimeRecord.cpp:123-192 and :382-450), so that its plotting scripts read
this implementation's timings.

One record per chain run: the batch shape, host<->device transfers and, per
stage, count / scan / store / wall / kernel milliseconds.  Records with the
same shape form a class; a row holds the class's means and standard
deviations over its runs.  Stage split (CUDA-event times of trax_get_timings):

  buildGrid            count = the fused grid kernel (count, scan and scatter in one)
  pairGen              count / store kernels; scan = the rest of the stage
  tripletPredict       count / store kernels; scan = the rest of the stage
  tripletFilter        count / store kernels; scan = the rest of the stage
  tripletConnectivityTight  count / store kernels; scan = the rest of the stage
  trackletCircleFitter store = the stage
  cellularAutomaton    count = the stage
  walltime             = the stage's device time (stages run without host waits)
"""
from __future__ import annotations

import math
from typing import Dict, List, Optional

STAGES = ["buildGrid", "pairGen", "tripletPredict", "tripletFilter", "tripletConnectivityTight",
          "trackletCircleFitter", "cellularAutomaton"]
SHAPE = ["events", "layers", "layerTriplets", "threads", "hits", "tracks"]
PARTS = ["Count", "Scan", "Store", "Walltime", "Kernel"]


def header() -> str:
    cols = SHAPE + ["n", "readTime", "readTimeVar", "readBytes", "readBytesVar", "writeTime", "writeTimeVar",
                    "writeBytes", "writeBytesVar"]
    for st in STAGES:
        for p in PARTS:
            cols += [st + p, st + p + "Var"]
    # the reference's own spelling of this one column (RuntimeRecord.cpp:170)
    i = cols.index("tripletConnectivityTightKernelVar")
    cols[i] = "tripletConnectivityTightWalltimeKernelVar"
    for p in PARTS:
        cols += ["total" + p, "total" + p + "Var"]
    return " ".join(cols)


def stage_split(stage_ms: Dict[str, float], kernel_ms: Dict[str, float]) -> Dict[str, Dict[str, float]]:
    """count / scan / store / walltime / kernel per reference stage from trax_get_timings."""
    def ms(d, k):
        v = d.get(k, -1.0)
        return 0.0 if v is None or v < 0 else float(v)
    out = {}
    pairs = {"pairGen": ("pairs", "pair_count", "pair_store"),
             "tripletPredict": ("predict", "predict_count", "predict_store"),
             "tripletFilter": ("filter", "filter", "filter_store"),
             "tripletConnectivityTight": ("connectivity", "connectivity_count", "connectivity_store")}
    g = ms(stage_ms, "grid")
    out["buildGrid"] = dict(Count=ms(kernel_ms, "grid_build") or g, Scan=0.0, Store=0.0, Walltime=g)
    for st, (s, c, w) in pairs.items():
        t, cc, ww = ms(stage_ms, s), ms(kernel_ms, c), ms(kernel_ms, w)
        out[st] = dict(Count=cc, Store=ww, Scan=max(t - cc - ww, 0.0), Walltime=t)
    f = ms(stage_ms, "circle_fit")
    out["trackletCircleFitter"] = dict(Count=0.0, Scan=0.0, Store=f, Walltime=f)
    ca = ms(stage_ms, "ca")
    out["cellularAutomaton"] = dict(Count=ca, Scan=0.0, Store=0.0, Walltime=ca)
    for v in out.values():
        v["Kernel"] = v["Count"] + v["Scan"] + v["Store"]
    return out


class RuntimeRecords:
    """Runs grouped by shape (RuntimeRecordClass); csv() gives the reference's file."""

    def __init__(self):
        self._classes: List[dict] = []

    def add(self, events: int, layers: int, layer_triplets: int, threads: int, hits: int, tracks: int,
            stage_ms: Dict[str, float], kernel_ms: Dict[str, float], read_ms: float = 0.0, read_bytes: int = 0,
            write_ms: float = 0.0, write_bytes: int = 0):
        shape = (events, layers, layer_triplets, threads, hits, tracks)
        split = stage_split(stage_ms, kernel_ms)
        values = [read_ms, float(read_bytes), write_ms, float(write_bytes)]
        for st in STAGES:
            values += [split[st][p] for p in PARTS]
        for p in PARTS:
            values.append(sum(split[st][p] for st in STAGES))
        for c in self._classes:
            if c["shape"] == shape:
                c["runs"].append(values)
                return
        self._classes.append({"shape": shape, "runs": [values]})

    def csv(self) -> str:
        lines = [header()]
        for c in self._classes:
            runs = c["runs"]
            n = len(runs)
            row = [str(v) for v in c["shape"]] + [str(n)]
            for k in range(len(runs[0])):
                vals = [r[k] for r in runs]
                mean = sum(vals) / n
                dev = math.sqrt(sum((v - mean) ** 2 for v in vals) / (n - 1)) if n > 1 else 0.0
                row += [f"{mean:.6g}", f"{dev:.6g}"]
            lines.append(" ".join(row))
        return "\n".join(lines) + "\n"
