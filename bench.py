#!/usr/bin/env python
"""Benchmark of the triplet-seeding chain on GB300.

Workload: 1000 ttbar-like events with uneven sizes (tracks ~ Poisson(lambda),
lambda ~ U[300, 3000]; 10 barrel layers, 6 layer triplets), seeded synthetic
data (the reference's own event files are not distributed).  One step is the
whole chain -- grid build, pairs, prediction, filter, connectivity, circle fit,
cellular automaton -- over the full batch, replayed from a CUDA graph.

value      events/s with the hits already resident in HBM, device time from
           CUDA events around each graph launch (inputs: ~270 MB of hits,
           larger than the 129 MB L2, so no L2 flush is needed between steps)
e2e        the same metric through the C ABI from host buffers: upload of the
           hit columns, the chain, and the download of the triplets and tracks
           inside the timed region (host wall clock, synchronized)
plain      the per-event launch structure of the reference (one event per
           stage call, host-synced count/scan/store) over the first events
roofline   the dominant kernel's algorithmic bytes / its CUDA-event time
           against the measured HBM copy bandwidth
cpu_baseline  the reference's own OpenCL kernel text compiled for the CPU
           (oracle/_ref, built where the reference's sources were available;
           "kind": "reference"), else the CPU oracle that restates it
           ("kind": "port"), on a bounded sample on all host cores
parity     every event of the batch against the oracle run on it alone

Both arms run the workload's grid (250 x 48, the autotuner's grid choice for
this workload on GB300); the GPU arm autotunes its block sizes live, and
searches the grid too with --tune-grid.

Multi-GPU (torchrun): every rank processes its own 1000-event batch on its
own GPU (events are independent; no collective on the data path); value is
all ranks' events over the slowest rank's time.

--impl reference times the reference's CPU path on the host cores instead
(rank 0 only): oracle/_ref when built, else the oracle port.
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "events/s & triplets/s on 1 GB300, batched vs per-event, bit-exact triplet sets"
CONFIG = 2


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--events", type=int, default=1000)
    p.add_argument("--plain-events", type=int, default=48)
    p.add_argument("--cpu-sample", type=int, default=128)
    p.add_argument("--e2e-steps", type=int, default=5)
    p.add_argument("--e2e-pipe-steps", type=int, default=25,
                   help="steps per context of the pipelined end-to-end run (enough to amortise its fill and drain)")
    p.add_argument("--e2e-contexts", type=int, default=4,
                   help="contexts (each with its own stream and host thread) that overlap copies with kernels")
    p.add_argument("--no-plain", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-parity", action="store_true")
    p.add_argument("--no-align", action="store_true", help="skip the alignment (differentiable fit) measurement")
    p.add_argument("--no-config3", action="store_true", help="skip the high-occupancy (config 3) measurement")
    p.add_argument("--config3-steps", type=int, default=10)
    p.add_argument("--config3-events", type=int, default=16, help="events of the config 3 batch (16: the full workload)")
    p.add_argument("--config3-fine", type=int, default=8,
                   help="fine z rows per grid row of config 3's prediction count (0: none)")
    p.add_argument("--runtime-csv", default=None, help="write the timed steps as the reference's runtime csv")
    p.add_argument("--grid", default=None, help="z x phi sectors, e.g. 200x256 (default: autotuned)")
    p.add_argument("--no-tune", action="store_true", help="skip the autotuner (grid of the workload, default blocks)")
    p.add_argument("--tune-grid", action="store_true",
                   help="let the autotuner search the grid too (the reference arm keeps the workload's grid)")
    p.add_argument("--tune-cache", default=None, help="JSON cache file of the autotuner")
    p.add_argument("--blocks", default=None,
                   help="block sizes of the pair, prediction and filter kernels, e.g. 256,64,256 (skips their tuning)")
    return p.parse_args()


# ----------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ["index", "clocks.sm", "clocks.max.sm", "power.draw", "clocks_event_reasons.active",
              "clocks_event_reasons.hw_slowdown", "clocks_event_reasons.hw_thermal_slowdown",
              "clocks_event_reasons.sw_thermal_slowdown", "clocks_event_reasons.sw_power_cap"]

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + ",".join(self.FIELDS),
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) != len(self.FIELDS):
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for k, name in enumerate(names):
                if parts[5 + k].lower() in ("active", "1", "yes"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------ CPU baseline
def cpu_engine():
    """The reference's CPU path to time: its own kernel text compiled for the
    CPU (oracle/_ref) when that was built, else the oracle port."""
    from oracle import ref
    if ref.available():
        return "reference"
    return "port"


def cpu_run(sample, cores: int, kind: str) -> int:
    """Runs the CPU path over `sample`, one event per group on `cores` host
    threads; returns the number of triplets."""
    if kind == "reference":
        from oracle import ref
        return int(ref.run_events(sample, workers=cores).sum())
    from oracle import oracle
    res = oracle.run(sample, event_grouping=1, n_workers=cores, arrays=("stats",))
    return sum(r["stats_dict"]["triplets"] for r in res)


CPU_KIND_NOTE = {
    "reference": "the reference's own OpenCL kernel text (src/algorithms/*.h KERNEL_CLASS blocks) compiled for the "
                 "CPU against a work-item shim, driven by its host sequences; exec.threads 1, a 32 KB CPU device",
    "port": "the oracle's restatement of the reference kernels (the reference's kernel text was not built here)",
}


def host_cpu() -> dict:
    """The host's processor: logical CPUs, architecture and model name."""
    import platform
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    return {"logical_cpus": os.cpu_count() or 1, "machine": platform.machine(), "model": model}


def cpu_baseline(batch, n_events: int, single_events: int = 8):
    sample = batch.subset(range(min(n_events, batch.n_events)))
    cores = os.cpu_count() or 1
    kind = cpu_engine()
    t0 = time.perf_counter()
    trip = cpu_run(sample, cores, kind)
    dt = time.perf_counter() - t0
    # the same path on one host thread, over the first few events
    one = batch.subset(range(min(single_events, batch.n_events)))
    t1 = time.perf_counter()
    trip1 = cpu_run(one, 1, kind)
    dt1 = time.perf_counter() - t1
    return {"value": round(sample.n_events / dt, 3), "unit": "events/s", "cores": cores, "kind": kind,
            "sample": f"first {sample.n_events} events of the 1000-event workload at the same grid "
                      f"({batch.n_z}x{batch.n_phi}), one event per group, {cores} host threads, {dt:.2f} s wall; "
                      + CPU_KIND_NOTE[kind],
            "triplets_per_s": round(trip / dt, 1),
            "single_thread": {"value": round(one.n_events / dt1, 3), "unit": "events/s",
                              "triplets_per_s": round(trip1 / dt1, 1),
                              "sample": f"first {one.n_events} events, one host thread, {dt1:.2f} s wall"},
            "host": host_cpu()}


def peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# Algorithmic bytes of the timed kernels: compulsory streams only (each input
# array read once, each output written once), from the sizes of the run.  The
# packed (x, y, z, phi) hit array is 16 B per hit, the grid 4 B per cell; the
# pair kernels read the cells of the inner layers only, the prediction those
# of the third layers (cells_inner, cells_third: the layers' cells of all
# events).
def kernel_bytes(name, st, n_tasks, n_hits, cells, cells_inner=None, cells_third=None):
    P, Cc, T = st.n_pairs, st.n_candidates, st.n_triplets
    ci = cells if cells_inner is None else cells_inner
    c3 = cells if cells_third is None else cells_third
    return {
        "grid_build": 56 * n_hits + 4 * cells,
        "pair_count": 16 * n_hits + 4 * ci + 4 * n_tasks,
        "pair_store": 16 * n_hits + 4 * ci + 4 * n_tasks + 8 * P,
        "predict_count": 16 * n_hits + 4 * c3 + 8 * P + 4 * P,
        "predict_store": 8 * P + 4 * P + 8 * Cc,
        "filter": 16 * n_hits + 8 * P + 8 * Cc + 4 * Cc,
        "filter_store": 8 * P + 8 * Cc + 4 * Cc + 12 * T,
        "connectivity_count": 12 * T + 4 * T + 4 * T,
        "connectivity_store": 12 * T + 8 * st.n_links,
    }.get(name, 0)


# DRAM bytes per unit of work of the kernels that can dominate the chain,
# from an ncu capture (dram__bytes_read.sum + dram__bytes_write.sum) of the
# same chain on the first 300 events of the workload; a full launch scales
# them by its units (traffic grows with pairs, candidates and hits).
TRAFFIC_PER_UNIT = {  # by grid (nZ x nPhi): the grid changes the cells read and the hits visited
    "150x64": {"predict_count": ("pairs", 32.5), "filter": ("candidates", 27.3), "grid_build": ("hits", 97.0)},
    "200x64": {"predict_count": ("pairs", 32.7), "filter": ("candidates", 27.3), "grid_build": ("hits", 110.9)},
    "250x48": {"predict_count": ("pairs", 32.2), "filter": ("candidates", 30.5), "grid_build": ("hits", 107.6)},
    "300x48": {"predict_count": ("pairs", 32.9), "filter": ("candidates", 27.1), "grid_build": ("hits", 118.4)},
    "250x32": {"predict_count": ("pairs", 32.2), "filter": ("candidates", 27.2), "grid_build": ("hits", 90.4)},
    "200x48": {"predict_count": ("pairs", 32.4), "filter": ("candidates", 27.2), "grid_build": ("hits", 97.2)},
    "250x64": {"predict_count": ("pairs", 33.0), "filter": ("candidates", 27.2), "grid_build": ("hits", 125.0)},
}


# warp instructions per unit of work (ncu smsp__inst_executed.sum of the same
# 300-event capture / its units): the dominant kernels are issue-bound, so
# their position against the SMs' issue rate is reported beside the HBM one.
# Captured for the current prediction kernel at the workload's grid only.
INST_PER_UNIT = {"250x48": {"predict_count": ("pairs", 23.55)}}


def kernel_issue(name, st, ms, clk, device, grid):
    """Issue roofline of a kernel: warp instructions per second against one
    instruction per cycle on each of the SMs' four schedulers at the SM clock
    seen during the timed region."""
    import torch
    table = INST_PER_UNIT.get(grid, {})
    if name not in table or not ms:
        return None
    unit, per = table[name]
    n = {"pairs": st.n_pairs}[unit]
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    mhz = clk.get("sm_mhz") or clk.get("sm_max_mhz")
    if not mhz:
        return None
    achieved = per * n / (ms * 1e-3)
    peak = sms * 4 * mhz * 1e6
    return {"achieved": round(achieved / 1e9, 1), "peak": round(peak / 1e9, 1), "unit": "G warp inst/s",
            "frac": round(achieved / peak, 4),
            "note": f"{per} warp instructions per {unit[:-1]} (ncu, 300-event case, grid {grid}) x units / live "
                    f"kernel time; "
                    f"peak = {sms} SMs x 4 schedulers x {mhz:.0f} MHz"}


def kernel_traffic(name, st, n_hits, grid):
    table = TRAFFIC_PER_UNIT.get(grid, {})
    if name not in table:
        return None
    unit, per = table[name]
    n = {"pairs": st.n_pairs, "candidates": st.n_candidates, "hits": n_hits}[unit]
    return int(per * n)


def chain_bytes(st, n_hits, cells, n_layers):
    # per-batch algorithmic bytes of the whole chain: hits read and written by
    # the grid build, every intermediate array written once and read once,
    # the CA's per-level link and state traffic
    P, Cc, T, Lk = st.n_pairs, st.n_candidates, st.n_triplets, st.n_links
    return (56 * n_hits + 4 * cells + 16 * P + 16 * Cc + 24 * T + 4 * T + 16 * Lk + 8 * st.n_connectable
            + (8 * Lk + 8 * T) * max(1, n_layers))


def run_plain(ctx, batch, n_events):
    """Reference launch structure: one event per call, every stage host-synced."""
    from trax_gb300 import capi  # noqa: F401
    times = []
    trip = 0
    for e in range(min(n_events, batch.n_events)):
        sub = batch.subset([e])
        ctx.upload(sub)
        t0 = time.perf_counter()
        ctx.grid_build()
        ctx.pair_gen()
        ctx.triplet_predict()
        trip += ctx.triplet_filter()
        if ctx.connectivity(batch.d_eta_cut):
            ctx.circle_fit()
            ctx.cellular_automaton()
        times.append(time.perf_counter() - t0)
    total = sum(times)
    return {"value": round(len(times) / total, 2), "unit": "events/s", "events": len(times),
            "triplets_per_s": round(trip / total, 1),
            "structure": "one event per stage call; host-synced count -> scan -> read total -> store"}


class WholeBatchOracle:
    """The oracle on the whole batch as one event group, in a background host
    thread (the call releases the GIL): links, connectable lists, pt and the
    CA depend on the events grouped together, so they are checked against
    this run, not against events run alone."""

    def __init__(self, batch):
        self.result, self.error, self.wall = None, None, 0.0
        self.thread = threading.Thread(target=self._run, args=(batch,), daemon=True)
        self.thread.start()

    def _run(self, batch):
        from oracle import oracle
        t0 = time.perf_counter()
        try:
            self.result = oracle.run(batch)[0]
        except Exception as exc:  # reported by parity_full
            self.error = exc
        self.wall = time.perf_counter() - t0

    def get(self):
        self.thread.join()
        if self.error is not None:
            raise self.error
        return self.result


def parity_full(ctx, batch, whole):
    """The batched results of the full batch against the oracle: every event's
    slice of pairs, candidates, triplets and eta against the event run alone,
    and every array against the whole batch run as one group
    (oracle/batch_slices.py)."""
    from oracle import batch_slices, oracle
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    refs = oracle.run(batch, event_grouping=1, n_workers=cores,
                      arrays=("pairs", "cands", "trip_h1", "trip_h2", "trip_h3", "eta"))
    ctx.upload(batch)
    ctx.seed_batch(use_graph=True)
    got = {}
    p, got["pair_offsets"] = ctx.pairs()
    got["pairs"] = p.reshape(-1)
    c, got["cand_offsets"] = ctx.candidates()
    got["cands"] = c.reshape(-1)
    got["trip_h1"], got["trip_h2"], got["trip_h3"], got["trip_offsets"] = ctx.triplets()
    got["eta"], got["pt"] = ctx.eta_pt()
    (got["link_basis"], got["link_follower"], got["connectable"],
     got["non_connectable"]) = ctx.links()
    got["ca_states"], got["tracks"], got["track_offsets"] = ctx.tracks()
    per_event = batch_slices.compare(batch, got, refs)
    t_events = time.perf_counter() - t0
    diff = batch_slices.compare_whole(got, whole.get())
    ok = not per_event["mismatch"] and not diff
    return {"result": "bit-exact" if ok else "MISMATCH",
            "events": per_event["events"], "per_event_mismatch": per_event["mismatch"],
            "whole_batch_mismatch": diff,
            "checked": "every event's slice of pairs, candidates, triplet hits and eta bits against the CPU "
                       "oracle run on the event alone (16 host threads); all arrays -- also links, "
                       "connectable lists, pt, CA states, best bases and tracks -- against the oracle run on "
                       "the whole batch as one event group",
            "oracle_wall_s": {"events_alone": round(t_events, 2), "whole_batch": round(whole.wall, 2)}}


def run_alignment(device: int):
    """Alignment workload (1000 events, hidden per-layer shifts): seeding, fit rows
    frozen, 50 gradient evaluations of the FP32 fit's adjoint kernel."""
    from trax_gb300 import align as AL, capi, events
    batch = events.generate(4)
    radii = np.array(events.BARREL10_RADII)
    ctx = capi.Context(device)
    try:
        ctx.upload(batch)
        ctx.seed_batch(use_graph=True, run_linking=False)
        n = ctx.fit_prepare(truth_only=True)
        zero = np.zeros((batch.n_layers, 3))
        for _ in range(3):
            ctx.fit_backward(zero)
        reps = 20
        t0 = time.perf_counter()
        for _ in range(reps):
            ctx.fit_backward(zero)
        bw = (time.perf_counter() - t0) / reps
        t0 = time.perf_counter()
        for _ in range(reps):
            ctx.fit_forward(zero)
        fw = (time.perf_counter() - t0) / reps
        t0 = time.perf_counter()
        a, hist = AL.align_context(ctx, radii, steps=50)
        t_align = time.perf_counter() - t0
        res = AL.Gauge(radii).residual_um(a, batch.misalignment)
        return {"workload": "alignment: 1000 ttbar-like events, 10 layers, 8 layer triplets, hidden shifts "
                            "dr, dz ~ N(0, 50 um), dphi ~ N(0, 20 urad), seed 4 (config 4)",
                "fit_rows": n, "forward_ms": round(fw * 1e3, 4), "backward_ms": round(bw * 1e3, 4),
                "backward_rows_per_s": round(n / bw, 1),
                "timing": "wall clock per C-ABI call, including the host read of chi2 and 30 gradients",
                "gradient_evaluations": hist[-1].evaluations, "align_wall_s": round(t_align, 3),
                "chi2_start": round(hist[0].loss, 1), "chi2_end": round(hist[-1].loss, 1),
                "recovery_max_um": round(float(np.abs(res).max()), 3),
                "recovery": "max |recovered - injected| over the 30 shifts (dphi as r dphi), outside the six "
                            "chi2-invariant deformations"}
    finally:
        ctx.close()


def run_config3(device: int, steps: int, n_events: int = 16, fine: int = 8):
    """The high-occupancy workload at full size (16 events x 20 vertices x 1000
    tracks, about 125 000 hits per event, grid 80 x 256): one CUDA-graph replay
    of the whole chain per step, device time from CUDA events.  The prediction
    count walks a z grid `fine` times finer than the grid's 7.5 cm rows (the
    same results; 0: the grid itself)."""
    from trax_gb300 import capi, events
    batch = events.generate(3, n_events=n_events)
    ctx = capi.Context(device)
    try:
        ctx.upload(batch)
        ctx.set_fine_rows(fine)
        first = ctx.seed_batch(use_graph=True)  # calibrates the capacities and captures the graph
        for _ in range(2):
            ctx.seed_batch(use_graph=True)
        ms, captures = [], 0
        for _ in range(max(steps, 1)):
            st = ctx.seed_batch(use_graph=True)
            ms.append(st.device_ms)
            captures += st.graph_captures
        t = float(np.mean(ms))
        return {"workload": f"pileup: {batch.n_events} events x 20 vertices x 1000 tracks + 5% noise, 10 layers, "
                            "6 layer triplets, grid 80x256, seed 3 (config 3)",
                "events_per_s": round(batch.n_events / (t * 1e-3), 2), "ms_per_batch": round(t, 3),
                "steps": len(ms), "hits": batch.n_hits,
                "sizes": {"pairs": st.n_pairs, "candidates": st.n_candidates, "triplets": st.n_triplets,
                          "links": st.n_links, "track_entries": st.n_track_entries,
                          "candidate_sentinels": st.n_candidate_sentinels},
                "triplets_per_s": round(st.n_triplets / (t * 1e-3), 1),
                "graph_captures": {"first_call": first.graph_captures, "timed_steps": captures,
                                   "note": "calibrate-and-capture passes: the first call sizes every buffer from a "
                                           "host-synced run and captures the graph; replays recapture only after "
                                           "a capacity overflow"},
                "kernel_launches_per_step": st.kernel_launches,
                "candidate_slots": ctx.candidate_slots(),
                "fine_rows": ctx.fine_rows(),
                "kernel_ms": {k: round(v, 3) for k, v in ctx.timings()[1].items() if v >= 0},
                "parity": "tests/test_gpu_parity.py::test_pileup_workload_at_full_size: every array equals the "
                          "oracle run on the whole batch"}
    finally:
        ctx.close()


def run_ours(args, ranks):
    from trax_gb300 import capi, events
    device = ranks.local
    seed = 2 + 1000 * ranks.rank
    batch = events.generate(CONFIG, n_events=args.events, seed=seed)
    if args.grid:
        batch.n_z, batch.n_phi = (int(v) for v in args.grid.lower().split("x"))
    n_hits = batch.n_hits
    ctx = capi.Context(device)
    ctx.upload(batch)
    tune = None
    if args.blocks:
        ctx.set_block_sizes(*(int(v) for v in args.blocks.split(",")))
    elif not args.no_tune:
        # block sizes always; the grid only with --tune-grid
        tune = ctx.autotune(cache_path=args.tune_cache, search_grid=bool(args.tune_grid and not args.grid))
        batch.n_z, batch.n_phi = tune["n_z"], tune["n_phi"]
    shape = ctx.launch_config()
    cells = batch.n_events * batch.n_layers * (batch.n_z + 1) * (batch.n_phi + 1)
    for _ in range(max(args.warmup, 3)):
        st = ctx.seed_batch(use_graph=True)
    clocks = ClockSampler(device)
    ranks.barrier()
    clocks.start()
    dev_ms = []
    kern = {k: [] for k in capi.Context.KERNELS}
    stage = {k: [] for k in capi.Context.STAGES}
    t_wall0 = time.perf_counter()
    records = None
    if args.runtime_csv:
        from trax_gb300 import runtime_csv
        records = runtime_csv.RuntimeRecords()
    for _ in range(args.steps):
        st = ctx.seed_batch(use_graph=True)
        dev_ms.append(st.device_ms)
        s_ms, k_ms = ctx.timings()
        for k, v in k_ms.items():
            kern[k].append(v)
        for k, v in s_ms.items():
            stage[k].append(v)
        if records is not None:
            records.add(batch.n_events, batch.n_layers, len(batch.lts), shape["predict_threads"], n_hits,
                        int(batch.hit_id.astype(np.int64).max()), s_ms, k_ms)
    t_wall = time.perf_counter() - t_wall0
    if records is not None:
        with open(args.runtime_csv, "w") as f:
            f.write(records.csv())
    clk = clocks.stop()
    # the oracle on the whole batch, on one host thread while the rest runs
    whole = WholeBatchOracle(batch) if (ranks.rank == 0 and not args.no_parity) else None
    ranks.barrier()
    my_time = sum(dev_ms) / 1e3
    t_max = ranks.max(my_time)
    events_all = ranks.sum(float(batch.n_events * args.steps))
    trip_all = ranks.sum(float(st.n_triplets * args.steps))
    value = events_all / t_max
    ms_per_step = 1e3 * t_max / args.steps
    launches = st.kernel_launches * args.steps

    # roofline of the dominant kernel (mean CUDA-event time over the steps)
    kmean = {k: float(np.mean(v)) for k, v in kern.items() if v and min(v) >= 0}
    if not kmean:
        raise RuntimeError("no per-kernel CUDA-event timings were recorded")
    dom = max(kmean, key=kmean.get)
    # pair-stage tasks: one per outer-layer hit of every (event, layer triplet)
    n_tasks = int(sum(int(batch.layer_hits[:, lt.layer2 - 1].sum()) for lt in batch.lts))
    hbm, peak_kind = peaks()
    per_layer = batch.n_events * (batch.n_z + 1) * (batch.n_phi + 1)
    cells_inner = per_layer * len({lt.layer1 for lt in batch.lts})
    cells_third = per_layer * len({lt.layer3 for lt in batch.lts})
    kb = kernel_bytes(dom, st, n_tasks, n_hits, cells, cells_inner, cells_third)
    achieved = kb / (kmean[dom] * 1e-3) / 1e9
    cb = chain_bytes(st, n_hits, cells, len(batch.lts))
    result = {
        "metric": METRIC, "value": round(value, 2), "unit": "events/s", "n_gpus": ranks.world,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": round(ms_per_step, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "ttbar-like batch: 1000 events, tracks ~ Poisson(U[300,3000]), 10 layers, 6 layer "
                               "triplets, seed 2 (config 2)",
                   "events_per_gpu": batch.n_events, "hits_per_gpu": n_hits, "grid": f"{batch.n_z}x{batch.n_phi}",
                   "block_sizes": {k: shape[k] for k in ("pair_threads", "predict_threads", "filter_threads")},
                   "predict_pairs_per_thread": ctx.pairs_per_thread(),
                   "predict_candidate_slots": ctx.candidate_slots(),
                   "predict_fine_rows": ctx.fine_rows(),
                   "autotune": None if tune is None else {
                       "shapes_timed": tune["shapes_timed"], "from_cache": bool(tune["from_cache"]),
                       "best_ms": round(tune["best_ms"], 4), "default_shape_ms": round(tune["default_ms"], 4)},
                   "layer_triplets": len(batch.lts),
                   "l2": f"inputs larger than L2 ({n_hits * 28 / 1e6:.0f} MB of hit columns per step), no flush",
                   "path": "batched: one CUDA-graph replay of the whole chain per step"},
        "triplets_per_s": round(trip_all / t_max, 1),
        "sizes": {"pairs": st.n_pairs, "candidates": st.n_candidates, "triplets": st.n_triplets,
                  "links": st.n_links, "track_entries": st.n_track_entries},
        "stage_ms": {k: round(float(np.mean(v)), 4) for k, v in stage.items() if v and min(v) >= 0},
        "kernel_ms": {k: round(v, 4) for k, v in kmean.items()},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 2), "peak": hbm, "unit": "GB/s",
                     "frac": round(achieved / hbm, 4), "traffic": kernel_traffic(dom, st, n_hits, f"{batch.n_z}x{batch.n_phi}"),
                     "traffic_note": "DRAM bytes per launch: ncu per-unit traffic of the 300-event case at this grid x "
                                     "units (null for a grid without a capture)",
                     "peak_kind": f"{peak_kind} hbm_gbs (copy bandwidth)",
                     "algorithmic_bytes": int(kb)},
        "issue_roofline": kernel_issue(dom, st, kmean[dom], clk, device, f"{batch.n_z}x{batch.n_phi}"),
        # window and cut evaluations per second of the FP32-heavy kernels:
        # one pair window per outer hit, one third-hit window per pair, the
        # dphi test per candidate (the rest on its survivors)
        "tests_per_s": {k: round(n / (kmean[kk] * 1e-3), 1) for k, kk, n in (
            ("pair_windows", "pair_count", n_tasks), ("predict_windows", "predict_count", st.n_pairs),
            ("filter_candidates", "filter", st.n_candidates)) if kmean.get(kk)},
        "chain_roofline": {"achieved": round(cb / (ms_per_step * 1e-3) / 1e9, 2), "unit": "GB/s",
                           "frac": round(cb / (ms_per_step * 1e-3) / 1e9 / hbm, 4), "bytes_per_step": int(cb)},
        "gpu_launches": int(launches),
        "wall_s": round(t_wall, 3),
        "clocks": clk,
    }

    # end to end through the C ABI from host buffers: every step uploads the
    # batch's hit columns and supplements from page-locked host memory, replays
    # the chain and reads the triplets and tracks back into page-locked memory
    if args.e2e_steps > 0:
        cols = ("x", "y", "z", "layer", "det_id", "hit_id", "event", "event_offsets", "layer_hits", "layer_offsets")
        pinned = {}
        for k in cols:
            src = np.ascontiguousarray(getattr(batch, k))
            pinned[k] = capi.pinned_empty(src.shape, src.dtype)
            pinned[k][...] = src
        pbatch = dataclasses.replace(batch, **pinned)
        n_off = batch.n_events * len(batch.lts) + 1
        out_t = [capi.pinned_empty((max(st.n_triplets, 1),), np.uint32) for _ in range(3)] + [
            capi.pinned_empty((n_off,), np.uint32)]
        out_k = [capi.pinned_empty((max(st.n_triplets, 1),), np.uint32),
                 capi.pinned_empty((max(st.n_track_entries, 1),), np.uint32),
                 capi.pinned_empty((st.n_triplets + 1,), np.uint32)]
        bi = int(sum(pinned[k].nbytes for k in cols))

        def e2e_run(b, pinned_out):
            times, bo = [], 0
            for it in range(args.e2e_steps + 1):
                t0 = time.perf_counter()
                ctx.upload_hits(b)
                ctx.seed_batch(use_graph=True)
                h1, h2, h3, _ = ctx.triplets(out=out_t if pinned_out else None)
                _, tr, toff = ctx.tracks(out=out_k if pinned_out else None)
                dt = time.perf_counter() - t0
                bo = int(h1.nbytes + h2.nbytes + h3.nbytes + tr.nbytes + toff.nbytes)
                if it > 0:
                    times.append(dt)
            return times, bo

        e2e_times, bo = e2e_run(pbatch, True)
        serial = {"value": round(ranks.sum(float(batch.n_events * len(e2e_times))) / ranks.max(sum(e2e_times)), 2),
                  "unit": "events/s", "note": "one context: upload, replay and download one after the other"}

        # several contexts on their own streams and host threads: one batch's
        # copies run while the others' kernels do (copy engines and SMs overlap)
        shape_now = ctx.launch_config()
        pipes = []
        for _ in range(max(args.e2e_contexts, 1)):
            c2 = capi.Context(device)
            c2.upload(pbatch)
            c2.set_grid(shape_now["n_z"], shape_now["n_phi"])
            c2.set_block_sizes(shape_now["pair_threads"], shape_now["predict_threads"],
                               shape_now["filter_threads"])
            c2.set_pairs_per_thread(ctx.pairs_per_thread())
            c2.set_candidate_slots(tune["candidate_slots"] if tune else 0)
            c2.set_fine_rows(ctx.fine_rows())
            for _w in range(2):
                c2.seed_batch(use_graph=True)
            outs = ([capi.pinned_empty((max(st.n_triplets, 1),), np.uint32) for _ in range(3)]
                    + [capi.pinned_empty((n_off,), np.uint32)],
                    [capi.pinned_empty((max(st.n_triplets, 1),), np.uint32),
                     capi.pinned_empty((max(st.n_track_entries, 1),), np.uint32),
                     capi.pinned_empty((st.n_triplets + 1,), np.uint32)])
            pipes.append((c2, outs))
        steps_each = max(args.e2e_pipe_steps, 2)
        errors = []

        def worker(c2, outs):
            try:
                for _s in range(steps_each):
                    c2.upload_hits(pbatch)
                    c2.seed_batch(use_graph=True)
                    c2.triplets(out=outs[0])
                    c2.tracks(out=outs[1])
            except Exception as exc:  # surfaced below
                errors.append(exc)

        ths = [threading.Thread(target=worker, args=pl) for pl in pipes]
        ranks.barrier()
        t0 = time.perf_counter()
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        dt = time.perf_counter() - t0
        if errors:
            raise errors[0]
        h1p, _, _, _ = pipes[0][0].triplets(out=pipes[0][1][0])
        if not np.array_equal(h1p, ctx.triplets()[0]):
            raise RuntimeError("pipelined contexts returned different triplets")
        for c2, _o in pipes:
            c2.close()
        n_steps = len(pipes) * steps_each
        e2e_t = ranks.max(dt)
        e2e_events = ranks.sum(float(batch.n_events * n_steps))
        result["e2e"] = {"value": round(e2e_events / e2e_t, 2), "unit": "events/s", "h2d_bytes_per_step": bi,
                         "d2h_bytes_per_step": bo, "steps": n_steps,
                         "contexts": len(pipes),
                         "note": "page-locked host arrays (trax_host_alloc); every step uploads the batch, replays "
                                 "the chain and downloads triplets and tracks; contexts on their own streams and "
                                 "host threads overlap one step's copies with the others' kernels; wall clock",
                         "serial": serial}
        pg_times, _ = e2e_run(batch, False)
        result["e2e_pageable"] = {"value": round(ranks.sum(float(batch.n_events * len(pg_times)))
                                                 / ranks.max(sum(pg_times)), 2), "unit": "events/s",
                                  "note": "the same from ordinary (pageable) numpy arrays"}
    if ranks.rank == 0:
        if not args.no_plain:
            plain = run_plain(ctx, batch, args.plain_events)
            result["plain_per_event"] = plain
            result["batched_over_plain"] = round(value / ranks.world / plain["value"], 2)
        if not args.no_parity:
            result["parity"] = parity_full(ctx, batch, whole)
        if not args.no_cpu:
            result["cpu_baseline"] = cpu_baseline(batch, args.cpu_sample)
        if not args.no_align:
            result["alignment"] = run_alignment(device)
        if not args.no_config3:
            result["config3"] = run_config3(device, args.config3_steps, args.config3_events, args.config3_fine)
    ctx.close()
    return result


def run_reference(args, ranks):
    if ranks.rank != 0:
        return None
    from trax_gb300 import events
    batch = events.generate(CONFIG, n_events=args.events)
    if args.grid:
        batch.n_z, batch.n_phi = (int(v) for v in args.grid.lower().split("x"))
    cores = os.cpu_count() or 1
    kind = cpu_engine()
    # 4 events per host thread per step, so that the threads stay busy to the
    # end of a step despite the spread of event sizes
    per_step = min(max(4 * cores, 32), batch.n_events)
    warm = batch.subset(range(min(cores, batch.n_events)))
    for _ in range(max(args.warmup, 3)):
        cpu_run(warm, cores, kind)
    times, evs, trip = [], 0, 0
    for k in range(args.steps):
        lo = (k * per_step) % max(1, batch.n_events - per_step)
        sample = batch.subset(range(lo, lo + per_step))
        t0 = time.perf_counter()
        trip += cpu_run(sample, cores, kind)
        times.append(time.perf_counter() - t0)
        evs += sample.n_events
    total = sum(times)
    v = round(evs / total, 3)
    return {
        "metric": METRIC, "impl": "reference", "value": v, "unit": "events/s", "n_gpus": ranks.world,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": round(1e3 * total / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "ttbar-like batch: 1000 events, tracks ~ Poisson(U[300,3000]), 10 layers, 6 layer "
                               "triplets, seed 2 (config 2)", "events_per_step": per_step,
                   "grid": f"{batch.n_z}x{batch.n_phi}"},
        "triplets_per_s": round(trip / total, 1),
        "cpu_baseline": {"value": v, "unit": "events/s", "cores": cores, "kind": kind,
                         "sample": f"{per_step} events per step of the 1000-event workload (rotating windows) at "
                                   f"grid {batch.n_z}x{batch.n_phi}, one event per group, {cores} host threads; "
                                   + CPU_KIND_NOTE[kind], "host": host_cpu()},
        "e2e": {"value": v, "unit": "events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    from trax_gb300.sharding import Ranks
    args = parse()
    ranks = Ranks("gloo")
    try:
        if args.impl == "reference":
            res = run_reference(args, ranks)
        else:
            res = run_ours(args, ranks)
        if ranks.rank == 0 and res is not None:
            print(json.dumps(res), flush=True)
    finally:
        ranks.close()


if __name__ == "__main__":
    main()
