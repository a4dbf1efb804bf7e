"""bench.py's JSON line, on the CPU: the reference arm (the oracle on the host
cores) prints every key of the contract, and the per-unit tables behind
roofline.traffic and issue_roofline are keyed by grid and give null for a
grid without a capture."""
import json
import os
import subprocess
import sys
import types

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_contract():
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1", "--events", "40"], capture_output=True, text=True, timeout=600, cwd=REPO)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["unit"] == "events/s" and line["value"] > 0
    assert line["warmup"] >= 3 and line["higher_is_better"] is True
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == line["value"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_per_unit_tables_are_keyed_by_grid():
    sys.path.insert(0, REPO)
    import bench
    st = types.SimpleNamespace(n_pairs=1000, n_candidates=500)
    per_pair = bench.TRAFFIC_PER_UNIT["250x48"]["predict_count"][1]
    assert 17.4 <= per_pair < 40  # at least the algorithmic bytes per pair
    assert bench.kernel_traffic("predict_count", st, 0, "250x48") == int(per_pair * 1000)
    assert bench.kernel_traffic("filter", st, 0, "150x64") == int(27.3 * 500)
    assert bench.kernel_traffic("predict_count", st, 0, "123x45") is None
    assert bench.kernel_traffic("pair_store", st, 0, "250x48") is None
    # instruction counts only where the current prediction kernel was captured:
    # the workload's own grid
    assert set(bench.INST_PER_UNIT) <= set(bench.TRAFFIC_PER_UNIT) and "250x48" in bench.INST_PER_UNIT
