"""Runtime records in the reference's csv layout."""
import os

from oracle.ref_extract import reference_dir
from trax_gb300 import runtime_csv

REF_CSV = os.path.join(reference_dir(), "plotting/data/runtime/runtime.bigOne.local.conf.events.100.test.gpu.csv")


def _timings(scale=1.0):
    stage = {"grid": 1.0, "pairs": 2.0, "predict": 5.0, "filter": 2.5, "connectivity": 0.5, "circle_fit": 0.1,
             "ca": 0.4}
    kern = {"grid_build": 0.9, "pair_count": 0.5, "pair_store": 1.0, "predict_count": 3.0, "predict_store": 1.0,
            "filter": 1.5, "filter_store": 0.5, "connectivity_count": 0.2, "connectivity_store": 0.2}
    return {k: v * scale for k, v in stage.items()}, {k: v * scale for k, v in kern.items()}


def test_header_columns_and_rows():
    rec = runtime_csv.RuntimeRecords()
    for s in (1.0, 1.2):
        st, k = _timings(s)
        rec.add(1000, 10, 6, 128, 9723189, 1650000, st, k, read_ms=30.0, read_bytes=272333292)
    st, k = _timings()
    rec.add(100, 4, 2, 128, 96000, 20000, st, k)
    lines = rec.csv().strip().split("\n")
    cols = lines[0].split()
    assert cols[:7] == ["events", "layers", "layerTriplets", "threads", "hits", "tracks", "n"]
    assert "tripletConnectivityTightWalltimeKernelVar" in cols and cols[-1] == "totalKernelVar"
    assert len(lines) == 3
    row = dict(zip(cols, lines[1].split()))
    assert row["n"] == "2" and float(row["pairGenCount"]) == 0.55 and float(row["readTime"]) == 30.0
    assert abs(float(row["pairGenScan"]) - 0.55) < 1e-9  # 2.2 - 0.55 - 1.1
    # every stage's count + scan + store: 11.4 ms at scale 1, so 12.54 on average over scales 1 and 1.2
    assert abs(float(row["totalKernel"]) - 12.54) < 1e-6
    assert len(lines[2].split()) == len(cols)


def test_header_matches_the_reference_files():
    if not os.path.exists(REF_CSV):
        import pytest
        pytest.skip("the reference's runtime csv is not on this machine")
    ref = open(REF_CSV).readline().split()
    ours = runtime_csv.header().split()
    # the reference's published files predate its connectivity/CA columns: ours add them in the same places
    assert [c for c in ours if not c.startswith(("tripletConnectivity", "trackletCircle", "cellular"))] == ref
