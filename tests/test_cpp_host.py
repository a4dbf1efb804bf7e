"""The C++ host classes (include/trax/trax.hpp): compiled against the C ABI
here; run on the GPU, where the stage-by-stage class chain must equal one
batched trax_seed_batch call element by element.  The loader classes
(EventFile, addEvents) run here, on the host, against the C ABI's loader."""
import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(REPO, "tests", "cpp", "host_classes_test.cpp")
XML = os.path.join(REPO, "tests", "golden", "layer_triplets_4layer.xml")


def _compile(tmp_path, lib_dir, src=SRC):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = os.path.join(str(tmp_path), os.path.splitext(os.path.basename(src))[0])
    cmd = [cxx, "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(REPO, "include"), src,
           "-L", lib_dir, "-ltrax_gb300", "-Wl,-rpath," + lib_dir, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_host_classes_compile_and_link(tmp_path):
    from trax_gb300 import build
    build.build()
    _compile(tmp_path, os.path.dirname(build.LIB_PATH))


@pytest.mark.gpu
def test_host_class_chain_equals_batched_call(tmp_path):
    from trax_gb300 import build
    build.build()
    exe = _compile(tmp_path, os.path.dirname(build.LIB_PATH))
    r = subprocess.run([exe, XML], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("OK host classes")


@pytest.mark.gpu
def test_ca_class_on_caller_links_and_pt(tmp_path):
    """CellularAutomaton::run computes on the links and pt it is given (the
    reference's connectivity fixture plus hand-made pt), on a Context without
    triplets of its own."""
    from trax_gb300 import build
    build.build()
    exe = _compile(tmp_path, os.path.dirname(build.LIB_PATH), os.path.join(REPO, "tests", "cpp", "ca_inputs_test.cpp"))
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("OK ca inputs")


def test_ca_inputs_program_compiles(tmp_path):
    from trax_gb300 import build
    build.build()
    _compile(tmp_path, os.path.dirname(build.LIB_PATH), os.path.join(REPO, "tests", "cpp", "ca_inputs_test.cpp"))


def test_loader_classes_equal_the_c_loader(tmp_path):
    """trax::EventFile + trax::addEvents (the reference's HitCollection::addEvent
    per event of a PEventContainer) give the columns, supplements and findable
    tracks of trax_events_load."""
    import numpy as np
    from trax_gb300 import build, eventio, events
    from tests.test_eventio import encode, synthetic_events
    build.build()
    exe = _compile(tmp_path, os.path.dirname(build.LIB_PATH), os.path.join(REPO, "tests", "cpp",
                                                                         "event_loader_test.cpp"))
    pb = tmp_path / "events.pb"
    pb.write_bytes(encode(synthetic_events(seed=5, n_events=3)))
    for num_tracks, only_tracks in ((-1, 0), (4, 1)):
        r = subprocess.run([exe, str(pb), XML, "1.0", str(num_tracks), str(only_tracks)], capture_output=True,
                           text=True, timeout=120)
        assert r.returncode == 0, r.stdout + r.stderr
        rows = [ln.split() for ln in r.stdout.splitlines()]
        lts = events.layer_triplets([1, 2])
        batch, fid, fev = eventio.EventFile(str(pb)).load(lts, 1.0, num_tracks=num_tracks,
                                                          only_tracks=bool(only_tracks))
        hits = [row for row in rows if row[0] == "HIT"]
        assert rows[0] == ["SIZES", str(batch.n_hits), str(batch.n_events), str(batch.n_layers), str(fid.size)]
        assert np.array_equal(np.float32([h[1] for h in hits]), batch.x)
        assert np.array_equal(np.float32([h[3] for h in hits]), batch.z)
        assert [int(h[4]) for h in hits] == batch.layer.tolist()
        assert [int(h[6]) for h in hits] == batch.hit_id.tolist()
        assert [int(h[7]) for h in hits] == batch.event.tolist()
        assert [int(row[1]) for row in rows if row[0] == "LAYER"] == batch.layer_hits.reshape(-1).tolist()
        assert [int(row[1]) for row in rows if row[0] == "EVENT"] == batch.event_offsets.tolist()
        assert [(int(row[1]), int(row[2])) for row in rows if row[0] == "FINDABLE"] == list(zip(fid.tolist(),
                                                                                               fev.tolist()))
