"""The C++ host classes (include/trax/trax.hpp): compiled against the C ABI
here; run on the GPU, where the stage-by-stage class chain must equal one
batched trax_seed_batch call element by element."""
import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(REPO, "tests", "cpp", "host_classes_test.cpp")
XML = os.path.join(REPO, "tests", "golden", "layer_triplets_4layer.xml")


def _compile(tmp_path, lib_dir):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = os.path.join(str(tmp_path), "host_classes_test")
    cmd = [cxx, "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(REPO, "include"), SRC,
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
