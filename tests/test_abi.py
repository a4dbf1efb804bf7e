"""The C ABI library: it builds for sm_103a, loads, and exports every entry
point include/trax/trax.h declares (no compute call: no GPU needed)."""
import os
import re
import subprocess

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "trax", "trax.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(trax_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_stage_entry_points():
    names = declared_functions()
    for n in ("trax_create", "trax_grid_build", "trax_pair_gen", "trax_triplet_predict", "trax_triplet_filter",
              "trax_connectivity", "trax_circle_fit", "trax_cellular_automaton", "trax_prefix_sum",
              "trax_seed_batch", "trax_set_tracklets"):
        assert n in names


def test_library_exports_every_declared_symbol(trax_lib):
    lib = trax_lib.load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.trax_version().startswith(b"trax_gb300")


def test_binding_covers_the_header(trax_lib):
    assert set(trax_lib.EXPORTED) <= set(declared_functions())


def test_product_library_does_not_contain_the_oracle(trax_lib):
    out = subprocess.run(["nm", "-D", trax_lib.library_path()], capture_output=True, text=True).stdout
    assert "oracle_" not in out
    assert "trax_seed_batch" in out


def test_build_targets_sm103a_without_fma():
    from trax_gb300 import build
    flags = " ".join(build.NVCC_FLAGS)
    assert "arch=compute_103a,code=sm_103a" in flags
    for f in ("-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false", "-ffp-contract=off"):
        assert f in flags


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    from trax_gb300 import capi
    monkeypatch.setattr(capi, "_lib", None)
    monkeypatch.setattr(capi, "library_path", lambda: str(tmp_path / "absent.so"))
    try:
        capi.load()
    except RuntimeError as e:
        assert "no CPU fallback" in str(e)
    else:
        raise AssertionError("loading a missing library must fail")
