"""Build recipe for oracle/_ref/: the reference's own OpenCL kernel text, run on the CPU.

TEST INFRASTRUCTURE ONLY.  The reference (JuantAldea/trax) cannot be built:
its OpenCL wrapper submodule is empty, it needs Boost, protobuf and an OpenCL
runtime.  Its kernels, though, are OpenCL C source text inside
``KERNEL_CLASS(...)`` / ``KERNEL_CLASSP(...)`` macros in
``src/algorithms/*.h``.  This script

1. reads those headers where they lie (``$TRAX_REFERENCE_DIR``, default
   ``/root/reference``) and copies the text of every kernel on the seeding
   path into ``oracle/_ref/ref_kernels.cpp``, inside ``namespace refk``,
   after ``oracle/ref_shim.h`` (the OpenCL work-item environment);
2. copies the track evaluation of ``src/triplet_builder/TripletBuilder.cpp``
   (track extraction, clone removal, real/fake split; host C++ over std
   containers) into ``oracle/_ref/ref_tracks.cpp``, inside ``namespace
   reftr``, with comments removed and nothing else changed;
3. compiles both with ``oracle/ref_driver.cpp`` (the reference's host-side
   ``run()`` sequences, restated) into ``oracle/_ref/libtraxref.so``.

Nothing it writes is committed: ``oracle/_ref/`` is git-ignored.  When the
reference is absent but ``oracle/_ref/ref_kernels.cpp`` was generated
earlier, step 2 alone runs.

The kernel text is copied as it is, with exactly these changes:

* comments are removed (commented-out kernels and PRINTF strings inside
  comments are not code);
* ``(float2)(``, ``(float3)(``, ``(float4)(``, ``(uint2)(``, ``(uint4)(`` --
  OpenCL vector literals -- become constructor calls ``float3(`` etc.  In C++
  the literal form would parse as a cast of a comma expression;
* the ``#define`` lines PrefixSum passes to its kernels
  (``PrefixSum.cpp:4-6``) are emitted before them.

Everything else (``__kernel``, ``__global``, ``__local``, the built-ins, the
work-item functions, ``M_PI_F``, ``PRINTF``) comes from ``ref_shim.h``.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from typing import Dict, List, Tuple

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
OUT_DIR = os.path.join(HERE, "_ref")
GEN_CPP = os.path.join(OUT_DIR, "ref_kernels.cpp")
GEN_TRACKS = os.path.join(OUT_DIR, "ref_tracks.cpp")
# the reference's track evaluation (host C++ over std containers): track
# extraction from the CA output, clone removal, real/fake split, distinct
# real tracks; copied from the Track typedef up to printTracks
TRACKS_SRC = "src/triplet_builder/TripletBuilder.cpp"
TRACKS_FIRST = "typedef typename std::pair<uint, std::shared_ptr<std::vector<uint>>> Track;"
TRACKS_END = "void printTracks("
LIB_PATH = os.path.join(OUT_DIR, "libtraxref.so")
DRIVER = os.path.join(HERE, "ref_driver.cpp")
SHIM = os.path.join(HERE, "ref_shim.h")
CSRC = os.path.join(REPO, "trax_gb300", "csrc")


def reference_dir() -> str:
    return os.environ.get("TRAX_REFERENCE_DIR", "/root/reference")


# header (relative to the reference root) -> kernels taken from it, in order
KERNELS: List[Tuple[str, List[str]]] = [
    ("src/algorithms/GridBuilder.h",
     ["gridCount", "gridNoLocalCount", "gridStore", "gridWrittenLocalStore", "gridNoLocalStore"]),
    ("src/algorithms/PrefixSum.h", ["prefixSumWG", "prefixSumPartial", "prefixSumUniformAdd"]),
    ("src/algorithms/PairGeneratorBeamspot.h", ["pairCount", "pairNoLocalCount", "pairStore"]),
    ("src/algorithms/TripletThetaPhiPredictor.h",
     ["predictCount", "predictStore", "predictOffsetMonotonizeStore"]),
    ("src/algorithms/TripletThetaPhiFilter.h",
     ["filterCount", "filterPopCount", "filterStore", "filterOffsetStore", "filterOffsetMonotonizeStore"]),
    ("src/algorithms/TripletConnectivityTight.h",
     ["tripletEtaCalculatorStore", "tripletConnectivityTightCount", "tripletConnectivityTightStore",
      "streamCompactionGetValidIndexesStore", "predicateInversionStore"]),
    ("src/algorithms/TrackletCircleFitter.h", ["trackletCircleFitterStore"]),
    ("src/algorithms/CellularAutomaton.h",
     ["iteration", "memset", "memcpy", "followerBasisCount", "followerBasisStore", "followerBestBasisStore",
      "handlersStateStore", "trackCollectionStore"]),
]

PREFIX_DEFINES_SRC = "src/algorithms/PrefixSum.cpp"

VECTOR_LITERAL = re.compile(r"\((float2|float3|float4|uint2|uint4)\)\s*\(")


def strip_comments(text: str) -> str:
    """Removes // and /* */ comments, keeping string and character literals and
    every newline (so line numbers stay those of the source)."""
    out = []
    i, n = 0, len(text)
    while i < n:
        c = text[i]
        if c == '"' or c == "'":
            j = i + 1
            while j < n and text[j] != c:
                j += 2 if text[j] == "\\" else 1
            out.append(text[i:j + 1])
            i = j + 1
        elif text.startswith("//", i):
            j = text.find("\n", i)
            i = n if j < 0 else j
        elif text.startswith("/*", i):
            j = text.find("*/", i + 2)
            j = n if j < 0 else j + 2
            out.append("\n" * text.count("\n", i, j))
            i = j
        else:
            out.append(c)
            i += 1
    return "".join(out)


def _match(text: str, open_pos: int, open_ch: str, close_ch: str) -> int:
    depth = 0
    for k in range(open_pos, len(text)):
        if text[k] == open_ch:
            depth += 1
        elif text[k] == close_ch:
            depth -= 1
            if depth == 0:
                return k
    raise ValueError(f"unbalanced {open_ch}{close_ch} from offset {open_pos}")


def extract_kernel(text: str, name: str) -> Tuple[str, int, int]:
    """Returns (kernel function text, first line, last line) of `__kernel void name(...) {...}`."""
    m = re.search(r"__kernel\s+void\s+" + re.escape(name) + r"\s*\(", text)
    if not m:
        raise ValueError(f"kernel {name} not found")
    paren = text.index("(", m.start())
    close = _match(text, paren, "(", ")")
    brace = text.index("{", close)
    end = _match(text, brace, "{", "}")
    body = text[m.start():end + 1]
    first = text.count("\n", 0, m.start()) + 1
    last = text.count("\n", 0, end) + 1
    return body, first, last


def prefix_defines(root: str) -> str:
    src = open(os.path.join(root, PREFIX_DEFINES_SRC), encoding="utf-8", errors="replace").read()
    m = re.search(r"PrefixSum::oclDEFINES\s*=\s*((?:\s*\"(?:[^\"\\]|\\.)*\")+)\s*;", src)
    if not m:
        raise ValueError("PrefixSum::oclDEFINES not found")
    parts = re.findall(r"\"((?:[^\"\\]|\\.)*)\"", m.group(1))
    return "".join(parts).replace("\\n", "\n")


def uses_barrier(body: str) -> bool:
    return re.search(r"\bbarrier\s*\(", body) is not None


def generate(root: str) -> Dict[str, bool]:
    """Writes oracle/_ref/ref_kernels.cpp; returns {kernel: uses barrier()}."""
    os.makedirs(OUT_DIR, exist_ok=True)
    lines = [
        "// GENERATED by oracle/ref_extract.py -- the reference's OpenCL kernel text,",
        "// copied from its KERNEL_CLASS blocks (comments removed, vector literals",
        "// written as constructor calls).  Not committed; rebuilt by the recipe.",
        '#include "ref_shim.h"',
        "",
        "namespace refk {",
        "",
        "// " + PREFIX_DEFINES_SRC + ":4-6 (the defines PrefixSum passes to its kernels)",
    ]
    lines += [ln.strip() for ln in prefix_defines(root).splitlines() if ln.strip()]
    barriers: Dict[str, bool] = {}
    for header, names in KERNELS:
        raw = open(os.path.join(root, header), encoding="utf-8", errors="replace").read()
        text = strip_comments(raw)
        for name in names:
            body, first, last = extract_kernel(text, name)
            body = VECTOR_LITERAL.sub(lambda mm: mm.group(1) + "(", body)
            barriers[name] = uses_barrier(body)
            lines += ["", f"// {header}:{first}-{last}", body]
    lines += ["", "// which kernels call barrier() (work-groups of more than one work-item run as fibers)"]
    for name, b in barriers.items():
        lines.append(f"constexpr bool kBarrier_{name} = {'true' if b else 'false'};")
    lines += ["", "}  // namespace refk", ""]
    tmp = GEN_CPP + f".tmp{os.getpid()}"
    with open(tmp, "w") as f:
        f.write("\n".join(lines))
    os.replace(tmp, GEN_CPP)
    return barriers


def generate_tracks(root: str) -> None:
    """Writes oracle/_ref/ref_tracks.cpp: TripletBuilder.cpp's track evaluation
    functions, verbatim but for the comments, inside namespace reftr, where
    ref_shim.h gives them the HitCollection / TrackletCollection accessors
    they call."""
    raw = open(os.path.join(root, TRACKS_SRC), encoding="utf-8", errors="replace").read().splitlines()
    first = next(i for i, ln in enumerate(raw) if ln.strip() == TRACKS_FIRST)
    last = next(i for i, ln in enumerate(raw) if i > first and ln.startswith(TRACKS_END))
    body = strip_comments("\n".join(raw[first:last]))
    lines = [
        "// GENERATED by oracle/ref_extract.py -- the reference's track evaluation,",
        "// copied from " + TRACKS_SRC + " (comments removed).  Not committed;",
        "// rebuilt by the recipe.",
        '#include "ref_shim.h"',
        "",
        "namespace reftr {",
        "using std::shared_ptr;  // the reference's own headers bring it in",
        "",
        f"// {TRACKS_SRC}:{first + 1}-{last}",
        body,
        "",
        "}  // namespace reftr",
        "",
    ]
    tmp = GEN_TRACKS + f".tmp{os.getpid()}"
    with open(tmp, "w") as f:
        f.write("\n".join(lines))
    os.replace(tmp, GEN_TRACKS)


CXXFLAGS = ["-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread",
            "-Wall", "-Wno-int-in-bool-context", "-Wno-unused-variable", "-Wno-unused-but-set-variable", "-Wno-sign-compare",
            "-Wfloat-conversion", "-Werror=narrowing"]

# A float -> integer conversion outside floor() would follow C++'s rules
# (undefined out of range) instead of the saturating definition the oracle
# and the CUDA kernels share; the build fails on any the compiler reports.
FLOAT_TO_INT = re.compile(r"conversion from .(float|double). to .(unsigned int|int|long|long unsigned int|"
                          r"unsigned char|char|short|size_t)")


def compile_lib() -> str:
    # the driver includes the generated ref_kernels.cpp: one translation unit
    cmd = ["g++"] + CXXFLAGS + ["-I", HERE, "-I", CSRC, "-I", OUT_DIR, "-o", LIB_PATH + ".tmp", DRIVER]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("building the reference kernels failed:\n" + r.stdout + r.stderr)
    bad = [ln for ln in r.stderr.splitlines() if FLOAT_TO_INT.search(ln)]
    if bad:
        raise RuntimeError("float -> integer conversions outside floor():\n" + "\n".join(bad))
    os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


def _newest_input() -> float:
    paths = [DRIVER, SHIM, os.path.abspath(__file__), os.path.join(CSRC, "trax_math.h"),
             os.path.join(CSRC, "trax_math_coeffs.h"), os.path.join(HERE, "trax_oracle.h")]
    return max(os.path.getmtime(p) for p in paths)


def build(force: bool = False) -> str:
    """Generates (when the reference is present) and compiles oracle/_ref/libtraxref.so.
    Returns the library path, or '' when neither the reference nor a generated file exists."""
    root = reference_dir()
    have_ref = os.path.isdir(os.path.join(root, "src", "algorithms"))
    if have_ref:
        srcs = [os.path.join(root, h) for h, _ in KERNELS] + [os.path.join(root, PREFIX_DEFINES_SRC),
                                                              os.path.join(root, TRACKS_SRC)]
        newest = max([os.path.getmtime(s) for s in srcs] + [_newest_input()])
        if force or not os.path.exists(GEN_CPP) or os.path.getmtime(GEN_CPP) < newest:
            generate(root)
        if force or not os.path.exists(GEN_TRACKS) or os.path.getmtime(GEN_TRACKS) < newest:
            generate_tracks(root)
    elif not (os.path.exists(GEN_CPP) and os.path.exists(GEN_TRACKS)):
        return ""
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(
            os.path.getmtime(GEN_CPP), os.path.getmtime(GEN_TRACKS), _newest_input()):
        compile_lib()
    return LIB_PATH


if __name__ == "__main__":
    path = build(force="--force" in sys.argv)
    print(path or "reference sources absent: nothing built")
