"""The bounds-checked debug build (-DTRAX_BOUNDS_CHECK, libtrax_gb300_checked.so).

No memory checker runs on this hardware, so this build checks every
data-dependent hit index on the device (grid offsets, pairs, candidates,
triplets): an index outside the batch sets TRAX_EBIT_BOUNDS, reads hit 0
instead and fails the call with TRAX_ERR_DEVICE_ASSERT.  The parity cases
below (with the grid walk and the fine z grid walk of the prediction count)
run through it in a child process (TRAX_GB300_BOUNDS_CHECK=1 selects
the library): every call must finish without a bounds error and every array
must equal the oracle's, as with the product build.
"""
import os
import subprocess
import sys
import textwrap

import pytest

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = textwrap.dedent("""
    import dataclasses, sys
    sys.path.insert(0, {repo!r})
    from oracle import oracle
    from tests.test_gpu_parity import compare, stagewise
    from tests.test_oracle_kats import degenerate_batch
    from trax_gb300 import capi, events
    assert capi.library_path().endswith("libtrax_gb300_checked.so"), capi.library_path()
    oracle.build()
    cases = [("config 0", events.generate(0)), ("config 1", events.generate(1)),
             ("ttbar-like", events.generate(2, n_events=12)), ("degenerate", degenerate_batch()),
             ("pileup event", events.generate_workload(
                 dataclasses.replace(events.workload(3), n_events=1, n_vertices=6)))]
    ctx = capi.Context(0)
    for name, batch in cases:
        ref = oracle.run(batch)[0]
        ctx.upload(batch)
        for graph, fine in ((True, 0), (False, 0), (True, 4)):
            ctx.set_fine_rows(fine)  # 4: the prediction count walks the fine z grid
            ctx.seed_batch(use_graph=graph)  # a bounds error raises TraxError here
            compare(ctx.results(), ref)
        ctx.set_fine_rows(0)
        print(name, "clean", flush=True)
    compare(stagewise(ctx, events.generate(1)), oracle.run(events.generate(1))[0])
    print("stage by stage clean", flush=True)
    ctx.close()
""")


def test_checked_build_runs_the_parity_cases_clean():
    from trax_gb300 import build
    build.build(checked=True)
    env = dict(os.environ, TRAX_GB300_BOUNDS_CHECK="1")
    r = subprocess.run([sys.executable, "-c", CHILD.format(repo=REPO)], env=env, cwd=REPO, capture_output=True,
                       text=True, timeout=1800)
    print(r.stdout)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert "stage by stage clean" in r.stdout
