"""The bounded device waits' error path, made to run out on purpose without a
GPU fault.

Every single-pass scan's tiles wait for their predecessors' look-back status
with a bounded number of polls.  A host-set fault (trax_debug_skip_publish /
trax_noalloc_set_wait) makes one tile publish nothing, so the waits after it
give up: the kernel records the timeout, finishes, and the call returns
TRAX_ERR_TIMEOUT.  The wait limit is set short (a few thousand polls of about
64 ns) so that the test takes milliseconds.  Only the standalone scans are
faulted: their wrong sums land in the call's own output buffer, which nothing
else reads.  Afterwards the same context (and the no-alloc entry point) must
scan correctly again.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TRAX_ERR_TIMEOUT = 4
TILE = 4096


def _expect(x):
    out = np.zeros(x.size, np.uint64)
    out[1:] = np.cumsum(x[:-1], dtype=np.uint64)
    return (out & 0xFFFFFFFF).astype(np.uint32)


@pytest.mark.parametrize("skip_tile", [0, 3])
def test_context_scan_times_out_then_recovers(trax_lib, skip_tile):
    rng = np.random.default_rng(5)
    x = rng.integers(0, 1 << 16, 40 * TILE + 17, dtype=np.uint32)
    with trax_lib.Context(0) as ctx:
        assert np.array_equal(ctx.prefix_sum(x), _expect(x))
        ctx.set_wait_limit(polls=2000, skip_publish_tile=skip_tile)
        with pytest.raises(trax_lib.TraxError) as e:
            ctx.prefix_sum(x)
        assert e.value.code == TRAX_ERR_TIMEOUT
        ctx.set_wait_limit()  # default limit, no fault
        assert np.array_equal(ctx.prefix_sum(x), _expect(x))


def test_noalloc_scan_times_out_then_recovers(trax_lib):
    torch = pytest.importorskip("torch")
    L = trax_lib.load()
    f = L.trax_prefix_sum_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_char_p,
                  ctypes.c_size_t]
    f.restype = ctypes.c_int
    rng = np.random.default_rng(9)
    x = rng.integers(0, 1 << 16, 30 * TILE, dtype=np.uint32)
    d_in = torch.from_numpy(x.view(np.int32)).to("cuda:0")
    d_out = torch.empty_like(d_in)
    stream = torch.cuda.current_stream(0).cuda_stream
    msg = ctypes.create_string_buffer(256)
    try:
        assert L.trax_noalloc_set_wait(2000, 2) == 0
        rc = f(d_in.data_ptr(), d_out.data_ptr(), x.size, stream, msg, len(msg))
        assert rc == TRAX_ERR_TIMEOUT, msg.value.decode()
        assert b"ran out" in msg.value
    finally:
        assert L.trax_noalloc_set_wait(0, 0xFFFFFFFF) == 0
    rc = f(d_in.data_ptr(), d_out.data_ptr(), x.size, stream, msg, len(msg))
    assert rc == 0, msg.value.decode()
    assert np.array_equal(d_out.cpu().numpy().view(np.uint32), _expect(x))
