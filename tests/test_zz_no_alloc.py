"""The allocation-free scan entry point (trax_prefix_sum_noalloc).

Some callers of this library cannot allocate device memory themselves: they
run inside another framework's memory pool, or under an allocator that
forbids new device allocations, and hand the library device buffers they
already own.  This test plays such a caller: the input and output live in
buffers that the caller (here torch) owns, the entry point is called through
the C ABI, and its result must equal the result of the ordinary scan entry
point (trax_prefix_sum) exactly, on two calls in a row (the second smaller, so
that scratch left over by the first call would show).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc_fn(capi):
    f = capi.load().trax_prefix_sum_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_char_p,
                  ctypes.c_size_t]
    f.restype = ctypes.c_int
    return f


def test_noalloc_scan_matches_context_scan(trax_lib):
    torch = pytest.importorskip("torch")
    f = _noalloc_fn(trax_lib)
    rng = np.random.default_rng(7)
    with trax_lib.Context(0) as ctx:
        for n in (3_000_001, 1_234_567):
            x = rng.integers(0, 1 << 20, n, dtype=np.uint32)
            ref = ctx.prefix_sum(x)
            d_in = torch.from_numpy(x.view(np.int32)).to("cuda:0")
            d_out = torch.empty_like(d_in)
            msg = ctypes.create_string_buffer(256)
            stream = torch.cuda.current_stream(0).cuda_stream
            rc = f(d_in.data_ptr(), d_out.data_ptr(), n, stream, msg, len(msg))
            assert rc == 0, msg.value.decode()
            got = d_out.cpu().numpy().view(np.uint32)
            assert np.array_equal(got, ref)


def test_noalloc_scan_rejects_sizes_above_limit(trax_lib):
    torch = pytest.importorskip("torch")
    f = _noalloc_fn(trax_lib)
    limit = 16 * 1024 * 1024
    buf = torch.zeros(16, dtype=torch.int32, device="cuda:0")
    msg = ctypes.create_string_buffer(256)
    rc = f(buf.data_ptr(), buf.data_ptr(), limit + 1, None, msg, len(msg))
    assert rc == 2
    assert b"limit" in msg.value
