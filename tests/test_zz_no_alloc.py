"""The allocation-free scan entry point (trax_prefix_sum_noalloc).

Some callers of this library cannot allocate device memory themselves: they
run inside another framework's memory pool, or under an allocator that
forbids new device allocations, and hand the library device buffers they
already own.  This test plays such a caller: the input and output live in
buffers that the caller (here torch) owns, the entry point is called through
the C ABI, and its result must equal numpy's exclusive cumulative sum (cast to
uint32) and the ordinary scan entry point's (trax_prefix_sum) exactly, on two
calls in a row (the second smaller, so that scratch left over by the first
call would show).  Further cases: exactly TRAX_NOALLOC_SCAN_MAX elements, which
uses every status word of the fixed scratch array; an in-place call; and
pointers one element past a 16-byte boundary, which take the kernel's scalar
loads and stores.

The file is named to be collected last, so that a run stopping at the first
failure has run every other test before it.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIMIT = 16 * 1024 * 1024  # TRAX_NOALLOC_SCAN_MAX


def _noalloc_fn(capi):
    f = capi.load().trax_prefix_sum_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_char_p,
                  ctypes.c_size_t]
    f.restype = ctypes.c_int
    return f


def _expect(x):
    out = np.zeros(x.size, np.uint64)
    out[1:] = np.cumsum(x[:-1], dtype=np.uint64)
    return (out & 0xFFFFFFFF).astype(np.uint32)


def _call(f, torch, d_in_ptr, d_out_ptr, n):
    msg = ctypes.create_string_buffer(256)
    stream = torch.cuda.current_stream(0).cuda_stream
    rc = f(d_in_ptr, d_out_ptr, n, stream, msg, len(msg))
    assert rc == 0, msg.value.decode()


def test_noalloc_scan_matches_numpy_and_context_scan(trax_lib):
    torch = pytest.importorskip("torch")
    f = _noalloc_fn(trax_lib)
    rng = np.random.default_rng(7)
    with trax_lib.Context(0) as ctx:
        for n in (3_000_001, 1_234_567):
            x = rng.integers(0, 1 << 20, n, dtype=np.uint32)
            d_in = torch.from_numpy(x.view(np.int32)).to("cuda:0")
            d_out = torch.empty_like(d_in)
            _call(f, torch, d_in.data_ptr(), d_out.data_ptr(), n)
            got = d_out.cpu().numpy().view(np.uint32)
            assert np.array_equal(got, _expect(x))
            assert np.array_equal(got, ctx.prefix_sum(x))


def test_noalloc_scan_at_the_limit_in_place_and_unaligned(trax_lib):
    torch = pytest.importorskip("torch")
    f = _noalloc_fn(trax_lib)
    rng = np.random.default_rng(11)
    # exactly the limit: every status word of the scratch array in use
    x = rng.integers(0, 1 << 12, LIMIT, dtype=np.uint32)
    d_in = torch.from_numpy(x.view(np.int32)).to("cuda:0")
    d_out = torch.empty_like(d_in)
    _call(f, torch, d_in.data_ptr(), d_out.data_ptr(), LIMIT)
    assert np.array_equal(d_out.cpu().numpy().view(np.uint32), _expect(x))
    # in place
    y = rng.integers(0, 1 << 20, 777_777, dtype=np.uint32)
    d = torch.from_numpy(y.view(np.int32)).to("cuda:0")
    _call(f, torch, d.data_ptr(), d.data_ptr(), y.size)
    assert np.array_equal(d.cpu().numpy().view(np.uint32), _expect(y))
    # input and output 4 bytes past a 16-byte boundary
    z = rng.integers(0, 1 << 20, 500_001, dtype=np.uint32)
    d_in = torch.from_numpy(np.concatenate([[0], z]).astype(np.uint32).view(np.int32)).to("cuda:0")
    d_out = torch.zeros(z.size + 1, dtype=torch.int32, device="cuda:0")
    assert d_in.data_ptr() % 16 == 0 and d_out.data_ptr() % 16 == 0
    _call(f, torch, d_in.data_ptr() + 4, d_out.data_ptr() + 4, z.size)
    got = d_out.cpu().numpy().view(np.uint32)
    assert got[0] == 0
    assert np.array_equal(got[1:], _expect(z))


def test_noalloc_scan_rejects_sizes_above_limit(trax_lib):
    torch = pytest.importorskip("torch")
    f = _noalloc_fn(trax_lib)
    buf = torch.zeros(16, dtype=torch.int32, device="cuda:0")
    msg = ctypes.create_string_buffer(256)
    rc = f(buf.data_ptr(), buf.data_ptr(), LIMIT + 1, None, msg, len(msg))
    assert rc == 2
    assert b"limit" in msg.value
