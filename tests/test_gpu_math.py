"""trax_math.h on the device (trax_math_eval) against the same header built
for the CPU (the oracle): every function must give the same bits, so that
the kernels' predicates decide exactly as the oracle's.  Also the accuracy
of our functions against CUDA's own (atan2f, acosf, atanf, asinhf, logf)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SPECIAL = np.array([0.0, -0.0, 1.0, -1.0, 0.5, -0.5, 2.0, np.inf, -np.inf, np.nan, 1e-45, -1e-45, 1.1754942e-38,
                    1.1754944e-38, 3.4028235e38, -3.4028235e38, np.pi, -np.pi, np.pi / 2, 0.99999994, -0.99999994,
                    1.0000001, -1.0000001, 2147483520.0, 2147483648.0, -2147483648.0, -2147483904.0,
                    4294967040.0, 4294967296.0, 16777216.0, 16777217.0, 0.49999997, 0.50000006, -0.9999999,
                    -1.5, 1.5, 1e10, -1e10, 1e-10, 300.0, -300.0, 2.4, 7.5e-3], dtype=np.float32)


def _inputs(n=1 << 20, seed=1):
    rng = np.random.default_rng(seed)
    bits = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)  # every class: NaN, inf, subnormal
    wide = bits.view(np.float32)
    unit = rng.uniform(-1.2, 1.2, n).astype(np.float32)
    scaled = (rng.standard_normal(n) * np.exp(rng.uniform(-12, 12, n))).astype(np.float32)
    return np.concatenate([SPECIAL, wide, unit, scaled])


def _same_bits(got, want):
    g, w = got.view(np.uint32), want.view(np.uint32)
    both_nan = np.isnan(got) & np.isnan(want)
    bad = (g != w) & ~both_nan
    return int(bad.sum()), np.nonzero(bad)[0][:5]


@pytest.mark.parametrize("fn", ["atan2", "acos", "atan", "asinh", "log", "div", "sqrt", "floor"])
def test_device_math_has_the_cpu_bits(trax_lib, oracle_lib, fn):
    a = _inputs()
    b = np.roll(_inputs(seed=2), 7)[:a.size] if fn in ("atan2", "div") else None
    got = trax_lib.math_eval(fn, a, b)
    want = oracle_lib.math_eval(fn, a, b)
    n_bad, where = _same_bits(got, want)
    assert n_bad == 0, (fn, [(float(a[i]), None if b is None else float(b[i]), float(got[i]), float(want[i]))
                             for i in where])


@pytest.mark.parametrize("fn,view", [("f2u_sat", np.uint32), ("f2i_sat", np.int32)])
def test_saturating_conversions_match_the_portable_definition(trax_lib, oracle_lib, fn, view):
    """The device converts with one instruction (truncate, clamp, NaN -> 0); the
    CPU build spells the same definition out."""
    a = _inputs()
    got = trax_lib.math_eval(fn, a).view(view)
    want = oracle_lib.math_eval(fn, a).view(view)
    assert np.array_equal(got, want)
    s = trax_lib.math_eval(fn, SPECIAL).view(view)

    def at(v):
        return int(s[int(np.nonzero(SPECIAL == np.float32(v))[0][0])])
    if view is np.uint32:
        assert at(4294967296.0) == 0xFFFFFFFF and at(-1.0) == 0 and at(0.99999994) == 0 and at(1.5) == 1
        assert at(np.inf) == 0xFFFFFFFF and at(-np.inf) == 0
    else:
        assert at(2147483648.0) == 2147483647 and at(-1.5) == -1 and at(-2147483904.0) == -(1 << 31)
        assert at(-np.inf) == -(1 << 31) and at(np.inf) == 2147483647
    nan_at = int(np.nonzero(np.isnan(SPECIAL))[0][0])
    assert s[nan_at] == 0


def _ulps(x, y):
    def key(v):
        i = v.view(np.int32).astype(np.int64)
        return np.where(i < 0, -(i & 0x7FFFFFFF), i)
    return np.abs(key(x) - key(y))


# bounds: ours is within about 1 ulp of the exact value (tests/test_math.py),
# CUDA's within its documented maximum (atan2f 3, acosf 2, atanf 2, asinhf 3,
# logf 1 ulp)
@pytest.mark.parametrize("fn,domain,max_ulp", [("atan2", None, 4), ("acos", (-1.0, 1.0), 3), ("atan", None, 3),
                                               ("asinh", None, 4), ("log", (1e-30, 1e30), 2)])
def test_accuracy_against_cuda(trax_lib, fn, domain, max_ulp):
    rng = np.random.default_rng(5)
    n = 1 << 20
    if domain is None:
        a = (rng.standard_normal(n) * np.exp(rng.uniform(-8, 8, n))).astype(np.float32)
    elif fn == "log":
        a = np.exp(rng.uniform(np.log(domain[0]), np.log(domain[1]), n)).astype(np.float32)
    else:
        a = rng.uniform(*domain, n).astype(np.float32)
    b = (rng.standard_normal(n) * np.exp(rng.uniform(-8, 8, n))).astype(np.float32) if fn == "atan2" else None
    ours = trax_lib.math_eval(fn, a, b)
    cuda = trax_lib.math_eval("cuda_" + fn + "f", a, b)
    assert np.array_equal(np.isnan(ours), np.isnan(cuda))
    ok = ~np.isnan(ours)
    d = _ulps(ours[ok], cuda[ok])
    print(fn, "max ulp vs CUDA", int(d.max()), "share equal", float((d == 0).mean()))
    assert d.max() <= max_ulp
