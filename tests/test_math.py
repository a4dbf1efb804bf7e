"""Accuracy of the shared FP32 math (trax_math.h) against float64.

The same functions run in the oracle and in the kernels, so their results
are identical on both sides by construction; these tests bound how far they
are from the exact functions (in units in the last place of float32) and
check the C99 Annex F special cases the cut predicates can meet.
"""
import numpy as np
import pytest


def ulp_err(got: np.ndarray, exact: np.ndarray) -> np.ndarray:
    ref = exact.astype(np.float32)
    spacing = np.spacing(np.abs(ref)).astype(np.float64)
    spacing[spacing == 0] = np.finfo(np.float32).tiny
    return np.abs(got.astype(np.float64) - exact) / spacing


@pytest.fixture(scope="module")
def rng():
    return np.random.default_rng(1234)


def test_atan2_accuracy(oracle_lib, rng):
    n = 400000
    mag = 10.0 ** rng.uniform(-6, 6, (2, n))
    y = (rng.choice([-1, 1], n) * mag[0]).astype(np.float32)
    x = (rng.choice([-1, 1], n) * mag[1]).astype(np.float32)
    got = oracle_lib.math_eval("atan2", y, x)
    exact = np.arctan2(y.astype(np.float64), x.astype(np.float64))
    assert ulp_err(got, exact).max() <= 3.0
    # hit-like coordinates (barrel radii), where the grid's phi cells are cut
    ang = rng.uniform(-np.pi, np.pi, n)
    r = rng.uniform(4.0, 110.0, n)
    y, x = (r * np.sin(ang)).astype(np.float32), (r * np.cos(ang)).astype(np.float32)
    got = oracle_lib.math_eval("atan2", y, x)
    assert ulp_err(got, np.arctan2(y.astype(np.float64), x.astype(np.float64))).max() <= 3.0
    assert np.all(np.abs(got) <= np.float32(np.pi))


def test_atan2_special_cases(oracle_lib):
    pi = np.float32(np.pi)
    inf = np.float32(np.inf)
    cases = [(0.0, 1.0, 0.0), (-0.0, 1.0, -0.0), (0.0, -1.0, pi), (-0.0, -1.0, -pi), (0.0, 0.0, 0.0),
             (0.0, -0.0, pi), (1.0, 0.0, np.float32(np.pi / 2)), (-1.0, 0.0, -np.float32(np.pi / 2)),
             (inf, 1.0, np.float32(np.pi / 2)), (1.0, inf, 0.0), (1.0, -inf, pi), (inf, inf, np.float32(np.pi / 4))]
    y = np.array([c[0] for c in cases], dtype=np.float32)
    x = np.array([c[1] for c in cases], dtype=np.float32)
    got = oracle_lib.math_eval("atan2", y, x)
    want = np.array([c[2] for c in cases], dtype=np.float32)
    assert np.allclose(got, want, rtol=2e-7, atol=0)
    assert np.array_equal(np.signbit(got), np.signbit(want))
    assert np.isnan(oracle_lib.math_eval("atan2", np.array([np.nan], np.float32), np.array([1.0], np.float32)))[0]


def test_acos_accuracy(oracle_lib, rng):
    x = np.concatenate([rng.uniform(-1, 1, 400000), np.linspace(-1, 1, 10001),
                        rng.uniform(0.0, 0.2, 100000)]).astype(np.float32)
    got = oracle_lib.math_eval("acos", x)
    assert ulp_err(got, np.arccos(x.astype(np.float64))).max() <= 3.0
    edge = oracle_lib.math_eval("acos", np.array([1.0, -1.0, 1.0000001, -1.5, np.nan], np.float32))
    assert edge[0] == 0.0 and edge[1] == np.float32(np.pi) and np.all(np.isnan(edge[2:]))


def test_atan_accuracy(oracle_lib, rng):
    x = (rng.choice([-1, 1], 500000) * 10.0 ** rng.uniform(-8, 8, 500000)).astype(np.float32)
    got = oracle_lib.math_eval("atan", x)
    assert ulp_err(got, np.arctan(x.astype(np.float64))).max() <= 3.0
    assert oracle_lib.math_eval("atan", np.array([np.inf], np.float32))[0] == np.float32(np.pi / 2)


def test_asinh_and_log_accuracy(oracle_lib, rng):
    x = (rng.choice([-1, 1], 500000) * 10.0 ** rng.uniform(-7, 6, 500000)).astype(np.float32)
    got = oracle_lib.math_eval("asinh", x)
    assert ulp_err(got, np.arcsinh(x.astype(np.float64))).max() <= 3.0
    p = (10.0 ** rng.uniform(-40, 38, 500000)).astype(np.float32)
    p = p[p > 0]
    got = oracle_lib.math_eval("log", p)
    assert ulp_err(got, np.log(p.astype(np.float64))).max() <= 3.0


def test_min_radius_curvature(oracle_lib):
    # TripletConfiguration.cpp:36-43: 87.52 cm at 1 GeV, 61.27 cm at 0.7 GeV (IDEAL_BZ = 3.8112 T)
    assert abs(oracle_lib.min_radius_curvature(1.0) - 87.52) < 0.01
    assert abs(oracle_lib.min_radius_curvature(0.7) - 61.27) < 0.01
