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


def test_dphi_decision_never_disagrees_with_atan2(oracle_lib, rng):
    """The filter kernel decides the dphi cut from the cross and dot products
    of the two transverse segments wherever that is certain; it must never
    contradict the atan2 evaluation of filterCount
    (TripletThetaPhiFilter.h:118-128), and away from the cut it must decide."""
    f32 = np.float32
    n = 1_000_000
    cuts = rng.choice(np.array([0.0, 0.01, 0.075, 0.2, 0.4, 1.0], f32), n)
    lu, lv = 10.0 ** rng.uniform(-2, 2.5, n), 10.0 ** rng.uniform(-2, 2.5, n)
    a = rng.uniform(-np.pi, np.pi, n)
    near = rng.random(n) < 0.6
    d = np.where(near, cuts.astype(np.float64) + rng.uniform(-3e-4, 3e-4, n), rng.uniform(0, np.pi, n))
    d *= rng.choice([-1.0, 1.0], n)
    ox, oy = rng.uniform(-60, 60, (2, n))  # hit coordinates, then the segments as the kernel forms them
    ax, ay = ox.astype(f32), oy.astype(f32)
    bx, by = (ox + lu * np.cos(a)).astype(f32), (oy + lu * np.sin(a)).astype(f32)
    cx, cy = (bx + lv * np.cos(a + d)).astype(f32), (by + lv * np.sin(a + d)).astype(f32)
    ux, uy, vx, vy = bx - ax, by - ay, cx - bx, cy - by
    exact, dec = oracle_lib.dphi_check(ux, uy, vx, vy, cuts)
    assert np.all((dec == -1) | (dec == exact))
    ang = np.abs(np.angle((vx + 1j * vy).astype(np.complex128) / (ux + 1j * uy).astype(np.complex128)))
    far = np.abs(ang - cuts) > 2e-4
    assert np.mean(dec[far] == -1) < 1e-4
    assert np.mean(dec[~far] == -1) > 0.3  # the band around the cut goes to atan2
    # degenerate segments and cuts: undecided or equal
    specials = np.array([0.0, -0.0, 1e-20, -1e-20, 1e-38, 1.0, -1.0, 1e20, np.inf, -np.inf, np.nan], f32)
    g = np.stack(np.meshgrid(specials, specials, specials, specials, indexing="ij"), 0).reshape(4, -1)
    for cut in (0.075, 0.0, -0.1, 1.5, np.nan, np.inf):
        c = np.full(g.shape[1], cut, f32)
        exact, dec = oracle_lib.dphi_check(g[0], g[1], g[2], g[3], c)
        assert np.all((dec == -1) | (dec == exact)), cut
