"""Differentiable triplet fit on the GPU (trax_fit_*), against the FP64 CPU
reference of the same fit (oracle/align_ref.py): parameters, chi2, the
adjoint's alignment and hit gradients against the FP64 adjoint and against
FP64 central finite differences (h = 1e-6), and the recovery of injected
layer shifts by 50 gradient evaluations."""
import numpy as np
import pytest

from trax_gb300 import align as AL
from trax_gb300 import events

pytestmark = pytest.mark.gpu

RADII = np.array(events.BARREL10_RADII)


def _prepared(trax_lib, n_events, seed=None, truth_only=True):
    batch = events.generate(4, n_events=n_events, seed=seed)
    ctx = trax_lib.Context(0)
    ctx.upload(batch)
    ctx.seed_batch(use_graph=True, run_linking=False)
    n_fit = ctx.fit_prepare(truth_only=truth_only)
    rows, sig = ctx.fit_rows()
    h1, h2, h3, _ = ctx.triplets()
    perm = ctx.hit_perm()
    ref = dict(x=batch.x[perm], y=batch.y[perm], z=batch.z[perm], layer=batch.layer[perm],
               h1=h1[rows].astype(np.int64), h2=h2[rows].astype(np.int64), h3=h3[rows].astype(np.int64),
               w=np.ones(n_fit), sigma_tip=sig[batch.layer[perm][h1[rows]] - 1].astype(np.float64))
    return batch, ctx, ref, perm


def _ref_args(ref):
    return (ref["x"], ref["y"], ref["z"], ref["layer"], ref["h1"], ref["h2"], ref["h3"], ref["w"])


@pytest.fixture(scope="module")
def small(trax_lib):
    batch, ctx, ref, perm = _prepared(trax_lib, 12)
    yield batch, ctx, ref, perm
    ctx.close()


def test_fit_rows_are_truth_matched_and_grouped(small):
    batch, ctx, ref, perm = small
    assert ctx.n_fit > 1000
    tid = batch.hit_id[perm]
    assert np.all(tid[ref["h1"]] == tid[ref["h2"]]) and np.all(tid[ref["h2"]] == tid[ref["h3"]])
    lt = ref["layer"][ref["h1"]]
    assert np.all(np.diff(lt.astype(np.int64)) >= 0)  # rows ordered by layer triplet


# Each fit parameter's error against FP64 (on the same FP32 hits), relative
# to its natural scale: the curvature to |kappa| + 1e-4 / cm (a 114 GeV track
# in 3.8 T, below the triplets' curvature resolution: kappa -> 0 is a
# straight track, where a bare relative error has no meaning); cot(theta) to
# max(|t|, 1); the impact parameter d0 to |d0| + r1, the lever arm from the
# first hit to the beam line; z0 to |z0| + r1 max(|t|, 1), the length of the
# extrapolation from the first hit.  The bar is 1e-5 for each, worst row.
KAPPA_FLOOR = 1e-4


def fit_param_errors(params, p64, r1):
    P = params.astype(np.float64)
    k, d0, z0, t = (p64[:, i] for i in range(4))
    return {"kappa": np.abs(P[:, 0] - k) / (np.abs(k) + KAPPA_FLOOR),
            "d0": np.abs(P[:, 1] - d0) / (np.abs(d0) + r1),
            "z0": np.abs(P[:, 2] - z0) / (np.abs(z0) + r1 * np.maximum(np.abs(t), 1.0)),
            "cot_theta": np.abs(P[:, 3] - t) / np.maximum(np.abs(t), 1.0),
            "kappa_relative": np.abs(P[:, 0] - k) / np.abs(k)}


@pytest.mark.parametrize("at", ["zero", "shifted"])
def test_fit_params_and_chi2_match_fp64(small, align_ref, at):
    batch, ctx, ref, _ = small
    a = np.zeros((batch.n_layers, 3))
    if at == "shifted":
        rng = np.random.default_rng(3)
        a = np.stack([rng.normal(0, 0.003, batch.n_layers), rng.normal(0, 0.003, batch.n_layers),
                      rng.normal(0, 1e-5, batch.n_layers)], axis=1)
    chi2, params = ctx.fit_forward(a, params=True)
    p64 = align_ref.triplet_params(ref["x"], ref["y"], ref["z"], ref["layer"], ref["h1"], ref["h2"], ref["h3"], a)
    l64 = align_ref.loss(*_ref_args(ref), a, ref["sigma_tip"], 0.002)
    assert abs(chi2 - l64) <= 1e-4 * l64
    r1 = np.hypot(ref["x"][ref["h1"]], ref["y"][ref["h1"]])
    err = fit_param_errors(params, p64, r1)
    # measured worst rows: 8.4e-7 (kappa), 3.3e-7 (d0), 6.5e-7 (z0), 4.7e-7 (cot theta)
    for k in ("kappa", "d0", "z0", "cot_theta"):
        assert err[k].max() <= 1e-5, (k, float(err[k].max()))
    assert np.median(err["kappa_relative"]) <= 1e-6


@pytest.mark.parametrize("at", ["zero", "shifted"])
def test_alignment_gradient_matches_fp64_and_finite_differences(small, align_ref, at):
    batch, ctx, ref, _ = small
    rng = np.random.default_rng(7)
    a = np.zeros((batch.n_layers, 3))
    if at == "shifted":
        a = np.stack([rng.normal(0, 0.003, batch.n_layers), rng.normal(0, 0.003, batch.n_layers),
                      rng.normal(0, 1e-5, batch.n_layers)], axis=1)
    chi2, g, _ = ctx.fit_backward(a)
    l64, g64, _ = align_ref.loss_and_grad(*_ref_args(ref), a, ref["sigma_tip"], 0.002)
    fd = align_ref.fd_grad_align(*_ref_args(ref), a, ref["sigma_tip"], 0.002, h=1e-6)
    assert abs(chi2 - l64) <= 1e-4 * l64
    # the FP64 adjoint and the FP64 differences agree to 1e-7; the FP32
    # adjoint kernel must be within 1e-4 of the differences
    assert np.linalg.norm(g64 - fd) <= 1e-6 * np.linalg.norm(fd)
    assert np.linalg.norm(g - fd) <= 1e-4 * np.linalg.norm(fd)
    big = np.abs(fd) > 1e-2 * np.abs(fd).max()
    assert np.all(np.abs(g - fd)[big] <= 1e-3 * np.abs(fd)[big])


def test_hit_gradient_matches_fp64_adjoint(small, align_ref):
    batch, ctx, ref, perm = small
    a = np.zeros((batch.n_layers, 3))
    _, _, gh = ctx.fit_backward(a, hits=True)
    _, _, gh64 = align_ref.loss_and_grad(*_ref_args(ref), a, ref["sigma_tip"], 0.002)
    want = np.zeros_like(gh64)
    want[perm] = gh64  # grid order -> input order
    assert gh.shape == want.shape
    # measured 1.6e-4 (the FP32 reverse pass through the circle and arc lengths)
    assert np.linalg.norm(gh - want) <= 3e-4 * np.linalg.norm(want)
    # hits that are in no fit row have zero gradient
    used = np.zeros(batch.n_hits, bool)
    used[perm[np.concatenate([ref["h1"], ref["h2"], ref["h3"]])]] = True
    assert np.all(gh[~used] == 0)


def test_gauss_newton_diagonal_matches_fp64(small, align_ref):
    batch, ctx, ref, _ = small
    a = np.zeros((batch.n_layers, 3))
    _, _, _, gn = ctx.fit_backward(a, squares=True)
    gn64 = align_ref.gn_diag(*_ref_args(ref), a, ref["sigma_tip"], 0.002)
    used = gn64 > 0
    assert np.all(np.abs(gn - gn64)[used] <= 1e-3 * gn64[used])


def test_fit_needs_prepare_on_current_triplets(trax_lib):
    batch = events.generate(4, n_events=2)
    ctx = trax_lib.Context(0)
    try:
        ctx.upload(batch)
        ctx.seed_batch(use_graph=False, run_linking=False)
        with pytest.raises(trax_lib.TraxError) as e:
            ctx.fit_forward(np.zeros((batch.n_layers, 3)))
        assert e.value.code == 6
        ctx.fit_prepare()
        ctx.fit_forward(np.zeros((batch.n_layers, 3)))
        ctx.seed_batch(use_graph=False, run_linking=False)  # new triplets
        with pytest.raises(trax_lib.TraxError):
            ctx.fit_backward(np.zeros((batch.n_layers, 3)))
    finally:
        ctx.close()


def test_fit_chi2_is_deterministic(small):
    batch, ctx, _, _ = small
    a = np.full((batch.n_layers, 3), 1e-4)
    r1 = ctx.fit_backward(a, squares=True)
    r2 = ctx.fit_backward(a, squares=True)
    assert r1[0] == r2[0] and np.array_equal(r1[1], r2[1]) and np.array_equal(r1[3], r2[3])


def test_apply_alignment_moves_the_uploaded_hits(trax_lib):
    """chi2 at shifts a on the original hits == chi2 at zero on the hits moved by a."""
    batch = events.generate(4, n_events=3)
    ctx = trax_lib.Context(0)
    try:
        ctx.upload(batch)
        ctx.seed_batch(use_graph=False, run_linking=False)
        h1, h2, h3, _ = ctx.triplets()
        perm = ctx.hit_perm()
        t1, t2, t3 = perm[h1], perm[h2], perm[h3]  # input-order hit indices
        a = np.stack([np.full(batch.n_layers, 0.004), np.full(batch.n_layers, -0.003),
                      np.full(batch.n_layers, 3e-5)], axis=1)
        sig = [0.01] * len(batch.lts)
        ctx.set_tracklets(t1, t2, t3)
        n1 = ctx.fit_prepare(sigma_tip=sig)
        chi2_before, p_before = ctx.fit_forward(a, params=True)
        ctx.apply_alignment(a)
        ctx.set_tracklets(t1, t2, t3)
        n2 = ctx.fit_prepare(sigma_tip=sig)
        chi2_after, p_after = ctx.fit_forward(np.zeros((batch.n_layers, 3)), params=True)
        assert n1 == n2 > 0
        assert chi2_after == pytest.approx(chi2_before, rel=1e-4)
        # moved hits are rounded to FP32 once more: parameters agree to that level
        rel_k = np.abs(p_after[:, 0] - p_before[:, 0]) / np.abs(p_before[:, 0])
        assert np.quantile(rel_k, 0.99) < 1e-3
        assert np.quantile(np.abs(p_after[:, 1] - p_before[:, 1]), 0.99) < 1e-4  # d0 [cm]
        assert np.quantile(np.abs(p_after[:, 2] - p_before[:, 2]), 0.99) < 1e-4  # z0 [cm]
        assert np.quantile(np.abs(p_after[:, 3] - p_before[:, 3]), 0.99) < 1e-4  # cot theta
    finally:
        ctx.close()


def test_fifty_gradient_steps_recover_the_injected_shifts(trax_lib):
    batch = events.generate(4)
    ctx = trax_lib.Context(0)
    try:
        ctx.upload(batch)
        ctx.seed_batch(use_graph=True, run_linking=False)
        ctx.fit_prepare(truth_only=True)
        a, hist = AL.align_context(ctx, RADII, steps=50)
        assert hist[-1].evaluations <= 50
        res = AL.Gauge(RADII).residual_um(a, batch.misalignment)
        print("recovery residual (um):", np.array2string(res, precision=2))
        assert np.abs(res).max() <= 5.0, res
        assert hist[-1].loss < 0.5 * hist[0].loss
    finally:
        ctx.close()
