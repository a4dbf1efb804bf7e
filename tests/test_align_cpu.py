"""CPU checks of the alignment machinery: the FP64 reference adjoint against
FP64 central differences and against torch autograd, the Gauss-Newton
diagonal, the weak-mode gauge, and the host-side optimiser."""
import numpy as np
import pytest

from trax_gb300 import align as AL
from trax_gb300 import events

RADII = np.array(events.BARREL10_RADII)


@pytest.fixture(scope="module")
def sample(oracle_lib):
    b = events.generate(4, n_events=4)
    r = oracle_lib.run(b)[0]
    perm = r["perm"]
    x, y, z, lay, tid = b.x[perm], b.y[perm], b.z[perm], b.layer[perm], b.hit_id[perm]
    h1, h2, h3 = (r[k].astype(np.int64) for k in ("trip_h1", "trip_h2", "trip_h3"))
    keep = (tid[h1] == tid[h2]) & (tid[h2] == tid[h3]) & (tid[h1] > 0)
    h1, h2, h3 = h1[keep], h2[keep], h3[keep]
    return b, (x, y, z, lay, h1, h2, h3, np.ones(h1.size))


def test_fp64_adjoint_matches_finite_differences(sample, align_ref):
    b, args = sample
    a = np.zeros((b.n_layers, 3))
    a[:, 0] = 0.002
    a[:, 2] = 1e-5
    _, g, _ = align_ref.loss_and_grad(*args, a, 0.01, 0.002)
    fd = align_ref.fd_grad_align(*args, a, 0.01, 0.002, h=1e-6)
    assert np.linalg.norm(g - fd) <= 1e-6 * np.linalg.norm(fd)


def test_fp64_adjoint_matches_torch_autograd(sample, align_ref):
    torch = pytest.importorskip("torch")
    b, (x, y, z, lay, h1, h2, h3, w) = sample
    st, sz = 0.01, 0.002
    a = np.zeros((b.n_layers, 3))
    _, g, gh = align_ref.loss_and_grad(x, y, z, lay, h1, h2, h3, w, a, st, sz)
    al = torch.zeros((b.n_layers, 3), dtype=torch.float64, requires_grad=True)
    xx, yy, zz = (torch.tensor(v.astype(np.float64), requires_grad=True) for v in (x, y, z))
    li = torch.as_tensor(lay.astype(np.int64) - 1)
    A = al[li]
    r = torch.sqrt(xx * xx + yy * yy)
    f = (r + A[:, 0]) / r
    c, s = torch.cos(A[:, 2]), torch.sin(A[:, 2])
    X, Y, Z = f * (xx * c - yy * s), f * (xx * s + yy * c), zz + A[:, 1]
    H = [torch.as_tensor(h) for h in (h1, h2, h3)]
    P = [(X[h], Y[h]) for h in H]
    Zs = [Z[h] for h in H]
    u2, v2 = P[1][0] - P[0][0], P[1][1] - P[0][1]
    u3, v3 = P[2][0] - P[0][0], P[2][1] - P[0][1]
    q2, q3 = u2 * u2 + v2 * v2, u3 * u3 + v3 * v3
    D = 2 * (u2 * v3 - u3 * v2)
    aa, bb = (v3 * q2 - v2 * q3) / D, (u2 * q3 - u3 * q2) / D
    R = torch.sqrt(aa * aa + bb * bb)
    Cx, Cy = P[0][0] + aa, P[0][1] + bb
    Cn = torch.sqrt(Cx * Cx + Cy * Cy)
    d0 = (P[0][0] ** 2 + P[0][1] ** 2 + 2 * (P[0][0] * aa + P[0][1] * bb)) / (Cn + R)
    sarc = [2 * R * torch.asin(torch.sqrt(px * px + py * py) / (2 * R)) for px, py in P]
    sb, zb = sum(sarc) / 3, sum(Zs) / 3
    t = sum((si - sb) * (zi - zb) for si, zi in zip(sarc, Zs)) / sum((si - sb) ** 2 for si in sarc)
    z0 = zb - t * sb
    loss = ((d0 / st) ** 2 + sum((zi - z0 - t * si) ** 2 for si, zi in zip(sarc, Zs)) / sz ** 2).sum()
    loss.backward()
    assert np.linalg.norm(al.grad.numpy() - g) <= 1e-10 * np.linalg.norm(g)
    gt = np.stack([xx.grad.numpy(), yy.grad.numpy(), zz.grad.numpy()], axis=1)
    assert np.linalg.norm(gt - gh) <= 1e-10 * np.linalg.norm(gh)


def test_weak_modes_leave_chi2_nearly_unchanged(sample, align_ref):
    b, args = sample
    a0 = np.zeros((b.n_layers, 3))
    l0 = align_ref.loss(*args, a0, 0.01, 0.002)
    M = AL.weak_modes(RADII)
    exact = [0, 1]  # common rotation and common z shift: exact symmetries
    for k in range(M.shape[1]):
        step = M[:, k].reshape(-1, 3) * np.array([1e-3 / 78.0, 1e-3 / 78.0, 1e-5 / 78.0])
        if k in exact:
            step = M[:, k].reshape(-1, 3) * np.array([1e-3, 1e-3, 1e-5])
        dl = align_ref.loss(*args, step, 0.01, 0.002) - l0
        assert abs(dl) <= 1e-3 * l0 if k in exact else abs(dl) <= 0.05 * l0


def test_gauge_projection_and_residual():
    g = AL.Gauge(RADII)
    M = AL.weak_modes(RADII)
    for k in range(M.shape[1]):
        z = g.to_scaled(M[:, k].reshape(-1, 3))
        assert np.linalg.norm(g.project(z)) <= 1e-9 * np.linalg.norm(z)
    truth = np.random.default_rng(3).normal(0, 0.005, (RADII.size, 3))
    moved = truth + 0.01 * M[:, 2].reshape(-1, 3) + 0.002 * M[:, 5].reshape(-1, 3)
    assert np.abs(g.residual_um(moved, truth)).max() < 1e-6


def test_lbfgs_solves_an_ill_conditioned_quadratic():
    rng = np.random.default_rng(5)
    n = 30
    Q, _ = np.linalg.qr(rng.normal(size=(n, n)))
    ev = np.logspace(0, 4, n)
    A = Q @ np.diag(ev) @ Q.T
    xs = rng.normal(size=n)

    def fg(x):
        d = x - xs
        return 0.5 * d @ A @ d, A @ d

    x, hist = AL.lbfgs(fg, np.zeros(n), steps=50)
    assert hist[-1].evaluations <= 50
    assert np.linalg.norm(x - xs) <= 1e-6 * np.linalg.norm(xs)


def test_preconditioned_steps_reduce_the_fp64_loss(sample, align_ref):
    b, args = sample
    st, sz = 0.01, 0.002
    D = align_ref.gn_diag(*args, np.zeros((b.n_layers, 3)), st, sz)
    assert np.all(D[:8] > 0)  # layers 1-8 are in triplets of the sample

    def fg(a):
        l, g, _ = align_ref.loss_and_grad(*args, a, st, sz)
        return l, g

    a, hist = AL.align_layers(fg, RADII, steps=30, precond=D)
    assert hist[-1].evaluations <= 30
    assert hist[-1].loss < 0.5 * hist[0].loss
    # the final point is measured, and its gradient in the gauge is small
    l_end, _ = fg(a)
    assert l_end == pytest.approx(hist[-1].loss, rel=1e-12)
    assert hist[-1].grad_norm <= 1e-3 * hist[0].grad_norm
