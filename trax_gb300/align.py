"""Layer alignment by gradient steps on the triplet-fit chi2.

The loss and its gradient come from the C ABI (trax_fit_forward /
trax_fit_backward, an FP32 fit with a hand-written adjoint kernel and FP64
sums); this module holds the host-side optimiser.  No counterpart in the
reference.

Parameters are the per-layer shifts (dr, dz, dphi).  Six deformations leave
the chi2 of triplets from the beam line unchanged, or nearly so, and no
amount of data fixes them:

  * a common rotation (dphi the same on all layers) and a common z shift;
  * a z shear (dz proportional to r), which only changes every cot(theta);
  * a phi shear (dphi proportional to r), which only changes every curvature;
  * a radial scaling (dr proportional to r) and a common radial shift,
    which move three-point circles through the beam line into circles that
    still pass it to within far less than the hit resolution.

The optimiser works in the complement of these modes (the gauge), in units
of 10 um (dr, dz) and 10 urad (dphi), with limited-memory BFGS: on this
nearly quadratic loss it behaves like conjugate gradients and settles in
well under 50 gradient evaluations.  Recovered shifts are compared with the
truth in the same complement.
"""
from __future__ import annotations

import dataclasses
from typing import Callable, List, Optional, Tuple

import numpy as np

UNITS = np.array([1e-3, 1e-3, 1e-5])  # scaled unit of (dr [cm], dz [cm], dphi [rad])


def weak_modes(radii: np.ndarray) -> np.ndarray:
    """The six chi2-invariant deformations as columns of a [3 L, 6] array."""
    radii = np.asarray(radii, dtype=np.float64)
    L = radii.size
    cols = []
    for comp, prof in ((2, np.ones(L)), (1, np.ones(L)), (1, radii), (2, radii), (0, radii), (0, np.ones(L))):
        v = np.zeros((L, 3))
        v[:, comp] = prof
        cols.append(v.ravel())
    return np.array(cols).T


class Gauge:
    """Scaled coordinates z = align / UNITS and the projector onto the complement
    of the weak modes (orthogonal in scaled coordinates)."""

    def __init__(self, radii: np.ndarray):
        self.L = int(np.asarray(radii).size)
        self.scale = np.tile(UNITS, self.L)
        M = weak_modes(radii) / self.scale[:, None]
        q, _ = np.linalg.qr(M)
        self.Q = q
        self.radii = np.asarray(radii, dtype=np.float64)

    def project(self, z: np.ndarray) -> np.ndarray:
        return z - self.Q @ (self.Q.T @ z)

    def to_align(self, z: np.ndarray) -> np.ndarray:
        return (z * self.scale).reshape(self.L, 3)

    def to_scaled(self, align: np.ndarray) -> np.ndarray:
        return np.asarray(align, dtype=np.float64).ravel() / self.scale

    def residual_um(self, align: np.ndarray, truth: np.ndarray) -> np.ndarray:
        """(align - truth) in the gauge, as displacements in um ([L, 3]; dphi times the radius)."""
        d = self.project(self.to_scaled(align) - self.to_scaled(truth))
        r = self.to_align(d) * 1e4
        r[:, 2] *= self.radii
        return r


@dataclasses.dataclass
class Step:
    loss: float
    grad_norm: float
    evaluations: int


def lbfgs(fg: Callable[[np.ndarray], Tuple[float, np.ndarray]], z0: np.ndarray, steps: int = 50,
          memory: int = 64, project: Optional[Callable[[np.ndarray], np.ndarray]] = None,
          first_step: float = 1.0, refresh: int = 8, gtol: float = 1e-10, h0: Optional[float] = None,
          max_extrapolation: float = 50.0) -> Tuple[np.ndarray, List[Step]]:
    """Minimise fg (loss, gradient) with at most `steps` gradient evaluations.

    Limited-memory BFGS with one gradient evaluation per iteration: the
    quasi-Newton direction d is tried with the unit step, the pair
    (d, g(z + d) - g(z)) updates the inverse-Hessian model, and the iterate
    moves to the zero of the directional derivative interpolated linearly
    between z and z + d, with its gradient interpolated the same way.  On a
    quadratic that line search is exact and the directions are conjugate, so
    an n-dimensional quadratic is solved in about n evaluations; on a nearly
    quadratic loss the interpolated gradient is re-measured every `refresh`
    iterations (and at the end).  `project` keeps iterates in a subspace.
    The first direction is -g / h0 when a curvature scale h0 is given (else a
    step of length `first_step`); interpolated step lengths beyond
    `max_extrapolation` times the trial step are not trusted (the trial point
    is kept), and trial points where the loss is not finite are shortened."""
    P = project or (lambda v: v)
    z = P(np.asarray(z0, dtype=np.float64).copy())
    f, g = fg(z)
    g = P(g)
    evals = 1
    hist = [Step(f, float(np.linalg.norm(g)), evals)]
    S, Y = [], []
    since = 0
    g_scale = max(np.linalg.norm(g), 1e-300)
    while evals < steps - 1:
        if np.linalg.norm(g) <= gtol * g_scale:
            break
        q = g.copy()
        alphas = []
        for s_, y_ in reversed(list(zip(S, Y))):
            rho = 1.0 / float(y_ @ s_)
            a = rho * float(s_ @ q)
            alphas.append((rho, a))
            q = q - a * y_
        if S:
            gamma = float(S[-1] @ Y[-1]) / float(Y[-1] @ Y[-1])
        else:
            gamma = 1.0 / h0 if h0 else first_step / max(np.linalg.norm(g), 1e-300)
        r = gamma * q
        for (s_, y_), (rho, a) in zip(zip(S, Y), reversed(alphas)):
            r = r + (a - rho * float(y_ @ r)) * s_
        d = -P(r)
        slope = float(g @ d)
        if slope >= 0:  # lost descent: restart from the gradient
            S, Y = [], []
            d = -g * (first_step / g_scale)
            slope = float(g @ d)
        zt = P(z + d)
        ft, gt = fg(zt)
        gt = P(gt)
        evals += 1
        while not (np.isfinite(ft) and np.all(np.isfinite(gt))) and evals < steps - 1:
            d = 0.25 * d  # outside the region where the loss is defined: shorten
            slope = float(g @ d)
            zt = P(z + d)
            ft, gt = fg(zt)
            gt = P(gt)
            evals += 1
        if not (np.isfinite(ft) and np.all(np.isfinite(gt))):
            break
        y_ = gt - g
        curv = float(y_ @ d)
        if curv > 1e-12 * abs(slope) and -slope / curv <= max_extrapolation:
            S.append(d)
            Y.append(y_)
            if len(S) > memory:
                S.pop(0)
                Y.pop(0)
            t = -slope / curv
            z = P(z + t * d)
            g = P(g + t * y_)
            f = f + t * slope + 0.5 * t * t * curv
            since += 1
            if since >= refresh and evals < steps - 1:
                f, g = fg(z)
                g = P(g)
                evals += 1
                since = 0
        else:  # no usable curvature along d: take the trial point as it is
            if curv > 1e-12 * abs(slope):
                S.append(d)
                Y.append(y_)
                if len(S) > memory:
                    S.pop(0)
                    Y.pop(0)
            z, f, g = zt, ft, gt
            since = 0
        hist.append(Step(f, float(np.linalg.norm(g)), evals))
    if since:  # measure the final point
        f, g = fg(z)
        g = P(g)
        evals += 1
        hist.append(Step(f, float(np.linalg.norm(g)), evals))
    return z, hist


def align_layers(fg_align: Callable[[np.ndarray], Tuple[float, np.ndarray]], radii: np.ndarray,
                 steps: int = 50, precond: Optional[np.ndarray] = None, start: Optional[np.ndarray] = None):
    """Recover per-layer shifts from a (loss, d loss / d align) function of
    align [L, 3]; returns (align [L, 3], history).

    `precond` [L, 3] is a positive diagonal curvature estimate (the
    Gauss-Newton diagonal of trax_fit_backward); parameters
    are scaled by its inverse square root, which evens out the curvature of
    radial, longitudinal and azimuthal shifts on inner and outer layers.  The
    gauge (weak modes) is removed in those scaled coordinates."""
    radii = np.asarray(radii, dtype=np.float64)
    L = radii.size
    if precond is None:
        sc = np.tile(UNITS, L)
    else:
        d = np.asarray(precond, dtype=np.float64).ravel()
        sc = np.where(d > 0, 1.0 / np.sqrt(np.where(d > 0, d, 1.0)), np.tile(UNITS, L))
    q, _ = np.linalg.qr(weak_modes(radii) / sc[:, None])

    def project(v):
        return v - q @ (q.T @ v)

    def fg(zv):
        f, g = fg_align((zv * sc).reshape(L, 3))
        return f, np.asarray(g, dtype=np.float64).ravel() * sc

    z0 = np.zeros(3 * L) if start is None else np.asarray(start, dtype=np.float64).ravel() / sc
    # with the Gauss-Newton scaling the chi2 Hessian is about 2 on the diagonal
    z, hist = lbfgs(fg, z0, steps=steps, project=project, h0=2.0 if precond is not None else None)
    return (z * sc).reshape(L, 3), hist


def align_context(ctx, radii: np.ndarray, steps: int = 50):
    """Align with a prepared context (trax_fit_prepare): the first gradient
    evaluation, at zero shifts, also gives the preconditioner; `steps` counts
    every gradient evaluation."""
    L = np.asarray(radii).size
    zero = np.zeros((L, 3))
    f0, g0, _, g2 = ctx.fit_backward(zero, squares=True)
    first = [(f0, g0)]

    def fg(align):
        if first and not np.any(align):
            return first.pop()
        chi2, g, _ = ctx.fit_backward(align)
        return chi2, g

    return align_layers(fg, radii, steps=steps, precond=g2)


def align_reseeding(ctx, radii: np.ndarray, steps: int = 50, rounds: int = 2, truth_only: bool = True,
                    run_linking: bool = False):
    """Alignment in rounds: fit rows frozen from the accepted triplets, gradient
    steps, then the uploaded hits corrected by the shifts found
    (trax_apply_alignment) and the seeding rerun, so that the next round's
    rows come from cuts applied to the corrected geometry.  The cut decisions
    are frozen inside each round; `steps` gradient evaluations in total are
    split evenly over the rounds.  The context must hold a seeded batch.
    Returns (total shifts [L, 3], list of per-round histories)."""
    radii = np.asarray(radii, dtype=np.float64)
    total = np.zeros((radii.size, 3))
    per = [steps // rounds + (1 if k < steps % rounds else 0) for k in range(rounds)]
    hists = []
    for k in range(rounds):
        if k > 0:
            ctx.apply_alignment(a)
            ctx.seed_batch(use_graph=True, run_linking=run_linking)
        ctx.fit_prepare(truth_only=truth_only)
        a, hist = align_context(ctx, radii, steps=per[k])
        total += a
        hists.append(hist)
    return total, hists
