"""FP64 CPU reference of the differentiable triplet fit and its adjoint.

TEST INFRASTRUCTURE ONLY: the tests and the benchmark's checks use it as the
checker of the sm_103a fit kernels; the product never imports it.

The reference (JuantAldea/trax) has no differentiable component.  The
per-triplet forward follows the geometry of its fitters -- the circle
through three points (TrackletCircleFitter.h:32-97, FastCircle.h:41-118)
and a straight line in the arc-length/z plane (FastLine.h:15-42) -- and
adds the alignment model:

  a hit (x, y, z) on layer l, reconstructed with nominal geometry, is
  corrected by the layer's shifts (dr, dz, dphi):
      r = |(x, y)|,  f = (r + dr) / r
      X = f (x cos dphi - y sin dphi),  Y = f (x sin dphi + y cos dphi),  Z = z + dz

  per triplet (P1, P2, P3 corrected):
      circle through the three points: centre C, radius R, curvature 1/R
      transverse impact parameter d0 = |C| - R (signed)
      arc lengths from the beam line s_i = 2 R asin(r_i / 2R), r_i = |P_i|
      (exact for a helix through the beam line; the part of a nonzero d0 that
      is linear in s is absorbed by the line fit)
      least-squares line Z = z0 + cot(theta) s through the three (s_i, Z_i)
      chi2 = (d0 / sigma_tip)^2 + sum_i e_i^2 / sigma_z^2,  e_i the line residuals

  loss = sum over the selected triplets of w_t chi2_t.

`loss_and_grad` is a hand-written reverse pass in FP64 (vectorised over
triplets); `loss` alone serves the central finite differences.
"""
from __future__ import annotations

import numpy as np


def transform(x, y, z, layer, align):
    """Corrected hit coordinates; align is [L, 3] = (dr, dz, dphi), layer 1-based."""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    z = np.asarray(z, np.float64)
    a = np.asarray(align, np.float64)[np.asarray(layer, np.int64) - 1]
    dr, dz, dp = a[:, 0], a[:, 1], a[:, 2]
    r = np.hypot(x, y)
    f = (r + dr) / r
    c, s = np.cos(dp), np.sin(dp)
    return f * (x * c - y * s), f * (x * s + y * c), z + dz


def _forward(X, Y, Z, h1, h2, h3):
    X1, Y1, Z1 = X[h1], Y[h1], Z[h1]
    X2, Y2, Z2 = X[h2], Y[h2], Z[h2]
    X3, Y3, Z3 = X[h3], Y[h3], Z[h3]
    u2, v2, u3, v3 = X2 - X1, Y2 - Y1, X3 - X1, Y3 - Y1
    q2, q3 = u2 * u2 + v2 * v2, u3 * u3 + v3 * v3
    D = 2.0 * (u2 * v3 - u3 * v2)
    a = (v3 * q2 - v2 * q3) / D
    b = (u2 * q3 - u3 * q2) / D
    R = np.sqrt(a * a + b * b)
    Cx, Cy = X1 + a, Y1 + b
    Cn = np.sqrt(Cx * Cx + Cy * Cy)
    num = X1 * X1 + Y1 * Y1 + 2.0 * (X1 * a + Y1 * b)
    d0 = num / (Cn + R)
    s, rho, sq = [], [], []
    for (Xi, Yi) in ((X1, Y1), (X2, Y2), (X3, Y3)):
        r_i = np.hypot(Xi, Yi)
        xi = np.minimum(r_i / (2.0 * R), 1.0)
        s.append(2.0 * R * np.arcsin(xi))
        rho.append(r_i)
        sq.append(np.sqrt(np.maximum(1.0 - xi * xi, 1e-300)))
    Zs = (Z1, Z2, Z3)
    sb = (s[0] + s[1] + s[2]) / 3.0
    zb = (Z1 + Z2 + Z3) / 3.0
    Sss = sum((si - sb) ** 2 for si in s)
    Ssz = sum((si - sb) * (zi - zb) for si, zi in zip(s, Zs))
    t = Ssz / Sss
    z0 = zb - t * sb
    e = [zi - z0 - t * si for si, zi in zip(s, Zs)]
    return dict(u2=u2, v2=v2, u3=u3, v3=v3, q2=q2, q3=q3, D=D, a=a, b=b, R=R, Cx=Cx, Cy=Cy, Cn=Cn,
                num=num, d0=d0, s=s, rho=rho, sq=sq, t=t, z0=z0, e=e,
                P=((X1, Y1), (X2, Y2), (X3, Y3)))


def triplet_params(x, y, z, layer, h1, h2, h3, align):
    """Per-triplet (curvature, d0, z0, cot theta) in FP64."""
    X, Y, Z = transform(x, y, z, layer, align)
    f = _forward(X, Y, Z, h1, h2, h3)
    return np.stack([1.0 / f["R"], f["d0"], f["z0"], f["t"]], axis=1)


def triplet_chi2(x, y, z, layer, h1, h2, h3, align, sigma_tip, sigma_z):
    X, Y, Z = transform(x, y, z, layer, align)
    f = _forward(X, Y, Z, h1, h2, h3)
    return (f["d0"] / sigma_tip) ** 2 + sum(ei * ei for ei in f["e"]) / sigma_z ** 2


def loss(x, y, z, layer, h1, h2, h3, w, align, sigma_tip, sigma_z) -> float:
    return float(np.sum(w * triplet_chi2(x, y, z, layer, h1, h2, h3, align, sigma_tip, sigma_z)))


def _adjoint(f, seed_d0, seed_e):
    """Reverse pass from d(.)/d d0 = seed_d0 and d(.)/d e_i = seed_e[i] (line
    parameters held at their least-squares optimum) to the corrected hits:
    returns ([(gX, gY)] * 3, [gZ] * 3) per triplet slot."""
    d0, R, Cn = f["d0"], f["R"], f["Cn"]
    t = f["t"]
    gP = [[np.zeros_like(d0), np.zeros_like(d0)] for _ in range(3)]
    gZ = [np.zeros_like(d0) for _ in range(3)]
    # line fit: (z0, t) are least-squares optimal, so chi2 moves with Z_i and
    # s_i at fixed (z0, t)
    g_s = []
    for i in range(3):
        gZ[i] = gZ[i] + seed_e[i]
        g_s.append(-t * seed_e[i])
    g_d0 = seed_d0 + 0.0 * d0
    g_R = np.zeros_like(d0)
    for i in range(3):
        xi = np.minimum(f["rho"][i] / (2.0 * R), 1.0)
        ds_dr = 1.0 / f["sq"][i]
        ds_dR = 2.0 * np.arcsin(xi) - (f["rho"][i] / R) / f["sq"][i]
        g_r = g_s[i] * ds_dr
        g_R = g_R + g_s[i] * ds_dR
        Xi, Yi = f["P"][i]
        gP[i][0] = gP[i][0] + g_r * Xi / f["rho"][i]
        gP[i][1] = gP[i][1] + g_r * Yi / f["rho"][i]
    g_Cx = np.zeros_like(d0)
    g_Cy = np.zeros_like(d0)
    g_Cn = np.zeros_like(d0)
    # d0 = num / (Cn + R)
    g_num = g_d0 / (Cn + R)
    g_Cn = g_Cn - g_d0 * d0 / (Cn + R)
    g_R = g_R - g_d0 * d0 / (Cn + R)
    X1, Y1 = f["P"][0]
    a, b = f["a"], f["b"]
    # num = X1^2 + Y1^2 + 2 (X1 a + Y1 b)
    gP[0][0] = gP[0][0] + g_num * (2.0 * X1 + 2.0 * a)
    gP[0][1] = gP[0][1] + g_num * (2.0 * Y1 + 2.0 * b)
    g_a = g_num * 2.0 * X1
    g_b = g_num * 2.0 * Y1
    # Cn = |C|, C = P1 + (a, b)
    g_Cx = g_Cx + g_Cn * f["Cx"] / Cn
    g_Cy = g_Cy + g_Cn * f["Cy"] / Cn
    gP[0][0] = gP[0][0] + g_Cx
    gP[0][1] = gP[0][1] + g_Cy
    g_a = g_a + g_Cx
    g_b = g_b + g_Cy
    # R = |(a, b)|
    g_a = g_a + g_R * a / R
    g_b = g_b + g_R * b / R
    # a = (v3 q2 - v2 q3) / D, b = (u2 q3 - u3 q2) / D
    D, q2, q3 = f["D"], f["q2"], f["q3"]
    u2, v2, u3, v3 = f["u2"], f["v2"], f["u3"], f["v3"]
    g_D = -(g_a * a + g_b * b) / D
    g_v3 = g_a * q2 / D
    g_q2 = g_a * v3 / D - g_b * u3 / D
    g_v2 = -g_a * q3 / D
    g_q3 = -g_a * v2 / D + g_b * u2 / D
    g_u2 = g_b * q3 / D
    g_u3 = -g_b * q2 / D
    # D = 2 (u2 v3 - u3 v2)
    g_u2 = g_u2 + 2.0 * g_D * v3
    g_v3 = g_v3 + 2.0 * g_D * u2
    g_u3 = g_u3 - 2.0 * g_D * v2
    g_v2 = g_v2 - 2.0 * g_D * u3
    g_u2 = g_u2 + 2.0 * u2 * g_q2
    g_v2 = g_v2 + 2.0 * v2 * g_q2
    g_u3 = g_u3 + 2.0 * u3 * g_q3
    g_v3 = g_v3 + 2.0 * v3 * g_q3
    gP[1][0] = gP[1][0] + g_u2
    gP[1][1] = gP[1][1] + g_v2
    gP[2][0] = gP[2][0] + g_u3
    gP[2][1] = gP[2][1] + g_v3
    gP[0][0] = gP[0][0] - g_u2 - g_u3
    gP[0][1] = gP[0][1] - g_v2 - g_v3
    return gP, gZ


def loss_and_grad(x, y, z, layer, h1, h2, h3, w, align, sigma_tip, sigma_z, squares=False):
    """(loss, dL/dalign [L, 3], dL/d(x, y, z) [H, 3]) by the hand-written adjoint;
    with `squares` also the sum over triplets of each triplet's dchi2/dalign
    squared [L, 3]."""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    z = np.asarray(z, np.float64)
    align = np.asarray(align, np.float64)
    lay = np.asarray(layer, np.int64) - 1
    X, Y, Z = transform(x, y, z, layer, align)
    f = _forward(X, Y, Z, h1, h2, h3)
    w = np.asarray(w, np.float64)
    d0 = f["d0"]
    L = float(np.sum(w * ((d0 / sigma_tip) ** 2 + sum(ei * ei for ei in f["e"]) / sigma_z ** 2)))
    gP, gZ = _adjoint(f, w * 2.0 * d0 / sigma_tip ** 2, [w * 2.0 * ei / sigma_z ** 2 for ei in f["e"]])
    # corrected-hit gradients -> alignment and raw-hit gradients
    H = x.shape[0]
    gX = np.zeros(H)
    gY = np.zeros(H)
    gZh = np.zeros(H)
    for i, h in enumerate((h1, h2, h3)):
        np.add.at(gX, h, gP[i][0])
        np.add.at(gY, h, gP[i][1])
        np.add.at(gZh, h, gZ[i])
    a_h = align[lay]
    dr, dp = a_h[:, 0], a_h[:, 2]
    r = np.hypot(x, y)
    fh = (r + dr) / r
    c, s = np.cos(dp), np.sin(dp)
    xr, yr = x * c - y * s, x * s + y * c
    dX_ddr, dY_ddr = xr / r, yr / r
    dX_ddp, dY_ddp = -fh * yr, fh * xr
    g_align = np.zeros_like(align)
    np.add.at(g_align[:, 0], lay, gX * dX_ddr + gY * dY_ddr)
    np.add.at(g_align[:, 1], lay, gZh)
    np.add.at(g_align[:, 2], lay, gX * dX_ddp + gY * dY_ddp)
    df_dx = -dr * x / r ** 3
    df_dy = -dr * y / r ** 3
    g_hits = np.zeros((H, 3))
    g_hits[:, 0] = gX * (fh * c + xr * df_dx) + gY * (fh * s + yr * df_dx)
    g_hits[:, 1] = gX * (-fh * s + xr * df_dy) + gY * (fh * c + yr * df_dy)
    g_hits[:, 2] = gZh
    if not squares:
        return L, g_align, g_hits
    g_sq = np.zeros_like(align)
    for i, h in enumerate((h1, h2, h3)):
        li = lay[h]
        per = np.stack([gP[i][0] * dX_ddr[h] + gP[i][1] * dY_ddr[h], gZ[i],
                        gP[i][0] * dX_ddp[h] + gP[i][1] * dY_ddp[h]], axis=1)
        for k in range(3):
            np.add.at(g_sq[:, k], li, per[:, k] ** 2)
    return L, g_align, g_hits, g_sq


def gn_diag(x, y, z, layer, h1, h2, h3, w, align, sigma_tip, sigma_z):
    """Approximate Gauss-Newton diagonal [L, 3], a preconditioner: sum over
    triplets of (d d0/d align)^2 / sigma_tip^2 for dr and dphi, of the z
    residuals' projector diagonal P_kk = (2/3 - ds_k^2 / S_ss) / sigma_z^2 for
    dz, and of cot(theta)^2 P_kk for dr (a radial shift slides the hit along
    its arc; the z residuals' dependence on dphi is left out)."""
    X, Y, Z = transform(x, y, z, layer, align)
    f = _forward(X, Y, Z, h1, h2, h3)
    ones = np.ones_like(f["d0"])
    zero = np.zeros_like(f["d0"])
    gP, _ = _adjoint(f, ones, [zero, zero, zero])
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    lay = np.asarray(layer, np.int64) - 1
    a_h = np.asarray(align, np.float64)[lay]
    dr, dp = a_h[:, 0], a_h[:, 2]
    r = np.hypot(x, y)
    fh = (r + dr) / r
    c, s_ = np.cos(dp), np.sin(dp)
    xr, yr = x * c - y * s_, x * s_ + y * c
    sb = (f["s"][0] + f["s"][1] + f["s"][2]) / 3.0
    Sss = sum((si - sb) ** 2 for si in f["s"])
    out = np.zeros((np.asarray(align).shape[0], 3))
    wt = np.asarray(w, np.float64) / np.asarray(sigma_tip, np.float64) ** 2
    for i, h in enumerate((h1, h2, h3)):
        ddr = (gP[i][0] * xr[h] + gP[i][1] * yr[h]) / r[h]
        ddp = fh[h] * (gP[i][1] * xr[h] - gP[i][0] * yr[h])
        np.add.at(out[:, 0], lay[h], wt * ddr ** 2)
        np.add.at(out[:, 2], lay[h], wt * ddp ** 2)
        proj = np.asarray(w, np.float64) * (2.0 / 3.0 - (f["s"][i] - sb) ** 2 / Sss) / sigma_z ** 2
        np.add.at(out[:, 1], lay[h], proj)
        # a radial shift moves the hit along its arc: ds = dr / sq, de ~ -cot(theta) ds
        np.add.at(out[:, 0], lay[h], proj * (f["t"] / f["sq"][i]) ** 2)
    return out


def fd_grad_align(x, y, z, layer, h1, h2, h3, w, align, sigma_tip, sigma_z, h=1e-6):
    """Central finite differences of the FP64 loss over the alignment parameters."""
    align = np.asarray(align, np.float64)
    g = np.zeros_like(align)
    for k in range(align.shape[0]):
        for j in range(3):
            ap = align.copy()
            am = align.copy()
            ap[k, j] += h
            am[k, j] -= h
            g[k, j] = (loss(x, y, z, layer, h1, h2, h3, w, ap, sigma_tip, sigma_z)
                       - loss(x, y, z, layer, h1, h2, h3, w, am, sigma_tip, sigma_z)) / (2.0 * h)
    return g
