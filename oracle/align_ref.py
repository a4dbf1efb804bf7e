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
      point of closest approach to the origin PCA = C d0 / |C|
      arc lengths s_i = 2 R asin(|P_i - PCA| / 2R)
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
    m = d0 / Cn
    Px, Py = Cx * m, Cy * m
    s, rho, sq = [], [], []
    for (Xi, Yi) in ((X1, Y1), (X2, Y2), (X3, Y3)):
        r_i = np.hypot(Xi - Px, Yi - Py)
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
                num=num, d0=d0, m=m, Px=Px, Py=Py, s=s, rho=rho, sq=sq, t=t, z0=z0, e=e,
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


def loss_and_grad(x, y, z, layer, h1, h2, h3, w, align, sigma_tip, sigma_z):
    """(loss, dL/dalign [L, 3], dL/d(x, y, z) [H, 3]) by the hand-written adjoint."""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    z = np.asarray(z, np.float64)
    align = np.asarray(align, np.float64)
    lay = np.asarray(layer, np.int64) - 1
    X, Y, Z = transform(x, y, z, layer, align)
    f = _forward(X, Y, Z, h1, h2, h3)
    w = np.asarray(w, np.float64)
    d0, R, Cn, m = f["d0"], f["R"], f["Cn"], f["m"]
    L = float(np.sum(w * ((d0 / sigma_tip) ** 2 + sum(ei * ei for ei in f["e"]) / sigma_z ** 2)))
    t = f["t"]
    gP = [[np.zeros_like(d0), np.zeros_like(d0)] for _ in range(3)]
    gZ = [np.zeros_like(d0) for _ in range(3)]
    # line fit: (z0, t) are least-squares optimal, so chi2 moves with Z_i and
    # s_i at fixed (z0, t)
    g_s = []
    for i in range(3):
        ge = w * 2.0 * f["e"][i] / sigma_z ** 2
        gZ[i] = gZ[i] + ge
        g_s.append(-t * ge)
    g_d0 = w * 2.0 * d0 / sigma_tip ** 2
    g_R = np.zeros_like(d0)
    gPx = np.zeros_like(d0)
    gPy = np.zeros_like(d0)
    for i in range(3):
        xi = np.minimum(f["rho"][i] / (2.0 * R), 1.0)
        ds_drho = 1.0 / f["sq"][i]
        ds_dR = 2.0 * np.arcsin(xi) - (f["rho"][i] / R) / f["sq"][i]
        g_rho = g_s[i] * ds_drho
        g_R = g_R + g_s[i] * ds_dR
        Xi, Yi = f["P"][i]
        dx, dy = Xi - f["Px"], Yi - f["Py"]
        gx, gy = g_rho * dx / f["rho"][i], g_rho * dy / f["rho"][i]
        gP[i][0] = gP[i][0] + gx
        gP[i][1] = gP[i][1] + gy
        gPx = gPx - gx
        gPy = gPy - gy
    # PCA = C m, m = d0 / Cn
    g_Cx = gPx * m
    g_Cy = gPy * m
    g_m = gPx * f["Cx"] + gPy * f["Cy"]
    g_d0 = g_d0 + g_m / Cn
    g_Cn = -g_m * d0 / Cn ** 2
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
    return L, g_align, g_hits


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
