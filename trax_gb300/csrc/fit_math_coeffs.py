"""Fit the polynomial kernels of trax_math.h and write trax_math_coeffs.h.

The single-precision transcendental functions shared by the CPU oracle and
the sm_103a kernels (atan2, atan, acos, asinh, log) are built from textbook
range reductions (Cephes-style three-interval reduction for atan, the
half-angle identity acos(x) = 2 asin(sqrt((1-x)/2)), the atanh series for
log(m) with m in [sqrt(1/2), sqrt(2))) and one odd polynomial per function:

    f(t) = t + t^3 * P(t^2)

This script fits each P by weighted least squares on Chebyshev nodes followed
by Lawson iterations (which drive the weighted least-squares solution towards
the minimax one), weighting by the effect on the RELATIVE error of f.  The
coefficients are then rounded to float32 and the float32 Horner evaluation
(no fused multiply-add, round-to-nearest) is checked against float64 over a
dense grid.  Nothing here is taken from a vendor math library: the
coefficients are whatever this fit produces.

Run:  python trax_gb300/csrc/fit_math_coeffs.py   (rewrites trax_math_coeffs.h)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _target(name: str, t: np.ndarray) -> np.ndarray:
    """(f(t) - t) / t^3 for the function `name`, in float64."""
    if name == "atan":
        f = np.arctan(t)
    elif name == "asin":
        f = np.arcsin(t)
    elif name == "atanh":
        f = np.arctanh(t)
    elif name == "asinh":
        f = np.arcsinh(t)
    else:
        raise ValueError(name)
    return (f - t) / (t * t * t)


def fit(name: str, tmax: float, degree: int, lawson_iters: int = 200):
    """Return float64 coefficients c[0..degree] of P(u) = sum c_k u^k."""
    n = 4000
    k = np.arange(n)
    # Chebyshev nodes in u = t^2 over (0, tmax^2]
    umax = tmax * tmax
    u = 0.5 * umax * (1.0 - np.cos(np.pi * (k + 0.5) / n))
    t = np.sqrt(u)
    y = _target(name, t)
    # relative error of f = t (1 + u P) caused by an error dP is u dP / (1 + u P)
    w_rel = u / np.abs(1.0 + u * y)
    A = np.vander(u, degree + 1, increasing=True)
    lw = np.ones_like(u) / n
    c = None
    for _ in range(lawson_iters):
        W = np.sqrt(lw) * w_rel
        c, *_ = np.linalg.lstsq(A * W[:, None], y * W, rcond=None)
        err = np.abs((A @ c - y) * w_rel)
        lw = lw * err
        s = lw.sum()
        if s == 0.0:
            break
        lw = lw / s
    return c


def horner32(c32: np.ndarray, u32: np.ndarray) -> np.ndarray:
    """Float32 Horner evaluation, one rounding per multiply and per add."""
    p = np.full_like(u32, c32[-1])
    for ck in c32[-2::-1]:
        p = np.float32(p * u32)
        p = np.float32(p + ck)
    return p


def check(name: str, c32: np.ndarray, tmax: float) -> float:
    """Max relative error (in units of 2^-24) of the float32 kernel t + t^3 P."""
    t = np.linspace(np.float32(1e-4), np.float32(tmax), 400001, dtype=np.float32)
    u = np.float32(t * t)
    p = horner32(c32, u)
    t3 = np.float32(np.float32(t * u))
    f32 = np.float32(t + np.float32(t3 * p))
    ref = {"atan": np.arctan, "asin": np.arcsin, "atanh": np.arctanh,
           "asinh": np.arcsinh}[name](t.astype(np.float64))
    rel = np.abs(f32.astype(np.float64) - ref) / np.abs(ref)
    return float(rel.max() / 2.0 ** -24)


KERNELS = [
    # name, tmax, degree
    ("atan", float(np.tan(np.pi / 8)), 6),
    ("asin", 0.5, 6),
    ("atanh", float((np.sqrt(2.0) - 1.0) / (np.sqrt(2.0) + 1.0)), 4),
    ("asinh", 1.0, 12),
]


def main(out_path: str | None = None) -> int:
    out_path = out_path or os.path.join(HERE, "trax_math_coeffs.h")
    lines = [
        "// Generated by fit_math_coeffs.py -- polynomial kernels of trax_math.h.",
        "// f(t) = t + t^3 * P(t^2),  P(u) = C0 + C1 u + ... (Horner, float32).",
        "// Weighted least squares + Lawson iterations on Chebyshev nodes; see the",
        "// script for the fitting method.  Max relative error of the float32 kernel",
        "// over its interval is given in units of 2^-24 beside each table.",
        "#pragma once",
        "",
    ]
    for name, tmax, deg in KERNELS:
        c = fit(name, tmax, deg)
        c32 = c.astype(np.float32)
        err = check(name, c32, tmax)
        print(f"{name:6s} tmax={tmax:.6f} degree={deg} max rel err = {err:.3f} x 2^-24")
        lines.append(f"// {name}: t in [0, {tmax:.9g}], max rel err {err:.2f} x 2^-24")
        lines.append(f"#define TRAX_{name.upper()}_NCOEF {deg + 1}")
        vals = ", ".join(f"{float(v):.9e}f" for v in c32)
        lines.append(f"#define TRAX_{name.upper()}_COEFS {{ {vals} }}")
        lines.append("")
    with open(out_path, "w") as f:
        f.write("\n".join(lines))
    print("wrote", out_path)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1] if len(sys.argv) > 1 else None))
