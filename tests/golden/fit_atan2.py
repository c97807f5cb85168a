"""Fits the arctangent polynomials of sift_internal.cuh (test infrastructure).

    python tests/golden/fit_atan2.py          # prints the coefficients

Both are odd polynomials in a = min(|x|, |y|) / max(|x|, |y|) on [0, 1],
written as a * P(a^2):

  atan2_poly   atan(a),        P of degree 7, minimax in relative error
  atan2_bins   atan(a) * 4/pi, P of degree 4, minimax in absolute error
               (in units of 45-degree descriptor bins)

Method: Lawson's algorithm (iteratively reweighted least squares, whose
weights converge to the minimax solution, C. L. Lawson 1961) on 4001
Chebyshev points of [0, 1] in float64, then each coefficient rounded to the
nearest float32. Deterministic: the same coefficients on every host. The
device code evaluates P by Horner's rule with fused multiply-adds in f32.
"""
from __future__ import annotations

import numpy as np

N_POINTS = 4001
ITERATIONS = 400


def lawson(degree: int, relative: bool, scale: float) -> np.ndarray:
    """Coefficients c[0..degree] of P (c[0] the constant) minimising
    max |a P(a^2) - scale atan(a)| (divided by scale atan(a) if relative)."""
    k = np.arange(N_POINTS)
    a = 0.5 - 0.5 * np.cos(np.pi * (k + 0.5) / N_POINTS)  # Chebyshev points of [0, 1]
    f = scale * np.arctan(a)
    t = a * a
    A = a[:, None] * t[:, None] ** np.arange(degree + 1)[None, :]
    rel = np.where(f > 0, f, 1.0) if relative else np.ones_like(a)
    A, f = A / rel[:, None], f / rel
    w = np.full(N_POINTS, 1.0 / N_POINTS)
    c = None
    for _ in range(ITERATIONS):
        sw = np.sqrt(w)
        c, *_ = np.linalg.lstsq(A * sw[:, None], f * sw, rcond=None)
        e = np.abs(A @ c - f)
        w = w * e
        w /= w.sum()
    return c


def to_f32(c: np.ndarray) -> list[float]:
    return [float(np.float32(v)) for v in c]


def horner_f32(c32: list[float], a: np.ndarray) -> np.ndarray:
    """a * P(a^2) in float32 with one rounding per multiply-add (the device's
    fmaf), highest coefficient first."""
    a = a.astype(np.float32)
    t = (a * a).astype(np.float32)
    p = np.full_like(a, np.float32(c32[-1]))
    for coef in reversed(c32[:-1]):
        p = (p.astype(np.float64) * t.astype(np.float64) + np.float64(np.float32(coef))).astype(np.float32)
    return (p * a).astype(np.float32)


def coefficients() -> dict[str, list[float]]:
    return {"atan2_poly": to_f32(lawson(7, True, 1.0)),
            "atan2_bins": to_f32(lawson(4, False, 4.0 / np.pi))}


def max_errors(coefs: dict[str, list[float]]) -> dict[str, float]:
    a = np.linspace(0.0, 1.0, 1 << 20)
    ref = np.arctan(a)
    out = {}
    p = horner_f32(coefs["atan2_poly"], a).astype(np.float64)
    nz = ref > 0
    out["atan2_poly_rel"] = float(np.max(np.abs(p[nz] - ref[nz]) / ref[nz]))
    b = horner_f32(coefs["atan2_bins"], a).astype(np.float64)
    out["atan2_bins_abs_bins"] = float(np.max(np.abs(b - ref * 4.0 / np.pi)))
    return out


if __name__ == "__main__":
    c = coefficients()
    for name, v in c.items():
        print(name, "(constant term first):")
        for x in v:
            print(f"    {x:.17g}f")
    print(max_errors(c))
