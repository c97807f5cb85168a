"""Exactness of the device-side arithmetic shortcuts, checked on the CPU in
exact rational arithmetic (no GPU needed)."""
from fractions import Fraction

import numpy as np


def round_f32(x: Fraction) -> Fraction:
    """x rounded to the nearest f32 (ties to even), for normal-range x."""
    if x == 0:
        return Fraction(0)
    sign = -1 if x < 0 else 1
    x = abs(x)
    e = x.numerator.bit_length() - x.denominator.bit_length()
    while Fraction(2) ** e > x:
        e -= 1
    while Fraction(2) ** (e + 1) <= x:
        e += 1
    ulp = Fraction(2) ** (e - 23)
    q = x / ulp
    n = q.numerator // q.denominator
    rem = q - n
    if rem > Fraction(1, 2) or (rem == Fraction(1, 2) and n % 2 == 1):
        n += 1
    return sign * n * ulp


def test_div255_is_the_ieee_division():
    """div255 (sift_internal.cuh): q = v * fl(1/255), then
    fma(fma(-q, 255, v), fl(1/255), q) equals fl(v / 255) for every u8 v."""
    r = round_f32(Fraction(1, 255))
    assert r == Fraction(int(np.float32(0.003921568859368563).view(np.uint32)) & 0x7FFFFF | 0x800000, 2 ** 31)
    for v in range(256):
        q = round_f32(v * r)
        e = round_f32(-q * 255 + v)
        assert round_f32(e * r + q) == round_f32(Fraction(v, 255)), v


def test_arctangent_coefficients_are_the_fits():
    """The coefficients in sift_internal.cuh are what tests/golden/fit_atan2.py
    makes, and their f32 errors on [0, 1] are the ones the comments state."""
    import re
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    sys.path.insert(0, str(root / "tests" / "golden"))
    import fit_atan2
    src = (root / "sift_wgpu_gb300" / "csrc" / "sift_internal.cuh").read_text()
    c = fit_atan2.coefficients()
    for name in ("atan2_poly", "atan2_bins"):
        body = src[src.index(f"float {name}(float y, float x)"):]
        body = body[:body.index("float r = p * a;")]
        got = [float(v) for v in re.findall(r"(-?\d+\.\d+(?:e-?\d+)?)f", body.split("float p = ", 1)[1])]
        assert got == c[name][::-1], name
    e = fit_atan2.max_errors(c)
    assert e["atan2_poly_rel"] < 3.0e-7 and e["atan2_bins_abs_bins"] < 1.5e-5, e
