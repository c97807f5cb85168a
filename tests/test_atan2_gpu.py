"""The engine's arctangent polynomials against CUDA's atan2f (GPU).

atan2_poly (and its f32x2 pair form atan2_poly2, which must give the same
values) decides orientation bins away from bin edges (within 1e-4 bin of an
edge the exact atan2f path decides), atan2_bins and its pair form
atan2_bins2 place descriptor samples in their 45-degree bins (linearly
interpolated). Both are evaluated on the
device by tests/atan2_probe.cu over a dense grid of directions and
magnitudes, the exact axes, the 36 orientation-bin edges and the 8
descriptor-bin edges, and quantised gradients (differences of v / 255)."""
import ctypes as C
import math
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = Path(__file__).resolve().parent


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out = tmp_path_factory.mktemp("atan2") / "libatan2probe.so"
    subprocess.run([nvcc, "-gencode=arch=compute_103a,code=sm_103a", "-O3", "--fmad=false", "-std=c++17",
                    "-I", str(HERE.parent / "include"), "-Xcompiler", "-fPIC", "-shared", "-o", str(out),
                    str(HERE / "atan2_probe.cu")], check=True)
    L = C.CDLL(str(out))
    L.atan2_probe.argtypes = [C.c_void_p, C.c_void_p, C.c_int] + [C.c_void_p] * 5
    return L


def inputs():
    f = np.float32
    ang = np.linspace(-math.pi, math.pi, 200001)
    mags = np.array([1e-3, 1 / 255, 0.05, 0.5, 1.0, 3.0])
    y = (np.sin(ang)[:, None] * mags[None, :]).ravel()
    x = (np.cos(ang)[:, None] * mags[None, :]).ravel()
    edges = np.concatenate([np.arange(36) * (2 * math.pi / 36), np.arange(8) * (math.pi / 4)])
    eps = np.array([0.0, 1e-7, -1e-7, 1e-6, -1e-6, 1e-5, -1e-5])
    e = (edges[:, None] + eps[None, :]).ravel()
    y = np.concatenate([y, np.sin(e), [0.0, 0.0, 0.0, 1.0, -1.0, 0.25]])
    x = np.concatenate([x, np.cos(e), [0.0, 1.0, -1.0, 0.0, 0.0, 0.0]])
    # quantised gradients: (a - b) / 255 in f32 for level values a, b
    q = (np.arange(-40, 41, dtype=f) / f(255.0)).astype(f)
    qy, qx = np.meshgrid(q, q)
    y = np.concatenate([y, qy.ravel()])
    x = np.concatenate([x, qx.ravel()])
    return np.ascontiguousarray(y, f), np.ascontiguousarray(x, f)


def test_polynomials_against_atan2f(probe):
    y, x = inputs()
    n = len(y)
    poly, bins, bins2, poly2, ref = (np.empty(n, np.float32) for _ in range(5))
    assert probe.atan2_probe(y.ctypes.data, x.ctypes.data, n, poly.ctypes.data, bins.ctypes.data, bins2.ctypes.data,
                             poly2.ctypes.data, ref.ctypes.data) == 0
    # the orientation's pair form gives atan2_poly's values bit for bit
    assert poly2.tobytes() == poly.tobytes()
    ref64 = ref.astype(np.float64)
    # atan2_poly: within 4 ulp of atan2f's angle (or 1e-12 rad near 0)
    err = np.abs(poly.astype(np.float64) - ref64)
    tol = np.maximum(4 * np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64), 1e-12)
    bad = err > tol
    assert not bad.any(), (int(bad.sum()), float(err[bad].max()), y[bad][:3], x[bad][:3])
    # as an orientation bin position (x 36 / 2 pi): far inside the 1e-4 bin
    # margin beyond which the exact path decides
    assert float((err * 36 / (2 * math.pi)).max()) < 1e-5
    # atan2_bins: within 1.5e-5 of atan2f * 4 / pi, in bins
    eb = np.abs(bins.astype(np.float64) - ref64 * 4 / math.pi)
    assert float(eb.max()) < 1.5e-5 + 1e-6, float(eb.max())
    # the pair form (hardware reciprocal instead of the fast division): the
    # same bound
    eb2 = np.abs(bins2.astype(np.float64) - ref64 * 4 / math.pi)
    assert float(eb2.max()) < 1.5e-5 + 1e-6, float(eb2.max())
    # exact axes and the origin
    for (yy, xx, want) in [(0.0, 0.0, 0.0), (0.0, 1.0, 0.0), (1.0, 0.0, 2.0), (-1.0, 0.0, -2.0)]:
        k = np.nonzero((y == yy) & (x == xx))[0][0]
        assert bins[k] == want
