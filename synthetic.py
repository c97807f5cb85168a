"""Seeded synthetic inputs of the benchmark and test workloads.

Pure numpy: no native library is loaded, so the bench's reference arm, the
CUDA arm, the tests and the smoke check all draw the same images without
touching either the engine or the oracle.

Image model (the 512 x 512 density: 200 blobs and 40 rectangles, scaled by
area): background 128; isotropic Gaussian blobs with centres uniform over the
image, sigma U(2, 20) px, amplitude U(-90, 90), each added over a window of
+-ceil(4 sigma); filled axis-aligned rectangles drawn over them (sides
8 + floor(89 U) px, intensity floor(256 U)); i.i.d. N(0, 3^2) noise (Box-Muller);
clamped to [0, 255] and rounded half away from zero to u8. All arithmetic is
f64.

RNG: counter-based. Draw i of stream k is splitmix64's output function applied
to seed * 0xD1B54A32D192ED03 + k * 0x8CB92BA72F3D8DD7 + (i + 1) *
0x9E3779B97F4A7C15 (mod 2^64), top 53 bits scaled to [0, 1). Streams: 1 blob
parameters (4 draws per blob), 2 rectangles (5 draws per rectangle), 3 noise
(2 draws per pixel). Every draw is independent of the others, so the whole
image vectorises and the same seed gives the same image on any host.
"""
from __future__ import annotations

import numpy as np

_GOLD = np.uint64(0x9E3779B97F4A7C15)
_SEED_MUL = np.uint64(0xD1B54A32D192ED03)
_STREAM_MUL = np.uint64(0x8CB92BA72F3D8DD7)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def _mix(z: np.ndarray) -> np.ndarray:
    z = (z ^ (z >> np.uint64(30))) * _M1
    z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


def uniforms(seed: int, stream: int, start: int, n: int) -> np.ndarray:
    """Draws [start, start + n) of `stream` under `seed`, as f64 in [0, 1)."""
    with np.errstate(over="ignore"):
        key = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) * _SEED_MUL + np.uint64(stream) * _STREAM_MUL
        idx = np.arange(start + 1, start + n + 1, dtype=np.uint64)
        z = _mix(key + idx * _GOLD)
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def density(width: int, height: int) -> tuple[int, int]:
    """Blob and rectangle counts at the 512 x 512 density (200 blobs, 40
    rectangles), rounded half away from zero."""
    area = width * height / (512.0 * 512.0)
    return int(np.floor(200.0 * area + 0.5)), int(np.floor(40.0 * area + 0.5))


def synth_image(seed: int, width: int, height: int, n_blobs: int | None = None,
                n_rects: int | None = None) -> np.ndarray:
    """The seeded height x width u8 image of the model above."""
    W, H = int(width), int(height)
    out = np.empty((H, W), dtype=np.uint8)
    if W == 0 or H == 0:
        return out
    db, dr = density(W, H)
    n_blobs = db if n_blobs is None else int(n_blobs)
    n_rects = dr if n_rects is None else int(n_rects)
    img = np.full((H, W), 128.0)
    bp = uniforms(seed, 1, 0, 4 * n_blobs).reshape(-1, 4)
    for u_cx, u_cy, u_sg, u_amp in bp:
        cx, cy = u_cx * W, u_cy * H
        sg = 2.0 + 18.0 * u_sg
        amp = -90.0 + 180.0 * u_amp
        rad = int(np.ceil(4.0 * sg))
        fx, fy = int(np.floor(cx)), int(np.floor(cy))
        x0, x1 = max(0, fx - rad), min(W - 1, fx + rad)
        y0, y1 = max(0, fy - rad), min(H - 1, fy + rad)
        if x0 > x1 or y0 > y1:
            continue
        dx2 = (np.arange(x0, x1 + 1, dtype=np.float64) - cx) ** 2
        dy2 = (np.arange(y0, y1 + 1, dtype=np.float64) - cy) ** 2
        inv = 1.0 / (2.0 * sg * sg)
        img[y0:y1 + 1, x0:x1 + 1] += amp * np.exp(-(dy2[:, None] + dx2[None, :]) * inv)
    rp = uniforms(seed, 2, 0, 5 * n_rects).reshape(-1, 5)
    for u_x, u_y, u_w, u_h, u_v in rp:
        rx, ry = int(u_x * W), int(u_y * H)
        rw, rh = 8 + int(u_w * 89.0), 8 + int(u_h * 89.0)
        img[ry:min(H, ry + rh), rx:min(W, rx + rw)] = np.floor(u_v * 256.0)
    rows = max(1, (1 << 21) // W)  # noise in bands of about 2 M pixels
    for y in range(0, H, rows):
        yb = min(H, y + rows)
        n = (yb - y) * W
        u = uniforms(seed, 3, 2 * y * W, 2 * n)
        u1 = 1.0 - u[0::2]  # (0, 1]
        noise = np.sqrt(-2.0 * np.log(u1)) * np.cos(6.283185307179586 * u[1::2])
        v = np.clip(img[y:yb].ravel() + 3.0 * noise, 0.0, 255.0)
        f = np.floor(v)
        out[y:yb] = (f + (v - f >= 0.5)).astype(np.uint8).reshape(yb - y, W)
    return out


def batch64_shapes() -> list[tuple[int, int]]:
    """(width, height) of the 64 images of the uneven batch: each uniform over
    the multiples of 16 in [320, 2560] (numpy default_rng(2))."""
    rng = np.random.default_rng(2)
    dims = rng.integers(20, 161, size=(64, 2)) * 16
    return [(int(w), int(h)) for w, h in dims]


def batch64_images() -> list[np.ndarray]:
    """The uneven batch: image i of batch64_shapes() drawn with seed 1000 + i."""
    return [synth_image(1000 + i, w, h) for i, (w, h) in enumerate(batch64_shapes())]
