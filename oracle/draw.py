"""draw_keypoints_to_image on the CPU: the oracle of the engine's
sift_cuda_draw_keypoints (test infrastructure only; the product path is the
CUDA kernel in sift_wgpu_gb300/csrc/draw.cu).

Follows src/lib.rs:69-116: the grey image as RGB (to_rgb8 replicates the
grey value); for each keypoint a filled circle of radius round(2.0 * 3) = 6
at (x as i32, y as i32), the orientation line from (x, y) to
(x + 6 cos(angle), y + 6 sin(angle)) and a filled circle of radius 1, all in
one colour. The drawing primitives belong to imageproc 0.25.0
(Cargo.lock:634-636), which is not vendored; they are restated from their
published algorithms: draw_filled_circle_mut as the midpoint-circle walk that
fills four horizontal spans per step, draw_line_segment_mut as a Bresenham
walk over f32 endpoints with an f32 error term (coordinates truncated with
`as i32`), each point kept if inside the image. Parity with imageproc itself is
unpinned (no reference test draws).
"""
from __future__ import annotations

import math

import numpy as np

f32 = np.float32


def _as_i32(v) -> int:
    return int(math.trunc(float(v)))


def _line(img, x0, y0, x1, y1, color):
    h, w = img.shape[:2]
    x0, y0, x1, y1 = f32(x0), f32(y0), f32(x1), f32(y1)
    steep = abs(f32(y1 - y0)) > abs(f32(x1 - x0))
    if steep:
        x0, y0, x1, y1 = y0, x0, y1, x1
    if x0 > x1:
        x0, x1, y0, y1 = x1, x0, y1, y0
    dx, dy = f32(x1 - x0), abs(f32(y1 - y0))
    x, y, end_x = _as_i32(x0), _as_i32(y0), _as_i32(x1)
    step = 1 if y0 < y1 else -1
    err = f32(dx / f32(2.0))
    while x <= end_x:
        px, py = (y, x) if steep else (x, y)
        if 0 <= px < w and 0 <= py < h:
            img[py, px] = color
        x += 1
        err = f32(err - dy)
        if err < 0:
            y += step
            err = f32(err + dx)


def _filled_circle(img, cx, cy, radius, color):
    x, y, p = 0, radius, 1 - radius
    while x <= y:
        _line(img, cx - x, cy + y, cx + x, cy + y, color)
        _line(img, cx - y, cy + x, cx + y, cy + x, color)
        _line(img, cx - x, cy - y, cx + x, cy - y, color)
        _line(img, cx - y, cy - x, cx + y, cy - x, color)
        x += 1
        if p < 0:
            p += 2 * x + 1
        else:
            y -= 1
            p += 2 * (x - y) + 1


def draw_keypoints_to_image(gray: np.ndarray, kps: np.ndarray, color=(255, 0, 0)) -> np.ndarray:
    img = np.repeat(np.asarray(gray, dtype=np.uint8)[:, :, None], 3, axis=2)
    col = np.array(color, dtype=np.uint8)
    radius = 6
    for k in kps:
        x, y, a = f32(k["x"]), f32(k["y"]), f32(k["angle"])
        cx, cy = _as_i32(x), _as_i32(y)
        _filled_circle(img, cx, cy, radius, col)
        ca, sa = f32(math.cos(float(a))), f32(math.sin(float(a)))
        _line(img, x, y, f32(x + f32(f32(radius) * ca)), f32(y + f32(f32(radius) * sa)), col)
        _filled_circle(img, cx, cy, 1, col)
    return img
