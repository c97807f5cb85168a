"""FP64 "ideal" SIFT — test infrastructure, the ground truth of the precision
statement.

The reference algorithm (src/sift.rs) step for step, with every Gaussian
level kept in float64 and no u8 rounding anywhere: the same blur taps
(imageproc 0.25.0 gaussian_blur_f32's kernel: radius ceil(2 sigma), density
samples, clamp-to-edge, horizontal then vertical pass), the same Lanczos3
taps (image 0.25.6 resize_exact) without the clamp and rounding to u8, the
same octave increments (src/sift.rs:129-177, including their 2^o scaling),
DoG as G/255 differences (src/sift.rs:92-124, 182-204), the strict
26-neighbour test (src/sift.rs:510-603), the Newton refinement with its
thresholds (src/sift.rs:299-503), the orientation histogram
(src/sift.rs:605-726) and the descriptor (src/sift.rs:889-1060). The
reference itself and the CUDA engine quantise every level to u8; the
difference between either and this model is the quantisation error the
precision statement reports. Vectorised with numpy; sized for images up to
about 1 Mpx.
"""
from __future__ import annotations

import math

import numpy as np

PI = math.pi
KEYPOINT_FIELDS = ("x", "y", "size", "angle", "response", "octave", "layer")


def gaussian_kernel(sigma: float) -> np.ndarray:
    r = int(math.ceil(2.0 * sigma))
    x = np.arange(-r, r + 1, dtype=np.float64)
    return np.exp(-(x * x) / (2.0 * sigma * sigma)) / (math.sqrt(2.0 * PI) * sigma)


def _filter(img: np.ndarray, k: np.ndarray, axis: int) -> np.ndarray:
    r = len(k) // 2
    pad = [(0, 0), (0, 0)]
    pad[axis] = (r, r)
    p = np.pad(img, pad, mode="edge")
    n = img.shape[axis]
    out = np.zeros_like(img)
    for i, w in enumerate(k):
        sl = [slice(None), slice(None)]
        sl[axis] = slice(i, i + n)
        out += p[tuple(sl)] * w
    return out


def _u8_trunc(a: np.ndarray) -> np.ndarray:
    """imageproc's Clamp<f32> to u8 (truncation), for the quantised check."""
    return np.clip(np.trunc(a), 0.0, 255.0)


def gaussian_blur(img: np.ndarray, sigma: float, quantize: bool = False) -> np.ndarray:
    if img.size == 0:
        return img
    k = gaussian_kernel(sigma)
    if quantize:
        return _u8_trunc(_filter(_u8_trunc(_filter(img, k, 1)), k, 0))
    return _filter(_filter(img, k, 1), k, 0)


def _lanczos3(x: np.ndarray) -> np.ndarray:
    def sinc(t):
        a = t * PI
        return np.where(t == 0.0, 1.0, np.sin(a) / np.where(a == 0.0, 1.0, a))
    return np.where(np.abs(x) < 3.0, sinc(x) * sinc(x / 3.0), 0.0)


def _resample_matrix(src: int, dst: int) -> np.ndarray:
    m = np.zeros((dst, src))
    ratio = src / dst
    sratio = max(ratio, 1.0)
    support = 3.0 * sratio
    for o in range(dst):
        c = (o + 0.5) * ratio
        left = min(max(int(math.floor(c - support)), 0), src - 1)
        right = max(left + 1, min(int(math.ceil(c + support)), src))
        j = np.arange(left, right)
        w = _lanczos3((j - (c - 0.5)) / sratio)
        m[o, left:right] = w / w.sum()
    return m


def resize_lanczos3(img: np.ndarray, nw: int, nh: int, quantize: bool = False) -> np.ndarray:
    h, w = img.shape
    if nw == 0 or nh == 0 or w == 0 or h == 0:
        return np.zeros((nh, nw))
    out = _resample_matrix(h, nh) @ img @ _resample_matrix(w, nw).T
    return np.floor(np.clip(out, 0.0, 255.0) + 0.5) if quantize else out


class Ideal64:
    """quantize=True puts back the reference's u8 rounding of every level and
    dog_f32=True its f32 DoG (v/255 differences rounded to f32): with both,
    the model must reproduce the u8 oracle's candidates and refined keypoints,
    which checks that it is the reference algorithm. (Later stages still
    differ where f32 and f64 put a gradient angle on opposite sides of a bin
    edge: quantised levels give many gradients with gx == 0 exactly, whose
    angle -pi/2 lands on the edge of orientation bins 26 and 27.)"""

    def __init__(self, sigma=1.6, num_octaves=4, num_intervals=3, assumed_blur=0.5, contrast_threshold=0.04,
                 edge_threshold=10.0, border=5, quantize=False, dog_f32=False):
        self.quantize = quantize
        self.dog_f32 = dog_f32
        self.sigma, self.O, self.S = sigma, num_octaves, num_intervals
        self.assumed_blur = assumed_blur
        self.contrast = contrast_threshold / num_intervals  # Sift::new divides by S (src/sift.rs:63-80)
        self.edge = edge_threshold
        self.border = border

    # -- pyramid -------------------------------------------------------------
    def pyramid(self, img: np.ndarray):
        g = img.astype(np.float64)
        amt = math.sqrt(self.sigma ** 2 - self.assumed_blur ** 2) if self.sigma > self.assumed_blur else 0.0
        if amt > 1e-4:
            g = gaussian_blur(g, amt, self.quantize)
        k = 2.0 ** (1.0 / self.S)
        target = [self.sigma * k ** s for s in range(self.S + 3)]
        pyr = []
        cur = g
        for o in range(self.O):
            levels = [cur]
            prev = self.sigma * 2.0 ** o
            for s in range(1, self.S + 3):
                t = target[s] * 2.0 ** o
                blur = math.sqrt(t * t - prev * prev)
                levels.append(levels[-1] if blur < 1e-4 else gaussian_blur(levels[-1], blur, self.quantize))
                prev = t
            pyr.append(levels)
            if o + 1 < self.O:
                src = levels[self.S]
                cur = resize_lanczos3(src, src.shape[1] // 2, src.shape[0] // 2, self.quantize)
        return pyr

    def dog(self, pyr):
        if self.dog_f32:
            f = np.float32
            return [[(lv[i + 1].astype(f) / f(255) - lv[i].astype(f) / f(255)).astype(np.float64)
                     for i in range(len(lv) - 1)] for lv in pyr]
        return [[lv[i + 1] / 255.0 - lv[i] / 255.0 for i in range(len(lv) - 1)] for lv in pyr]

    # -- extrema and refinement -------------------------------------------------
    def extrema(self, dog):
        b = self.border
        out = []
        for o, d in enumerate(dog):
            H, W = d[0].shape
            if H < 3 or W < 3:
                continue
            for s in range(1, self.S + 1):
                if not s < len(d) - 1:
                    continue
                c = d[s][1:-1, 1:-1]
                mx = np.full(c.shape, -np.inf)
                mn = np.full(c.shape, np.inf)
                for dz in (-1, 0, 1):
                    im = d[s + dz]
                    for dy in (-1, 0, 1):
                        for dx in (-1, 0, 1):
                            if dz == 0 and dy == 0 and dx == 0:
                                continue
                            nv = im[1 + dy:H - 1 + dy, 1 + dx:W - 1 + dx]
                            mx = np.maximum(mx, nv)
                            mn = np.minimum(mn, nv)
                ext = (c > mx) | (c < mn)
                ys, xs = np.nonzero(ext)
                ys, xs = ys + 1, xs + 1
                keep = (ys >= b) & (ys < H - b) & (xs >= b) & (xs < W - b)
                for y, x in zip(ys[keep], xs[keep]):
                    out.append((o, s, int(x), int(y)))
        return out

    def refine(self, cands, dog):
        res = []
        for (o, s, x, y) in cands:
            d = dog[o]
            cx, cy, cl = x, y, s
            nl = len(d)
            scale = 2.0 ** o
            for _ in range(5):
                if cl < 1 or cl >= nl - 1:
                    break
                ip, ic, inx = d[cl - 1], d[cl], d[cl + 1]
                H, W = ic.shape
                if cx < 1 or cx >= W - 1 or cy < 1 or cy >= H - 1:
                    break
                c = ic[cy, cx]
                dx = (ic[cy, cx + 1] - ic[cy, cx - 1]) / 2
                dy = (ic[cy + 1, cx] - ic[cy - 1, cx]) / 2
                ds = (inx[cy, cx] - ip[cy, cx]) / 2
                dxx = ic[cy, cx + 1] + ic[cy, cx - 1] - 2 * c
                dyy = ic[cy + 1, cx] + ic[cy - 1, cx] - 2 * c
                dss = inx[cy, cx] + ip[cy, cx] - 2 * c
                dxy = (ic[cy + 1, cx + 1] - ic[cy + 1, cx - 1] - ic[cy - 1, cx + 1] + ic[cy - 1, cx - 1]) / 4
                dxs = (inx[cy, cx + 1] - inx[cy, cx - 1] - (ip[cy, cx + 1] - ip[cy, cx - 1])) / 4
                dys = (inx[cy + 1, cx] - inx[cy - 1, cx] - (ip[cy + 1, cx] - ip[cy - 1, cx])) / 4
                hm = np.array([[dxx, dxy, dxs], [dxy, dyy, dys], [dxs, dys, dss]])
                if abs(np.linalg.det(hm)) < 1e-10:
                    break
                off = np.linalg.solve(hm, -np.array([dx, dy, ds]))
                if np.all(np.abs(off) < 0.5):
                    val = c + 0.5 * (dx * off[0] + dy * off[1] + ds * off[2])
                    if abs(val) < self.contrast:
                        break
                    tr, det = dxx + dyy, dxx * dyy - dxy * dxy
                    if det <= 0 or tr * tr / det >= (self.edge + 1) ** 2 / self.edge:
                        break
                    lf = cl + off[2]
                    res.append(dict(x=(cx + off[0]) * scale, y=(cy + off[1]) * scale,
                                    size=self.sigma * 2.0 ** (o + lf / self.S), angle=0.0, response=val,
                                    octave=o, layer=int(np.floor(lf + 0.5)) if lf >= 0 else -int(np.floor(-lf + 0.5))))
                    break
                cx = int(round(cx + off[0]))
                cy = int(round(cy + off[1]))
                cl = int(round(cl + off[2]))
                if cl < 0 or cl >= nl:
                    break
        return res

    # -- orientation and descriptor ---------------------------------------------
    @staticmethod
    def _pix(im, xi, yi):
        H, W = im.shape
        return im[np.clip(yi, 0, H - 1), np.clip(xi, 0, W - 1)] / 255.0

    def orientations(self, kps, pyr):
        out = []
        for kp in kps:
            o = kp["octave"]
            li = min(max(kp["layer"], 0), self.S + 2)
            im = pyr[o][li]
            H, W = im.shape
            scale = 2.0 ** o
            xo, yo, so = kp["x"] / scale, kp["y"] / scale, kp["size"] / scale
            r = int(math.floor(4.5 * so + 0.5))
            wd = 2.0 * (1.5 * so) ** 2
            dy, dx = np.mgrid[-r:r + 1, -r:r + 1].astype(np.float64)
            xi = np.floor(xo + dx + 0.5).astype(np.int64)
            yi = np.floor(yo + dy + 0.5).astype(np.int64)
            ok = (xi >= 1) & (xi < W - 1) & (yi >= 1) & (yi < H - 1)
            xi, yi, dx, dy = xi[ok], yi[ok], dx[ok], dy[ok]
            gx = self._pix(im, xi + 1, yi) - self._pix(im, xi - 1, yi)
            gy = self._pix(im, xi, yi + 1) - self._pix(im, xi, yi - 1)
            mag = np.hypot(gx, gy)
            ang = np.arctan2(gy, gx)
            w = np.exp(-(dx * dx + dy * dy) / wd)
            an = np.where(ang < 0, ang + 2 * PI, ang)
            b = np.floor(an * 36 / (2 * PI)).astype(np.int64) % 36
            hist = np.bincount(b, weights=mag * w, minlength=36)
            for _ in range(2):
                hist = (np.roll(hist, 1) + hist + np.roll(hist, -1)) / 3.0
            thr = hist.max() * 0.8
            for bi in range(36):
                cv, pv, nv = hist[bi], hist[(bi - 1) % 36], hist[(bi + 1) % 36]
                if cv >= thr and cv > pv and cv > nv:
                    den = pv - 2 * cv + nv
                    off = 0.5 * (pv - nv) / den if abs(den) > 1e-5 else 0.0
                    a = (bi + 0.5 + off) * (2 * PI / 36)
                    fa = a % (2 * PI)
                    if fa > PI:
                        fa -= 2 * PI
                    out.append(dict(kp, angle=fa))
        return out

    def _bilinear(self, im, x, y):
        xf, yf = np.floor(x), np.floor(y)
        dx, dy = x - xf, y - yf
        x0, y0 = xf.astype(np.int64), yf.astype(np.int64)
        q11, q21 = self._pix(im, x0, y0), self._pix(im, x0 + 1, y0)
        q12, q22 = self._pix(im, x0, y0 + 1), self._pix(im, x0 + 1, y0 + 1)
        return q11 * (1 - dx) * (1 - dy) + q21 * dx * (1 - dy) + q12 * (1 - dx) * dy + q22 * dx * dy

    def descriptor(self, kp, pyr):
        o = kp["octave"]
        li = min(max(kp["layer"], 0), self.S + 2)
        im = pyr[o][li]
        H, W = im.shape
        scale = 2.0 ** o
        xo, yo, so = kp["x"] / scale, kp["y"] / scale, kp["size"] / scale
        ca, sa = math.cos(kp["angle"]), math.sin(kp["angle"])
        bw = 3.0 * so
        ww = 4.0 * bw
        wd = 2.0 * (0.5 * ww) ** 2
        rad = int(math.ceil(ww * math.sqrt(2.0) * 0.5))
        py, px = np.mgrid[-rad:rad + 1, -rad:rad + 1].astype(np.float64)
        rx, ry = ca * px + sa * py, -sa * px + ca * py
        xb, yb = rx / bw + 1.5, ry / bw + 1.5
        xs, ys = xo + px, yo + py
        ok = (xb > -1) & (xb < 4) & (yb > -1) & (yb < 4) & (xs >= 0) & (xs < W - 1) & (ys >= 0) & (ys < H - 1)
        px, py, xb, yb, xs, ys = px[ok], py[ok], xb[ok], yb[ok], xs[ok], ys[ok]
        gx = self._bilinear(im, xs + 1, ys) - self._bilinear(im, xs - 1, ys)
        gy = self._bilinear(im, xs, ys + 1) - self._bilinear(im, xs, ys - 1)
        wm = np.hypot(gx, gy) * np.exp(-(px * px + py * py) / wd)
        ab = ((np.arctan2(gy, gx) - kp["angle"]) % (2 * PI)) * 8 / (2 * PI)
        xbi, ybi, abi = np.floor(xb).astype(np.int64), np.floor(yb).astype(np.int64), np.floor(ab).astype(np.int64)
        fx, fy, fa = xb - xbi, yb - ybi, ab - abi
        hist = np.zeros(128)
        for i in (0, 1):
            for j in (0, 1):
                for k in (0, 1):
                    ix, iy, ia = xbi + i, ybi + j, (abi + k) % 8
                    m = (ix >= 0) & (ix < 4) & (iy >= 0) & (iy < 4)
                    c = wm * (fx if i else 1 - fx) * (fy if j else 1 - fy) * (fa if k else 1 - fa)
                    np.add.at(hist, ((iy * 4 + ix) * 8 + ia)[m], c[m])
        n = np.linalg.norm(hist)
        if n >= 1e-8:
            hist = np.minimum(hist / n, 0.2)
            n2 = np.linalg.norm(hist)
            if n2 >= 1e-8:
                hist /= n2
        return hist

    def detect_and_compute(self, img: np.ndarray):
        pyr = self.pyramid(img)
        dog = self.dog(pyr)
        kps = self.orientations(self.refine(self.extrema(dog), dog), pyr)
        desc = np.array([self.descriptor(kp, pyr) for kp in kps]).reshape(-1, 128)
        arr = np.zeros(len(kps), dtype=[(f, np.float64) for f in KEYPOINT_FIELDS])
        for f in KEYPOINT_FIELDS:
            arr[f] = [kp[f] for kp in kps]
        return arr, desc, pyr, dog
