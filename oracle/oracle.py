"""ctypes wrapper of the CPU oracle (oracle/sift_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and by
bench.py's CPU-baseline leg, never by the product package.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from .build import LIB, build

KEYPOINT_DTYPE = np.dtype(
    [("x", "<f4"), ("y", "<f4"), ("size", "<f4"), ("angle", "<f4"), ("response", "<f4"),
     ("octave", "<i4"), ("layer", "<i4")]
)


class OracleParams(C.Structure):
    _fields_ = [
        ("sigma", C.c_float),
        ("num_octaves", C.c_uint32),
        ("num_intervals", C.c_uint32),
        ("assumed_blur", C.c_float),
        ("contrast_threshold", C.c_float),
        ("edge_threshold", C.c_float),
        ("image_border_width", C.c_uint32),
    ]


class OracleResult(C.Structure):
    _fields_ = [("n", C.c_uint32), ("kps", C.c_void_p), ("desc", C.POINTER(C.c_float))]


class OracleStages(C.Structure):
    _fields_ = [
        ("num_octaves", C.c_uint32),
        ("levels_per_octave", C.c_uint32),
        ("oct_w", C.POINTER(C.c_uint32)),
        ("oct_h", C.POINTER(C.c_uint32)),
        ("pyramid", C.POINTER(C.c_uint8)),
        ("pyramid_bytes", C.c_uint64),
        ("n_candidates", C.c_uint32),
        ("candidates", C.c_void_p),
        ("n_refined", C.c_uint32),
        ("refined", C.c_void_p),
        ("result", OracleResult),
    ]


class OracleBlurModel(C.Structure):
    _fields_ = [("blur_radius_factor_x100", C.c_int), ("blur_normalize", C.c_int), ("blur_round", C.c_int)]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        P = C.POINTER
        u32, f32 = C.c_uint32, C.c_float
        L.oracle_default_params.argtypes = [P(OracleParams)]
        L.oracle_new_params.argtypes = [P(OracleParams), f32, u32, u32, f32, f32, f32]
        L.oracle_detect_and_compute.argtypes = [P(OracleParams), C.c_void_p, u32, u32, u32, C.c_int, P(OracleResult)]
        L.oracle_detect.argtypes = L.oracle_detect_and_compute.argtypes
        L.oracle_result_free.argtypes = [P(OracleResult)]
        L.oracle_stages.argtypes = [P(OracleParams), C.c_void_p, u32, u32, u32, C.c_int, P(OracleStages)]
        L.oracle_stages_free.argtypes = [P(OracleStages)]
        L.oracle_gaussian_blur_u8.argtypes = [C.c_void_p, u32, u32, f32, C.c_void_p]
        L.oracle_gaussian_kernel.argtypes = [f32, P(f32), C.c_int]
        L.oracle_resize_lanczos3_u8.argtypes = [C.c_void_p, u32, u32, u32, u32, C.c_void_p]
        L.oracle_solve3.argtypes = [P(f32), P(f32), P(f32)]
        L.oracle_bilinear.argtypes = [C.c_void_p, u32, u32, f32, f32]
        L.oracle_bilinear.restype = f32
        L.oracle_blur_sigmas.argtypes = [P(OracleParams), P(f32), C.c_int]
        L.oracle_get_blur_model.argtypes = [P(OracleBlurModel)]
        L.oracle_set_blur_model.argtypes = [P(OracleBlurModel)]
        _lib = L
    return _lib


def params(sigma=1.6, num_octaves=4, num_intervals=3, assumed_blur=0.5, contrast_threshold=0.04,
           edge_threshold=10.0) -> OracleParams:
    """Sift::new semantics (contrast divided by num_intervals)."""
    p = OracleParams()
    lib().oracle_new_params(C.byref(p), sigma, num_octaves, num_intervals, assumed_blur, contrast_threshold,
                            edge_threshold)
    return p


def _kps(ptr, n) -> np.ndarray:
    a = np.empty(n, dtype=KEYPOINT_DTYPE)
    if n:
        C.memmove(a.ctypes.data, ptr, n * KEYPOINT_DTYPE.itemsize)
    return a


def detect_and_compute(img: np.ndarray, p: OracleParams | None = None, threads: int = 0):
    """(keypoints, descriptors) of detect_and_compute_cpu."""
    p = p or params()
    img = np.ascontiguousarray(img, dtype=np.uint8)
    h, w = img.shape
    r = OracleResult()
    rc = lib().oracle_detect_and_compute(C.byref(p), img.ctypes.data if img.size else None, w, h, w, threads,
                                         C.byref(r))
    if rc != 0:
        raise RuntimeError("oracle rejected its arguments")
    try:
        kps = _kps(r.kps, r.n)
        desc = np.empty((r.n, 128), dtype=np.float32)
        if r.n:
            C.memmove(desc.ctypes.data, r.desc, r.n * 128 * 4)
    finally:
        lib().oracle_result_free(C.byref(r))
    return kps, desc


@dataclass
class Stages:
    octave_dims: list
    levels: int
    pyramid: np.ndarray  # flat u8, octave-major / level / row-major
    candidates: np.ndarray
    refined: np.ndarray
    keypoints: np.ndarray
    descriptors: np.ndarray

    def level(self, o: int, s: int) -> np.ndarray:
        off = 0
        for oo, (w, h) in enumerate(self.octave_dims):
            for ss in range(self.levels):
                if oo == o and ss == s:
                    return self.pyramid[off:off + w * h].reshape(h, w)
                off += w * h
        raise IndexError((o, s))


def stages(img: np.ndarray, p: OracleParams | None = None, threads: int = 0) -> Stages:
    p = p or params()
    img = np.ascontiguousarray(img, dtype=np.uint8)
    h, w = img.shape
    s = OracleStages()
    rc = lib().oracle_stages(C.byref(p), img.ctypes.data if img.size else None, w, h, w, threads, C.byref(s))
    if rc != 0:
        raise RuntimeError("oracle rejected its arguments")
    try:
        dims = [(s.oct_w[i], s.oct_h[i]) for i in range(s.num_octaves)]
        pyr = np.ctypeslib.as_array(s.pyramid, shape=(s.pyramid_bytes,)).copy() if s.pyramid_bytes else \
            np.zeros(0, np.uint8)
        n = s.result.n
        desc = np.empty((n, 128), dtype=np.float32)
        if n:
            C.memmove(desc.ctypes.data, s.result.desc, n * 128 * 4)
        return Stages(dims, s.levels_per_octave, pyr, _kps(s.candidates, s.n_candidates),
                      _kps(s.refined, s.n_refined), _kps(s.result.kps, n), desc)
    finally:
        lib().oracle_stages_free(C.byref(s))


def gaussian_blur(img: np.ndarray, sigma: float) -> np.ndarray:
    img = np.ascontiguousarray(img, dtype=np.uint8)
    h, w = img.shape
    out = np.empty_like(img)
    lib().oracle_gaussian_blur_u8(img.ctypes.data, w, h, sigma, out.ctypes.data)
    return out


def gaussian_kernel(sigma: float) -> np.ndarray:
    buf = (C.c_float * 4096)()
    n = lib().oracle_gaussian_kernel(sigma, buf, 4096)
    return np.array(buf[:n], dtype=np.float32)


def resize_lanczos3(img: np.ndarray, nw: int, nh: int) -> np.ndarray:
    img = np.ascontiguousarray(img, dtype=np.uint8)
    h, w = img.shape
    out = np.empty((nh, nw), dtype=np.uint8)
    lib().oracle_resize_lanczos3_u8(img.ctypes.data, w, h, nw, nh, out.ctypes.data)
    return out


def solve3(a, b):
    A = (C.c_float * 9)(*np.asarray(a, dtype=np.float32).ravel().tolist())
    B = (C.c_float * 3)(*np.asarray(b, dtype=np.float32).tolist())
    X = (C.c_float * 3)()
    ok = lib().oracle_solve3(A, B, X)
    return [X[0], X[1], X[2]] if ok else None


def bilinear(img: np.ndarray, x: float, y: float) -> float:
    img = np.ascontiguousarray(img, dtype=np.uint8)
    h, w = img.shape
    return float(lib().oracle_bilinear(img.ctypes.data, w, h, x, y))


def blur_sigmas(p: OracleParams | None = None) -> np.ndarray:
    p = p or params()
    buf = (C.c_float * 1024)()
    n = lib().oracle_blur_sigmas(C.byref(p), buf, 1024)
    return np.array(buf[:n], dtype=np.float32)


def get_blur_model() -> OracleBlurModel:
    m = OracleBlurModel()
    lib().oracle_get_blur_model(C.byref(m))
    return m


def set_blur_model(m: OracleBlurModel) -> None:
    lib().oracle_set_blur_model(C.byref(m))


def luma_u8(pixels: np.ndarray, fmt: int) -> np.ndarray:
    """Colour to 8-bit luma, restated for the conversion kernel's parity test.

    fmt 1 / 2 (RGB8 / RGBA8): image 0.25.6 DynamicImage::to_luma8, the path of
    src/sift.rs:1202 and 1256 (the crate is not vendored): integer
    (2126 r + 7152 g + 722 b) / 10000, truncating, alpha ignored.
    fmt 3 (RGBA8 canvas): img_from_raw, src/wasm.rs:89-93: f32
    0.299 r + 0.587 g + 0.114 b, each product and sum rounded to f32 in that
    order, then `as u8` (truncation, saturating)."""
    p = np.asarray(pixels)
    r, g, b = (p[..., k].astype(np.uint32) for k in range(3))
    if fmt in (1, 2):
        return ((2126 * r + 7152 * g + 722 * b) // 10000).astype(np.uint8)
    f = np.float32
    rf, gf, bf = r.astype(f), g.astype(f), b.astype(f)
    lum = (f(0.299) * rf + f(0.587) * gf) + f(0.114) * bf
    return np.clip(np.trunc(lum), 0, 255).astype(np.uint8)
