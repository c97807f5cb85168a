"""Python mirror of the reference crate's public SIFT API over libsiftcuda.so.

Names, fields and argument meanings follow the Rust crate stevel705/sift-wgpu:

* ``Sift`` / ``Sift.new`` / ``Sift.default``      — src/sift.rs:36-80
* ``KeyPoint``                                    — src/keypoints.rs:2-10
* ``SiftBackend`` and ``SiftBackend.from_str``    — src/lib.rs:19-50, plus the
  new ``Cuda`` arm and its ``"cuda"`` string
* ``Sift.detect_and_compute_with_backend``        — src/sift.rs:1244-1355
* ``Sift.detect``                                 — src/sift.rs:846-886

Only the ``Cuda`` arm is implemented here; the other arms belong to the
reference crate. Failures raise ``SiftError`` (the reference's Err(String)); no
call ever falls back to a CPU path.
"""
from __future__ import annotations

import ctypes as C
import enum
import threading
from dataclasses import dataclass

import numpy as np

from . import _capi
from ._capi import DESC_LEN, KEYPOINT_DTYPE, SiftCudaError

__all__ = [
    "Engine", "KeyPoint", "Sift", "SiftBackend", "SiftError", "keypoints_from_array",
]

DEFAULT_SIGMA = 1.6
DEFAULT_NUM_OCTAVES = 4
DEFAULT_NUM_INTERVALS = 3
DEFAULT_ASSUMED_BLUR = 0.5
DEFAULT_CONTRAST_THRESHOLD = 0.04
DEFAULT_EDGE_THRESHOLD = 10.0
DEFAULT_IMAGE_BORDER_WIDTH = 5


class SiftError(RuntimeError):
    """Err(String) of detect_and_compute_with_backend."""


class SiftBackend(enum.Enum):
    Cpu = "cpu"
    WebGpu = "webgpu"
    WebGpuWithCpuFallback = "fallback"
    WebGpuV2 = "gpuv2"
    Cuda = "cuda"

    @classmethod
    def default(cls) -> "SiftBackend":
        return cls.WebGpuWithCpuFallback  # src/lib.rs:30-34

    @classmethod
    def from_str(cls, value: str) -> "SiftBackend":
        """FromStr for SiftBackend (src/lib.rs:38-50) with the added "cuda"."""
        v = value.strip().lower()
        table = {
            "cpu": cls.Cpu,
            "webgpu": cls.WebGpu, "wgpu": cls.WebGpu, "gpu": cls.WebGpu,
            "auto": cls.WebGpuWithCpuFallback, "fallback": cls.WebGpuWithCpuFallback,
            "prefer-gpu": cls.WebGpuWithCpuFallback,
            "gpuv2": cls.WebGpuV2, "gpu-v2": cls.WebGpuV2, "webgpu-v2": cls.WebGpuV2, "v2": cls.WebGpuV2,
            "cuda": cls.Cuda,
        }
        if v not in table:
            raise SiftError(f"Unknown SIFT backend: {value}")
        return table[v]


@dataclass
class KeyPoint:
    """KeyPoint (src/keypoints.rs:2-10)."""

    x: float
    y: float
    size: float
    angle: float
    response: float
    octave: int
    layer: int


def keypoints_from_array(a: np.ndarray) -> list[KeyPoint]:
    return [KeyPoint(float(r["x"]), float(r["y"]), float(r["size"]), float(r["angle"]),
                     float(r["response"]), int(r["octave"]), int(r["layer"])) for r in a]


def _as_gray(img) -> np.ndarray:
    a = np.asarray(img)
    if a.dtype != np.uint8 or a.ndim != 2:
        raise SiftError("expected a 2-D uint8 grayscale image (the to_luma8() layout)")
    return a


def _keypoint_array(keypoints) -> np.ndarray:
    if isinstance(keypoints, np.ndarray) and keypoints.dtype == KEYPOINT_DTYPE:
        return np.ascontiguousarray(keypoints)
    a = np.zeros(len(keypoints), dtype=KEYPOINT_DTYPE)
    for i, k in enumerate(keypoints):
        a[i] = (k.x, k.y, k.size, k.angle, k.response, k.octave, k.layer)
    return a


class _ResultOwner:
    """Frees a SiftCudaResult's arrays when the numpy arrays over them are gone."""

    def __init__(self, res):
        self.res = res

    def __del__(self):
        try:
            _capi.lib().sift_cuda_result_free(C.byref(self.res))
        except Exception:
            pass


def _owned_result(res, with_desc: bool):
    """(keypoints, descriptors) over the arrays a non-view entry allocated."""
    n = res.n
    owner = _ResultOwner(res)
    kb = (C.c_char * (n * KEYPOINT_DTYPE.itemsize)).from_address(C.cast(res.kps, C.c_void_p).value)
    kb._owner = owner
    kps = np.frombuffer(kb, dtype=KEYPOINT_DTYPE)
    desc = None
    if with_desc:
        db = (C.c_float * (n * DESC_LEN)).from_address(C.cast(res.desc, C.c_void_p).value)
        db._owner = owner
        desc = np.frombuffer(db, dtype=np.float32).reshape(n, DESC_LEN)
    return kps, desc


class Engine:
    """One libsiftcuda engine: a CUDA stream plus resident device arenas."""

    def __init__(self, params: "Sift | _capi.Params | None" = None, device: int = 0, storage: str = "u8",
                 level_tile_rows: int = 0):
        L = _capi.lib()
        if params is None:
            params = Sift.default()
        p = params.to_c() if isinstance(params, Sift) else params
        opts = _capi.Options()
        L.sift_cuda_options_default(C.byref(opts))
        opts.device = device
        opts.storage = {"f32": _capi.STORAGE_F32, "f16": _capi.STORAGE_F16, "u8": _capi.STORAGE_U8}[storage]
        opts.level_tile_rows = level_tile_rows  # 0: the default (64-row tiles)
        h = C.c_void_p()
        _capi.check(L.sift_cuda_create(C.byref(p), C.byref(opts), C.byref(h)))
        self._h = h
        self.storage = storage
        self.params = p

    @property
    def handle(self) -> C.c_void_p:
        if not self._h:
            raise SiftError("engine is closed")
        return self._h

    def close(self) -> None:
        if getattr(self, "_h", None):
            _capi.lib().sift_cuda_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _call(self, fn, img: np.ndarray, with_desc: bool, view: bool = False):
        """Runs fn and returns its result as arrays the caller owns. view=True:
        fn is a view entry (results in the engine's host buffers), copied out;
        otherwise fn returns arrays the library allocated for this call, which
        the returned numpy arrays wrap without a copy and free with
        sift_cuda_result_free when both are gone."""
        img = _as_gray(img)
        h, w = img.shape
        stride = img.strides[0]
        if img.strides[1] != 1:
            img = np.ascontiguousarray(img)
            stride = w
        res = _capi.Result()
        _capi.check(fn(self.handle, img.ctypes.data if img.size else None, w, h, stride, C.byref(res)))
        n = res.n
        if not view and n:
            return _owned_result(res, with_desc)
        try:
            kps = np.empty(n, dtype=KEYPOINT_DTYPE)
            if n:
                C.memmove(kps.ctypes.data, res.kps, n * KEYPOINT_DTYPE.itemsize)
            desc = None
            if with_desc:
                desc = np.empty((n, DESC_LEN), dtype=np.float32)
                if n:
                    C.memmove(desc.ctypes.data, res.desc, n * DESC_LEN * 4)
        finally:
            if not view:
                _capi.lib().sift_cuda_result_free(C.byref(res))
        return kps, desc

    def detect_and_compute(self, img) -> tuple[np.ndarray, np.ndarray]:
        """Keypoints (structured array) and descriptors (n x 128 f32).
        H x W x 3 (RGB) and H x W x 4 (RGBA) uint8 images are converted to
        luma on the device the way DynamicImage::to_luma8 does."""
        a = np.asarray(img)
        if a.ndim == 3 and a.dtype == np.uint8 and a.shape[2] in (3, 4):
            return self.detect_and_compute_pixels(a, _capi.PIXELS_RGB8 if a.shape[2] == 3 else _capi.PIXELS_RGBA8)
        # the drop-in entry: the library copies the results out of the
        # buffers the GPU wrote (over a few host threads) into arrays that
        # are returned without another copy
        return self._call(_capi.lib().sift_cuda_detect_and_compute, img, True)

    def detect_and_compute_pixels(self, img, fmt: int) -> tuple[np.ndarray, np.ndarray]:
        """A colour image (H x W x 3 for PIXELS_RGB8, H x W x 4 for PIXELS_RGBA8
        or PIXELS_RGBA8_CANVAS) converted to luma on the device, then the
        pipeline (sift_cuda_detect_and_compute_pixels)."""
        a = np.asarray(img)
        ch = {_capi.PIXELS_RGB8: 3, _capi.PIXELS_RGBA8: 4, _capi.PIXELS_RGBA8_CANVAS: 4}.get(fmt)
        if ch is None or a.dtype != np.uint8 or a.ndim != 3 or a.shape[2] != ch:
            raise SiftError(f"expected an H x W x {ch} uint8 image for pixel format {fmt}")
        if a.strides[2] != 1 or a.strides[1] != ch:
            a = np.ascontiguousarray(a)
        h, w = a.shape[:2]
        res = _capi.Result()
        L = _capi.lib()
        _capi.check(L.sift_cuda_detect_and_compute_pixels(self.handle, a.ctypes.data if a.size else None, w, h,
                                                          a.strides[0], fmt, C.byref(res)))
        try:
            n = res.n
            kps = np.empty(n, dtype=KEYPOINT_DTYPE)
            desc = np.empty((n, DESC_LEN), dtype=np.float32)
            if n:
                C.memmove(kps.ctypes.data, res.kps, n * KEYPOINT_DTYPE.itemsize)
                C.memmove(desc.ctypes.data, res.desc, n * DESC_LEN * 4)
        finally:
            L.sift_cuda_result_free(C.byref(res))
        return kps, desc

    def detect(self, img) -> np.ndarray:
        return self._call(_capi.lib().sift_cuda_detect, img, False)[0]

    def detect_and_compute_view(self, img) -> tuple[np.ndarray, np.ndarray]:
        """Zero-copy form: numpy views of the engine's pinned result buffers,
        valid until the next call on this engine."""
        img = _as_gray(img)
        h, w = img.shape
        if img.strides[1] != 1:
            img = np.ascontiguousarray(img)
        res = _capi.Result()
        _capi.check(_capi.lib().sift_cuda_detect_and_compute_view(
            self.handle, img.ctypes.data if img.size else None, w, h, img.strides[0], C.byref(res)))
        n = res.n
        if n == 0:
            return np.empty(0, KEYPOINT_DTYPE), np.empty((0, DESC_LEN), np.float32)
        kbuf = (C.c_char * (n * KEYPOINT_DTYPE.itemsize)).from_address(C.cast(res.kps, C.c_void_p).value)
        dbuf = (C.c_char * (n * DESC_LEN * 4)).from_address(C.cast(res.desc, C.c_void_p).value)
        return (np.frombuffer(kbuf, dtype=KEYPOINT_DTYPE, count=n),
                np.frombuffer(dbuf, dtype=np.float32, count=n * DESC_LEN).reshape(n, DESC_LEN))

    # drawing -----------------------------------------------------------------
    def draw_keypoints(self, img, keypoints, color=(255, 0, 0)) -> np.ndarray:
        """draw_keypoints_to_image (src/lib.rs:69-116) on the GPU: an
        (h, w, 3) uint8 RGB image. keypoints: a KEYPOINT_DTYPE array or a
        sequence of KeyPoint."""
        g = _as_gray(img)
        if g.strides[1] != 1:
            g = np.ascontiguousarray(g)
        h, w = g.shape
        kps = _keypoint_array(keypoints)
        out = np.empty((h, w, 3), dtype=np.uint8)
        if h == 0 or w == 0:
            return out
        r, gr, b = (int(c) for c in color)
        _capi.check(_capi.lib().sift_cuda_draw_keypoints(
            self.handle, g.ctypes.data, w, h, g.strides[0], kps.ctypes.data if len(kps) else None, len(kps), r, gr, b,
            out.ctypes.data, 3 * w))
        return out

    # descriptor matching ----------------------------------------------------
    def match(self, query, train) -> np.ndarray:
        """Nearest and second-nearest train descriptor of every query
        descriptor by Euclidean distance (brute force on the GPU, ties to the
        lower index): a MATCH_DTYPE array of len(query) entries. Not in the
        reference crate; the consumer of detect_and_compute's descriptors."""
        q = np.ascontiguousarray(query, dtype=np.float32).reshape(-1, DESC_LEN)
        t = np.ascontiguousarray(train, dtype=np.float32).reshape(-1, DESC_LEN)
        out = np.empty(len(q), dtype=_capi.MATCH_DTYPE)
        if len(q) == 0:
            return out
        _capi.check(_capi.lib().sift_cuda_match(self.handle, q.ctypes.data, len(q), t.ctypes.data if len(t) else None,
                                                len(t), out.ctypes.data))
        return out

    # device-resident form -------------------------------------------------
    def run_device(self, d_img: int, width: int, height: int, stride: int, with_descriptors: bool = True) -> None:
        _capi.check(_capi.lib().sift_cuda_run_device(self.handle, C.c_void_p(d_img), width, height, stride,
                                                     1 if with_descriptors else 0))

    def device_outputs(self) -> tuple[int, int, int]:
        c, k, d = C.c_void_p(), C.c_void_p(), C.c_void_p()
        _capi.check(_capi.lib().sift_cuda_device_outputs(self.handle, C.byref(c), C.byref(k), C.byref(d)))
        return c.value or 0, k.value or 0, d.value or 0

    def synchronize(self) -> None:
        _capi.check(_capi.lib().sift_cuda_synchronize(self.handle))

    @property
    def stream(self) -> int:
        return _capi.lib().sift_cuda_stream(self.handle) or 0

    @property
    def last_launch_count(self) -> int:
        return int(_capi.lib().sift_cuda_last_launch_count(self.handle))

    @property
    def last_image_in_place(self) -> bool:
        """Whether the last host call read the image where the caller keeps it."""
        return bool(_capi.lib().sift_cuda_last_image_in_place(self.handle))

    STAGE_NAMES = ("pyramid_dog", "extrema_refine", "orientation", "descriptor")

    def profile(self, enable: bool) -> None:
        _capi.check(_capi.lib().sift_cuda_profile_enable(self.handle, 1 if enable else 0))

    def profile_read(self) -> tuple[dict, int]:
        """Summed per-stage device milliseconds since the last read, and runs."""
        ms = (C.c_float * 4)()
        runs = C.c_uint32()
        _capi.check(_capi.lib().sift_cuda_profile_read(self.handle, ms, 4, C.byref(runs)))
        return {k: float(ms[i]) for i, k in enumerate(self.STAGE_NAMES)}, int(runs.value)

    def debug_stage(self, stage: int) -> np.ndarray:
        L = _capi.lib()
        n = C.c_uint64()
        _capi.check(L.sift_cuda_debug_stage(self.handle, stage, None, 0, C.byref(n)))
        if stage == _capi.STAGE_PYRAMID:
            out = np.empty(n.value, dtype=np.uint8)
        elif stage in (_capi.STAGE_DOG, _capi.STAGE_DESCRIPTORS):
            out = np.empty(n.value, dtype=np.float32)
        else:
            out = np.empty(n.value, dtype=KEYPOINT_DTYPE)
        _capi.check(L.sift_cuda_debug_stage(self.handle, stage, out.ctypes.data if n.value else None,
                                            n.value, C.byref(n)))
        if stage == _capi.STAGE_DESCRIPTORS:
            out = out.reshape(-1, DESC_LEN)
        return out


class Sift:
    """Sift parameters (src/sift.rs:36-45); contrast_threshold stored / S."""

    _engines: dict = {}
    _lock = threading.RLock()

    def __init__(self, sigma: float = DEFAULT_SIGMA, num_octaves: int = DEFAULT_NUM_OCTAVES,
                 num_intervals: int = DEFAULT_NUM_INTERVALS, assumed_blur: float = DEFAULT_ASSUMED_BLUR,
                 contrast_threshold: float | None = None, edge_threshold: float = DEFAULT_EDGE_THRESHOLD,
                 image_border_width: int = DEFAULT_IMAGE_BORDER_WIDTH):
        self.sigma = float(np.float32(sigma))
        self.num_octaves = int(num_octaves)
        self.num_intervals = int(num_intervals)
        self.assumed_blur = float(np.float32(assumed_blur))
        if contrast_threshold is None:
            contrast_threshold = float(np.float32(DEFAULT_CONTRAST_THRESHOLD) / np.float32(num_intervals))
        self.contrast_threshold = float(np.float32(contrast_threshold))
        self.edge_threshold = float(np.float32(edge_threshold))
        self.image_border_width = int(image_border_width)

    @classmethod
    def default(cls) -> "Sift":
        """Sift::default() (src/sift.rs:47-59)."""
        return cls()

    @classmethod
    def new(cls, sigma: float, num_octaves: int, num_intervals: int, assumed_blur: float,
            contrast_threshold: float, edge_threshold: float) -> "Sift":
        """Sift::new (src/sift.rs:63-80): stores contrast_threshold / num_intervals in f32."""
        c = float(np.float32(contrast_threshold) / np.float32(num_intervals))
        return cls(sigma, num_octaves, num_intervals, assumed_blur, c, edge_threshold)

    def to_c(self) -> _capi.Params:
        return _capi.Params(self.sigma, self.num_octaves, self.num_intervals, self.assumed_blur,
                            self.contrast_threshold, self.edge_threshold, self.image_border_width)

    def _key(self):
        return (self.sigma, self.num_octaves, self.num_intervals, self.assumed_blur,
                self.contrast_threshold, self.edge_threshold, self.image_border_width)

    def _engine(self) -> Engine:
        # One process-wide engine per parameter set (the Rust arm keeps a
        # lazily created global engine behind a mutex).
        with Sift._lock:
            eng = Sift._engines.get(self._key())
            if eng is None:
                eng = Engine(self)
                Sift._engines[self._key()] = eng
            return eng

    def detect_and_compute_with_backend(self, img, backend: SiftBackend):
        """(keypoints, descriptors) like the reference; raises SiftError."""
        if backend is not SiftBackend.Cuda:
            raise SiftError(f"backend {backend.name} is provided by the reference crate, not by this engine")
        try:
            with Sift._lock:
                kps, desc = self._engine().detect_and_compute(img)
        except SiftCudaError as e:
            raise SiftError(f"CUDA detection failed: {e}") from e
        return keypoints_from_array(kps), [list(map(float, d)) for d in desc]

    def detect_and_compute_arrays(self, img, backend: SiftBackend = SiftBackend.Cuda):
        """Same as detect_and_compute_with_backend, as numpy arrays."""
        if backend is not SiftBackend.Cuda:
            raise SiftError(f"backend {backend.name} is provided by the reference crate, not by this engine")
        try:
            with Sift._lock:
                return self._engine().detect_and_compute(img)
        except SiftCudaError as e:
            raise SiftError(f"CUDA detection failed: {e}") from e

    def detect(self, img, backend: SiftBackend = SiftBackend.Cuda) -> list[KeyPoint]:
        """Sift::detect (src/sift.rs:846-886) on the CUDA engine."""
        if backend is not SiftBackend.Cuda:
            raise SiftError(f"backend {backend.name} is provided by the reference crate, not by this engine")
        try:
            with Sift._lock:
                return keypoints_from_array(self._engine().detect(img))
        except SiftCudaError as e:
            raise SiftError(f"CUDA detection failed: {e}") from e


def draw_keypoints_to_image(img, keypoints, color=(255, 0, 0)) -> np.ndarray:
    """draw_keypoints_to_image (src/lib.rs:69-116): the image as RGB with each
    keypoint's circle, orientation line and centre dot in `color`, drawn on
    the GPU by the default engine."""
    with Sift._lock:
        return Sift.default()._engine().draw_keypoints(img, keypoints, color)


class Batch:
    """The batched form (sift_cuda_batch_*): one run over many grayscale
    images of any sizes, each stage one launch over the flattened work of all
    of them, captured as one CUDA graph per batch geometry. Every image's
    result is detect_and_compute's on it, bit for bit. Levels are kept as u8
    planes."""

    def __init__(self, params: "Sift | _capi.Params | None" = None, device: int = 0):
        L = _capi.lib()
        if params is None:
            params = Sift.default()
        p = params.to_c() if isinstance(params, Sift) else params
        opts = _capi.Options()
        L.sift_cuda_options_default(C.byref(opts))
        opts.device = device
        opts.storage = _capi.STORAGE_U8
        h = C.c_void_p()
        _capi.check(L.sift_cuda_batch_create(C.byref(p), C.byref(opts), C.byref(h)))
        self._h = h
        self.last_launch_count = 0
        self.last_device_ms = 0.0
        self.last_images_in_place = False

    def close(self) -> None:
        if getattr(self, "_h", None):
            _capi.lib().sift_cuda_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def detect_and_compute(self, images, copy: bool = True) -> list[tuple[np.ndarray, np.ndarray]]:
        """(keypoints, descriptors) per image, in input order. copy=False
        returns views of the batch's host buffers, valid until its next call."""
        if not self._h:
            raise SiftError("batch is closed")
        imgs = []
        for img in images:
            g = _as_gray(img)
            if g.strides[1] != 1:
                g = np.ascontiguousarray(g)
            imgs.append(g)
        n = len(imgs)
        arr = (_capi.BatchImage * max(n, 1))()
        for i, g in enumerate(imgs):
            arr[i].data = g.ctypes.data if g.size else None
            arr[i].width = g.shape[1]
            arr[i].height = g.shape[0]
            arr[i].stride = g.strides[0] if g.size else g.shape[1]
        res = _capi.BatchResult()
        _capi.check(_capi.lib().sift_cuda_batch_detect_and_compute(self._h, arr, n, C.byref(res)))
        self.last_launch_count = res.launches
        self.last_device_ms = float(res.device_ms)
        self.last_images_in_place = bool(res.images_in_place)
        if n == 0:
            return []
        off = np.ctypeslib.as_array(res.offsets, shape=(n + 1,)).copy()
        total = int(res.total)
        if total:
            kbuf = (C.c_char * (total * KEYPOINT_DTYPE.itemsize)).from_address(res.kps)
            dbuf = (C.c_char * (total * DESC_LEN * 4)).from_address(res.desc)
            kall = np.frombuffer(kbuf, dtype=KEYPOINT_DTYPE, count=total)
            dall = np.frombuffer(dbuf, dtype=np.float32, count=total * DESC_LEN).reshape(total, DESC_LEN)
        else:
            kall = np.empty(0, KEYPOINT_DTYPE)
            dall = np.empty((0, DESC_LEN), np.float32)
        out = []
        for i in range(n):
            k, d = kall[off[i]:off[i + 1]], dall[off[i]:off[i + 1]]
            out.append((k.copy(), d.copy()) if copy else (k, d))
        return out
