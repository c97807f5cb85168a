"""ctypes binding of libsiftcuda.so (include/sift_cuda.h).

The library is built in-tree by ``sift_wgpu_gb300.build_ext.build()``; loading
fails loudly when it is missing — there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libsiftcuda.so"

DESC_LEN = 128

STATUS = {
    0: "OK",
    1: "INVALID_ARGUMENT",
    2: "CUDA",
    3: "OUT_OF_MEMORY",
    4: "CAPACITY",
    5: "NO_DEVICE",
    6: "UNSUPPORTED",
}

STORAGE_F32 = 0
STORAGE_F16 = 1
STORAGE_U8 = 2

PIXELS_GRAY8 = 0
PIXELS_RGB8 = 1
PIXELS_RGBA8 = 2
PIXELS_RGBA8_CANVAS = 3

STAGE_PYRAMID = 0
STAGE_CANDIDATES = 1
STAGE_REFINED = 2
STAGE_DOG = 3
STAGE_KEYPOINTS = 4
STAGE_DESCRIPTORS = 5


class Params(C.Structure):
    _fields_ = [
        ("sigma", C.c_float),
        ("num_octaves", C.c_uint32),
        ("num_intervals", C.c_uint32),
        ("assumed_blur", C.c_float),
        ("contrast_threshold", C.c_float),
        ("edge_threshold", C.c_float),
        ("image_border_width", C.c_uint32),
    ]


class Options(C.Structure):
    _fields_ = [("device", C.c_int32), ("storage", C.c_int32), ("level_tile_rows", C.c_int32),
                ("reserved", C.c_uint32 * 5)]


class Keypoint(C.Structure):
    _fields_ = [
        ("x", C.c_float),
        ("y", C.c_float),
        ("size", C.c_float),
        ("angle", C.c_float),
        ("response", C.c_float),
        ("octave", C.c_int32),
        ("layer", C.c_int32),
    ]


class Result(C.Structure):
    _fields_ = [("n", C.c_uint32), ("kps", C.POINTER(Keypoint)), ("desc", C.POINTER(C.c_float))]


# numpy view of SiftCudaKeypoint / OracleKeypoint (28 bytes, packed C layout)
KEYPOINT_DTYPE = np.dtype(
    [("x", "<f4"), ("y", "<f4"), ("size", "<f4"), ("angle", "<f4"), ("response", "<f4"),
     ("octave", "<i4"), ("layer", "<i4")]
)
assert KEYPOINT_DTYPE.itemsize == C.sizeof(Keypoint) == 28

# numpy view of SiftCudaMatch (16 bytes)
MATCH_DTYPE = np.dtype([("train_idx", "<i4"), ("distance", "<f4"), ("second_idx", "<i4"), ("second_distance", "<f4")])

_lib = None


class SiftCudaError(RuntimeError):
    """A failed call into libsiftcuda.so (the reference's Err(String))."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{STATUS.get(code, code)}: {message}")
        self.code = code


class ServerOptions(C.Structure):
    _fields_ = [("device", C.c_int32), ("storage", C.c_int32), ("arena_bytes", C.c_uint64),
                ("max_inflight", C.c_uint32), ("autotune", C.c_uint32), ("reserved", C.c_uint32 * 4)]


class Served(C.Structure):
    _fields_ = [("ticket", C.c_uint64), ("tag", C.c_uint64), ("status", C.c_int32), ("n", C.c_uint32),
                ("kps", C.c_void_p), ("desc", C.c_void_p), ("submit_s", C.c_double), ("start_s", C.c_double),
                ("done_s", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("slots", C.c_uint32), ("running", C.c_uint32), ("pending", C.c_uint32), ("reserved", C.c_uint32),
                ("device_bytes", C.c_uint64), ("completed", C.c_uint64), ("reruns", C.c_uint64),
                ("evicted", C.c_uint64), ("max_pending", C.c_uint64)]


class ReplayImage(C.Structure):
    _fields_ = [("data", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32), ("stride", C.c_uint32),
                ("reserved", C.c_uint32)]


class BatchImage(C.Structure):
    _fields_ = [("data", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32), ("stride", C.c_uint32),
                ("reserved", C.c_uint32)]


class BatchResult(C.Structure):
    _fields_ = [("n_images", C.c_uint32), ("total", C.c_uint32), ("offsets", C.POINTER(C.c_uint32)),
                ("kps", C.c_void_p), ("desc", C.c_void_p), ("launches", C.c_uint32), ("device_ms", C.c_float),
                ("images_in_place", C.c_uint32)]


class ReplayRequest(C.Structure):
    _fields_ = [("arrival_s", C.c_double), ("image", C.c_uint32), ("reserved", C.c_uint32)]


class ReplayResult(C.Structure):
    _fields_ = [("latency_s", C.c_double), ("n", C.c_uint32), ("status", C.c_int32)]


SUBMIT_BORROW = 1


def lib() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH} is missing: build it with sift_wgpu_gb300.build_ext.build() "
            "(the CUDA engine has no CPU fallback)"
        )
    L = C.CDLL(str(LIB_PATH))
    P = C.POINTER
    u32, i32, f32, u64 = C.c_uint32, C.c_int32, C.c_float, C.c_uint64
    sig = {
        "sift_cuda_params_default": (None, [P(Params)]),
        "sift_cuda_params_new": (None, [P(Params), f32, u32, u32, f32, f32, f32]),
        "sift_cuda_options_default": (None, [P(Options)]),
        "sift_cuda_create": (C.c_int, [P(Params), P(Options), P(C.c_void_p)]),
        "sift_cuda_destroy": (None, [C.c_void_p]),
        "sift_cuda_detect_and_compute": (C.c_int, [C.c_void_p, C.c_void_p, u32, u32, u32, P(Result)]),
        "sift_cuda_detect": (C.c_int, [C.c_void_p, C.c_void_p, u32, u32, u32, P(Result)]),
        "sift_cuda_detect_and_compute_view": (C.c_int, [C.c_void_p, C.c_void_p, u32, u32, u32, P(Result)]),
        "sift_cuda_detect_and_compute_pixels": (C.c_int, [C.c_void_p, C.c_void_p, u32, u32, u32, i32, P(Result)]),
        "sift_cuda_to_luma": (C.c_int, [C.c_void_p, u32, u32, u32, i32, C.c_void_p, u32, C.c_void_p]),
        "sift_cuda_result_free": (None, [P(Result)]),
        "sift_cuda_last_error": (C.c_char_p, []),
        "sift_cuda_run_device": (C.c_int, [C.c_void_p, C.c_void_p, u32, u32, u32, C.c_int]),
        "sift_cuda_device_outputs": (C.c_int, [C.c_void_p, P(C.c_void_p), P(C.c_void_p), P(C.c_void_p)]),
        "sift_cuda_synchronize": (C.c_int, [C.c_void_p]),
        "sift_cuda_stream": (C.c_void_p, [C.c_void_p]),
        "sift_cuda_debug_stage": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, u64, P(u64)]),
        "sift_cuda_last_launch_count": (u32, [C.c_void_p]),
        "sift_cuda_last_image_in_place": (u32, [C.c_void_p]),
        "sift_cuda_profile_enable": (C.c_int, [C.c_void_p, C.c_int]),
        "sift_cuda_profile_read": (C.c_int, [C.c_void_p, P(f32), u32, P(u32)]),
        "sift_cuda_gaussian_blur_u8_noalloc": (C.c_int, [C.c_void_p, u32, u32, u32, C.c_void_p, u32, f32,
                                                         C.c_void_p]),
        "sift_cuda_server_options_default": (None, [P(ServerOptions)]),
        "sift_cuda_server_create": (C.c_int, [P(Params), P(ServerOptions), P(C.c_void_p)]),
        "sift_cuda_server_destroy": (None, [C.c_void_p]),
        "sift_cuda_server_submit": (C.c_int, [C.c_void_p, C.c_void_p, u32, u32, u32, u64, u32, P(u64)]),
        "sift_cuda_server_poll": (C.c_int, [C.c_void_p, P(Served), C.c_int64]),
        "sift_cuda_server_release": (C.c_int, [C.c_void_p, u64]),
        "sift_cuda_server_warm": (C.c_int, [C.c_void_p, C.c_void_p, u32, u32, u32, u32]),
        "sift_cuda_server_stats": (C.c_int, [C.c_void_p, P(ServerStats)]),
        "sift_cuda_server_tuning": (C.c_int, [C.c_void_p, u32, u32, P(i32)]),
        "sift_cuda_server_tuning_knobs": (C.c_int, [C.c_void_p, u32, u32, P(i32), u32]),
        "sift_cuda_footprint_bytes": (u64, [P(Params), i32, u32, u32]),
        "sift_cuda_replay": (C.c_int, [C.c_void_p, P(Params), P(Options), P(ReplayImage), u32, P(ReplayRequest),
                                       u32, P(ReplayResult), P(C.c_double)]),
        "sift_cuda_draw_keypoints": (C.c_int, [C.c_void_p, C.c_void_p, u32, u32, u32, C.c_void_p, u32, C.c_uint8,
                                               C.c_uint8, C.c_uint8, C.c_void_p, u32]),
        "sift_cuda_match": (C.c_int, [C.c_void_p, C.c_void_p, u32, C.c_void_p, u32, C.c_void_p]),
        "sift_cuda_match_scratch_bytes": (C.c_size_t, [u32, u32]),
        "sift_cuda_batch_create": (C.c_int, [P(Params), P(Options), P(C.c_void_p)]),
        "sift_cuda_batch_destroy": (None, [C.c_void_p]),
        "sift_cuda_batch_detect_and_compute": (C.c_int, [C.c_void_p, P(BatchImage), u32, P(BatchResult)]),
        "sift_cuda_match_device": (C.c_int, [C.c_void_p, u32, C.c_void_p, u32, C.c_void_p, C.c_void_p, C.c_void_p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def exported_symbols() -> list[str]:
    """Names declared in include/sift_cuda.h that the loaded library must export."""
    return [
        "sift_cuda_params_default", "sift_cuda_params_new", "sift_cuda_options_default",
        "sift_cuda_create", "sift_cuda_destroy", "sift_cuda_detect_and_compute", "sift_cuda_detect",
        "sift_cuda_detect_and_compute_view", "sift_cuda_detect_and_compute_pixels", "sift_cuda_to_luma",
        "sift_cuda_result_free", "sift_cuda_last_error", "sift_cuda_run_device",
        "sift_cuda_device_outputs", "sift_cuda_synchronize", "sift_cuda_stream",
        "sift_cuda_debug_stage", "sift_cuda_last_launch_count", "sift_cuda_last_image_in_place", "sift_cuda_profile_enable",
        "sift_cuda_profile_read", "sift_cuda_server_options_default", "sift_cuda_server_create",
        "sift_cuda_server_destroy", "sift_cuda_server_submit", "sift_cuda_server_poll", "sift_cuda_server_release",
        "sift_cuda_server_warm", "sift_cuda_server_stats", "sift_cuda_server_tuning",
        "sift_cuda_server_tuning_knobs", "sift_cuda_footprint_bytes",
        "sift_cuda_replay", "sift_cuda_gaussian_blur_u8_noalloc", "sift_cuda_draw_keypoints", "sift_cuda_match",
        "sift_cuda_match_scratch_bytes",
        "sift_cuda_match_device", "sift_cuda_batch_create", "sift_cuda_batch_destroy",
        "sift_cuda_batch_detect_and_compute",
    ]


def check(rc: int) -> None:
    if rc != 0:
        raise SiftCudaError(rc, lib().sift_cuda_last_error().decode(errors="replace"))
