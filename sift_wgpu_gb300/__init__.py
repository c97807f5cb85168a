"""GB300 (sm_103a) SIFT engine: a CUDA drop-in for the reference crate's
Sift::detect_and_compute_with_backend, behind the C ABI of include/sift_cuda.h."""
from ._capi import (DESC_LEN, KEYPOINT_DTYPE, MATCH_DTYPE, STAGE_CANDIDATES, STAGE_DESCRIPTORS, STAGE_DOG, STAGE_KEYPOINTS,
                    STAGE_PYRAMID, STAGE_REFINED, SiftCudaError)
from .serve import Served, Server, footprint_bytes, replay
from .sift import Batch, Engine, KeyPoint, Sift, SiftBackend, SiftError, draw_keypoints_to_image, keypoints_from_array

__all__ = [
    "DESC_LEN", "KEYPOINT_DTYPE", "MATCH_DTYPE", "STAGE_CANDIDATES", "STAGE_DESCRIPTORS", "STAGE_DOG", "STAGE_KEYPOINTS",
    "STAGE_PYRAMID", "STAGE_REFINED",
    "Batch", "Engine", "KeyPoint", "Served", "Server", "Sift", "SiftBackend", "SiftCudaError", "SiftError",
    "draw_keypoints_to_image", "footprint_bytes", "keypoints_from_array", "replay",
]
