"""Brute-force descriptor matching on the CPU: the oracle of the engine's
sift_cuda_match (test infrastructure only; the product path is the CUDA
kernel in sift_wgpu_gb300/csrc/match.cu).

Matching is not part of the reference crate (stevel705/sift-wgpu); it is the
consumer of the 128-float descriptors that Sift::detect_and_compute returns
(src/sift.rs:1244-1355). The restated algorithm is the textbook one behind
Lowe's ratio test: for every query descriptor, the train descriptors with the
smallest and second-smallest Euclidean distance, ties to the lower index.
Distances are computed here in float64 from the float32 descriptors.
"""
from __future__ import annotations

import numpy as np

MATCH_FIELDS = ("train_idx", "distance", "second_idx", "second_distance")


def match(query: np.ndarray, train: np.ndarray, chunk: int = 2048):
    """Returns (d2 sorted pairs) as four arrays: train_idx, distance,
    second_idx, second_distance (index -1 and distance inf when absent), and
    the squared distance of the third nearest (inf if absent), which the
    tests use to skip near-ties."""
    q = np.asarray(query, dtype=np.float64).reshape(-1, 128)
    t = np.asarray(train, dtype=np.float64).reshape(-1, 128)
    nq, nt = len(q), len(t)
    idx = np.full((nq, 3), -1, dtype=np.int64)
    d2 = np.full((nq, 3), np.inf)
    tn = (t * t).sum(1)
    for a in range(0, nq, chunk):
        qa = q[a:a + chunk]
        if nt == 0:
            continue
        d = (qa * qa).sum(1)[:, None] + tn[None, :] - 2.0 * qa @ t.T
        k = min(3, nt)
        # stable sort on (distance, index): ties go to the lower index
        order = np.argsort(d, axis=1, kind="stable")[:, :k]
        idx[a:a + chunk, :k] = order
        d2[a:a + chunk, :k] = np.take_along_axis(d, order, axis=1)
    dist = np.sqrt(np.maximum(d2, 0.0))
    return idx[:, 0], dist[:, 0], idx[:, 1], dist[:, 1], d2[:, 2], d2
