"""Keypoint matching between the CUDA engine and the oracle.

The parity bar: at least 99.5% of the oracle's keypoints match 1:1 a CUDA
keypoint of the same octave within 0.01 px in x and y, 1e-3 relative size and
0.5 degrees of angle; matched descriptors agree within 1e-3 relative L2.
"""
from __future__ import annotations

import math
from collections import defaultdict
from dataclasses import dataclass, field

import numpy as np

POS_TOL = 0.01
SIZE_RTOL = 1e-3
ANGLE_TOL = math.radians(0.5)
DESC_RTOL = 1e-3
MATCH_RATE = 0.995


@dataclass
class Match:
    n_ref: int
    n_got: int
    pairs: list = field(default_factory=list)
    unmatched_ref: list = field(default_factory=list)
    unmatched_got: list = field(default_factory=list)
    desc_err: np.ndarray | None = None
    same_order: bool = False

    @property
    def rate(self) -> float:
        return len(self.pairs) / self.n_ref if self.n_ref else 1.0

    def summary(self) -> str:
        worst = float(self.desc_err.max()) if self.desc_err is not None and len(self.desc_err) else 0.0
        return (f"ref={self.n_ref} got={self.n_got} matched={len(self.pairs)} rate={self.rate:.5f} "
                f"same_order={self.same_order} worst_desc_rel_l2={worst:.2e} "
                f"unmatched_ref={len(self.unmatched_ref)} unmatched_got={len(self.unmatched_got)}")


def _angle_diff(a, b):
    d = abs(float(a) - float(b)) % (2 * math.pi)
    return min(d, 2 * math.pi - d)


def _ok(r, g):
    return (int(r["octave"]) == int(g["octave"])
            and abs(float(r["x"]) - float(g["x"])) <= POS_TOL
            and abs(float(r["y"]) - float(g["y"])) <= POS_TOL
            and abs(float(r["size"]) - float(g["size"])) <= SIZE_RTOL * abs(float(r["size"]))
            and _angle_diff(r["angle"], g["angle"]) <= ANGLE_TOL)


def match(ref_k, ref_d, got_k, got_d) -> Match:
    m = Match(len(ref_k), len(got_k))
    cell = 0.05
    grid = defaultdict(list)
    for j, g in enumerate(got_k):
        grid[(int(math.floor(g["x"] / cell)), int(math.floor(g["y"] / cell)))].append(j)
    used = np.zeros(len(got_k), dtype=bool)
    for i, r in enumerate(ref_k):
        cx, cy = int(math.floor(r["x"] / cell)), int(math.floor(r["y"] / cell))
        best = None
        # prefer the same index (identical order), then the nearest angle
        if i < len(got_k) and not used[i] and _ok(r, got_k[i]):
            best = i
        else:
            cands = []
            for dx in (-1, 0, 1):
                for dy in (-1, 0, 1):
                    for j in grid.get((cx + dx, cy + dy), ()):
                        if not used[j] and _ok(r, got_k[j]):
                            cands.append((_angle_diff(r["angle"], got_k[j]["angle"]), j))
            if cands:
                best = min(cands)[1]
        if best is None:
            m.unmatched_ref.append(i)
        else:
            used[best] = True
            m.pairs.append((i, best))
    m.unmatched_got = [j for j in range(len(got_k)) if not used[j]]
    m.same_order = len(ref_k) == len(got_k) and all(i == j for i, j in m.pairs) and not m.unmatched_ref
    if ref_d is not None and got_d is not None and m.pairs:
        ii = np.array([p[0] for p in m.pairs])
        jj = np.array([p[1] for p in m.pairs])
        a, b = ref_d[ii].astype(np.float64), got_d[jj].astype(np.float64)
        m.desc_err = np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(a, axis=1), 1e-12)
    return m
