"""Errors of a storage mode's outputs against the FP64 ideal model
(oracle/ideal64.py): DoG values, keypoint positions, sizes and angles, and
descriptors. Keypoints are paired greedily by position within one
octave-pixel in the same octave, then by nearest angle; descriptors are
compared on pairs whose angles agree within 5 degrees.
"""
from __future__ import annotations

import math

import numpy as np


def dog_errors(dog_stage: np.ndarray, octave_dims, ideal_dog) -> list[dict]:
    """dog_stage: the engine's DoG levels concatenated octave-major, level,
    row-major (STAGE_DOG); ideal_dog[o][l] float64 planes."""
    out, off = [], 0
    for o, (w, h) in enumerate(octave_dims):
        n = w * h
        errs = []
        for lv in ideal_dog[o]:
            got = dog_stage[off: off + n].reshape(h, w).astype(np.float64)
            errs.append(got - lv)
            off += n
        e = np.stack(errs)
        out.append({"octave": o, "max_abs": float(np.abs(e).max()), "rms": float(np.sqrt((e * e).mean())),
                    "mean": float(e.mean())})
    return out


def keypoint_errors(kps, desc, ideal_kps, ideal_desc) -> dict:
    pairs = []
    used = set()
    for i in range(len(ideal_kps)):
        o = int(ideal_kps["octave"][i])
        scale = 2.0 ** o
        same = np.nonzero(kps["octave"] == o)[0]
        if len(same) == 0:
            continue
        d = np.hypot(kps["x"][same] - ideal_kps["x"][i], kps["y"][same] - ideal_kps["y"][i]) / scale
        near = same[d <= 1.0]
        if len(near) == 0:
            continue
        da = np.abs((kps["angle"][near] - ideal_kps["angle"][i] + math.pi) % (2 * math.pi) - math.pi)
        order = np.argsort(da)
        for j in near[order]:
            if int(j) not in used:
                used.add(int(j))
                pairs.append((i, int(j)))
                break
    res = {"ideal_keypoints": int(len(ideal_kps)), "keypoints": int(len(kps)), "paired": len(pairs),
           "paired_fraction_of_ideal": len(pairs) / max(len(ideal_kps), 1)}
    if pairs:
        ii = np.array([p[0] for p in pairs])
        jj = np.array([p[1] for p in pairs])
        pos = np.hypot(kps["x"][jj] - ideal_kps["x"][ii], kps["y"][jj] - ideal_kps["y"][ii])
        size = np.abs(kps["size"][jj] - ideal_kps["size"][ii]) / ideal_kps["size"][ii]
        ang = np.abs((kps["angle"][jj] - ideal_kps["angle"][ii] + math.pi) % (2 * math.pi) - math.pi)
        res.update({"position_px_median": float(np.median(pos)), "position_px_p95": float(np.percentile(pos, 95)),
                    "size_rel_median": float(np.median(size)), "size_rel_p95": float(np.percentile(size, 95)),
                    "angle_deg_median": float(np.degrees(np.median(ang))),
                    "angle_deg_p95": float(np.degrees(np.percentile(ang, 95)))})
        close = ang <= math.radians(5.0)
        if close.any():
            a, b = desc[jj[close]].astype(np.float64), ideal_desc[ii[close]]
            rel = np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-12)
            res.update({"descriptor_pairs": int(close.sum()), "descriptor_rel_l2_median": float(np.median(rel)),
                        "descriptor_rel_l2_p95": float(np.percentile(rel, 95))})
    return res
