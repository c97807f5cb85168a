"""Precision statement: the three storage modes against the FP64 ideal model
(GPU).

F32 storage keeps Gaussian levels as f32 (v/255), F16 storage as f16 (v), U8
storage keeps only the u8 level planes; all three form every DoG value in
f32 from the u8 level planes. All hold the reference's u8-quantised levels
exactly, so their outputs are bit-identical and their errors against the
FP64 model (no u8 rounding; oracle/ideal64.py) are the reference CPU path's
own. The test prints the statement and checks that the modes give the same
numbers.
"""
import json

import numpy as np
import pytest

from precision import dog_errors, keypoint_errors
from synthetic import synth_image

pytestmark = pytest.mark.gpu


def test_precision_statement(built_lib, oracle_mod):
    import sift_wgpu_gb300 as sg
    from oracle.ideal64 import Ideal64
    img = synth_image(0, 512, 512)
    k64, d64, pyr64, dog64 = Ideal64().detect_and_compute(img)
    dims = [(lv[0].shape[1], lv[0].shape[0]) for lv in pyr64]
    report = {"image": "512x512 synthetic, seed 0, Sift::default()"}
    outs = {}
    for storage in ("f32", "f16", "u8"):
        with sg.Engine(sg.Sift.default(), storage=storage) as eng:
            kps, desc = eng.detect_and_compute(img)
            dog = eng.debug_stage(sg.STAGE_DOG)
        outs[storage] = (kps, desc, dog)
        report[storage] = {"dog": dog_errors(dog, dims, dog64), "keypoints": keypoint_errors(kps, desc, k64, d64)}
    print(json.dumps(report, indent=1))
    k32, dsc32, dog32 = outs["f32"]
    for storage in ("f16", "u8"):
        k, dsc, dog = outs[storage]
        assert k.tobytes() == k32.tobytes() and dsc.tobytes() == dsc32.tobytes(), storage
        assert np.array_equal(dog, dog32), storage
    # the u8 truncation of every blur pass makes the levels darker, the DoG
    # biased negative by about 1/255 per level
    for row in report["f32"]["dog"]:
        assert -0.02 < row["mean"] <= 0.0
    assert report["f32"]["keypoints"]["paired"] > 0
