"""Writes tests/golden/oracle_256_seed0.npz: a 256 x 256 synthetic image
(synthetic.synth_image, seed 0, the 512 x 512 density) and the oracle's keypoints
and descriptors for it under Sift::default().

    python tests/golden/make_oracle_fixtures.py

The fixture freezes the oracle's output so that a change of the oracle shows
up as a test failure on its own, and gives the GPU tests a committed target.
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

OUT = Path(__file__).resolve().parent / "oracle_256_seed0.npz"


def main() -> None:
    from oracle import oracle
    from synthetic import synth_image
    img = synth_image(0, 256, 256)
    kps, desc = oracle.detect_and_compute(img)
    np.savez_compressed(OUT, image=img, keypoints=kps, descriptors=desc.astype(np.float32))
    print(f"{OUT.name}: {len(kps)} keypoints")


if __name__ == "__main__":
    main()
