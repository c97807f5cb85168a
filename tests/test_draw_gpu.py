"""draw_keypoints_to_image (src/lib.rs:69-116) on the GPU
(sift_cuda_draw_keypoints, csrc/draw.cu) against the CPU oracle
(oracle/draw.py), through the C ABI: bit-exact RGB images."""
import numpy as np
import pytest
from synthetic import synth_image

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sgb(built_lib):
    import sift_wgpu_gb300
    return sift_wgpu_gb300


def test_detected_keypoints_bit_exact(sgb):
    from oracle.draw import draw_keypoints_to_image
    img = synth_image(0, 512, 512)
    with sgb.Engine(sgb.Sift.default()) as eng:
        kps, _ = eng.detect_and_compute(img)
        got = eng.draw_keypoints(img, kps, (255, 0, 0))
    want = draw_keypoints_to_image(img, kps, (255, 0, 0))
    assert got.shape == (512, 512, 3)
    assert np.array_equal(got, want), f"{np.count_nonzero(np.any(got != want, axis=2))} pixels differ"
    assert np.count_nonzero(np.all(got == [255, 0, 0], axis=2)) > 10000


def test_borders_angles_and_strides(sgb):
    """Keypoints on and beyond the image border, every axis and diagonal
    angle, a padded input stride; the module-level function of the API."""
    from oracle.draw import draw_keypoints_to_image
    rng = np.random.default_rng(2)
    base = rng.integers(0, 256, size=(97, 131), dtype=np.uint8)
    padded = np.zeros((97, 160), np.uint8)
    padded[:, :131] = base
    view = padded[:, :131]
    kps = np.zeros(40, sgb.KEYPOINT_DTYPE)
    kps["x"] = np.concatenate([[0.0, 130.9, -3.5, 135.2, 65.5], rng.uniform(-8, 139, 35)])
    kps["y"] = np.concatenate([[0.0, 96.9, 50.0, -7.0, 101.0], rng.uniform(-8, 105, 35)])
    kps["angle"] = np.concatenate([np.arange(8) * (np.pi / 4), rng.uniform(0, 2 * np.pi, 32)]).astype(np.float32)
    got = sgb.draw_keypoints_to_image(view, kps, (10, 200, 30))
    want = draw_keypoints_to_image(base, kps, (10, 200, 30))
    assert np.array_equal(got, want), f"{np.count_nonzero(np.any(got != want, axis=2))} pixels differ"
    kl = sgb.keypoints_from_array(kps[:5])
    assert np.array_equal(sgb.draw_keypoints_to_image(base, kl, (1, 2, 3)),
                          draw_keypoints_to_image(base, kps[:5], (1, 2, 3)))
    empty = sgb.draw_keypoints_to_image(base, kps[:0])
    assert np.array_equal(empty, np.repeat(base[:, :, None], 3, axis=2))
