"""The batched form (sift_cuda_batch_*, csrc/batch.cu) against the
single-image engine (GPU): one run over images of uneven sizes, each stage one
launch over the flattened work of all of them, gives every image the
keypoints and descriptors of detect_and_compute on it, bit for bit and in the
same order (the single-image engine's results are the ones the oracle parity
tests check)."""
import numpy as np
import pytest
from synthetic import batch64_shapes, synth_image

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sgb(built_lib):
    import sift_wgpu_gb300
    return sift_wgpu_gb300


def same(a, b):
    return a[0].tobytes() == b[0].tobytes() and a[1].tobytes() == b[1].tobytes()


def uneven_images():
    shapes = [(640, 480), (333, 217), (1920, 1080), (64, 3), (20, 15), (1, 1), (0, 0), (96, 80), (1280, 720)]
    imgs = [synth_image(500 + i, w, h) for i, (w, h) in enumerate(shapes)]
    imgs[4] = np.tile((np.arange(20) * 10).astype(np.uint8), (15, 1))  # tests/integration_test.rs:166-203
    imgs.append(np.full((100, 100), 128, np.uint8))  # tests/integration_test.rs:205-226: no keypoints
    return imgs


def test_batch_equals_single_engine(sgb):
    imgs = uneven_images()
    with sgb.Engine(sgb.Sift.default(), storage="u8") as eng:
        alone = [eng.detect_and_compute(im) for im in imgs]
    with sgb.Batch(sgb.Sift.default()) as b:
        got = b.detect_and_compute(imgs)
        assert len(got) == len(imgs)
        for i, (g, a) in enumerate(zip(got, alone)):
            assert same(g, a), f"image {i} {imgs[i].shape}: {len(g[0])} vs {len(a[0])} keypoints"
        assert sum(len(k) for k, _ in got) > 1000
        assert len(got[-1][0]) == 0  # the uniform image
        # the same geometry again (graph replay), then another geometry, then back
        again = b.detect_and_compute(imgs)
        assert all(same(g, a) for g, a in zip(again, alone))
        two = b.detect_and_compute([imgs[2], imgs[0]])
        assert same(two[0], alone[2]) and same(two[1], alone[0])
        views = b.detect_and_compute(imgs, copy=False)
        assert all(same(g, a) for g, a in zip(views, alone))
        assert b.last_launch_count > 0
        assert b.detect_and_compute([]) == []


def test_images_in_place_and_copied_agree(sgb):
    """Images that start and stride on 16 bytes are read where they are on a
    device that reads pageable host memory (a GB300 with its Grace host); the
    same images with a 1-byte wider stride go through the device copy. Both
    runs give the same results."""
    import torch
    imgs = [synth_image(700 + i, w, h) for i, (w, h) in enumerate([(640, 480), (1280, 720), (512, 1024)])]
    padded = []
    for im in imgs:
        h, w = im.shape
        buf = np.zeros((h, w + 1), np.uint8)
        buf[:, :w] = im
        padded.append(buf[:, :w])  # stride w + 1
    with sgb.Batch(sgb.Sift.default()) as b:
        a = b.detect_and_compute(imgs)
        in_place = b.last_images_in_place
        c = b.detect_and_compute(padded)
        assert not b.last_images_in_place
    assert all(same(x, y) for x, y in zip(a, c))
    assert sum(len(k) for k, _ in a) > 100
    if "GB300" in torch.cuda.get_device_name(0):  # Grace host: pageable memory is device-readable
        assert in_place


def test_batch64_sample_with_six_octaves(sgb):
    """Twelve images of the uneven 64-image batch (the smallest, the largest,
    the most elongated and nine more) under Sift::new(1.6, 6, 3, 0.5, 0.04,
    10.0): octaves of a few pixels, radii wider than the planes."""
    shapes = batch64_shapes()
    area = [w * h for w, h in shapes]
    elong = [max(w / h, h / w) for w, h in shapes]
    pick = []
    for i in [int(np.argmin(area)), int(np.argmax(area)), int(np.argmax(elong))] + list(range(9)):
        if i not in pick:
            pick.append(i)
    imgs = [synth_image(1000 + i, *shapes[i]) for i in pick]
    params = sgb.Sift.new(1.6, 6, 3, 0.5, 0.04, 10.0)
    with sgb.Engine(params, storage="u8") as eng:
        alone = [eng.detect_and_compute(im) for im in imgs]
    with sgb.Batch(params) as b:
        got = b.detect_and_compute(imgs)
    for i, (g, a) in enumerate(zip(got, alone)):
        assert same(g, a), f"image {pick[i]} {shapes[pick[i]]}"


def test_batch_rejects_other_storage(sgb):
    import ctypes as C
    from sift_wgpu_gb300 import _capi
    L = _capi.lib()
    p = sgb.Sift.default().to_c()
    o = _capi.Options()
    L.sift_cuda_options_default(C.byref(o))
    o.storage = _capi.STORAGE_F32
    h = C.c_void_p()
    assert L.sift_cuda_batch_create(C.byref(p), C.byref(o), C.byref(h)) == 6  # SIFT_CUDA_ERR_UNSUPPORTED
