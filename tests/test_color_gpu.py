"""Colour input converted to luma on the device (GPU): the conversion kernel
against the oracle's restatement, bit for bit, and the pipeline on a colour
image against the pipeline on its host-converted luma."""
import ctypes as C

import numpy as np
import pytest
from synthetic import synth_image

pytestmark = pytest.mark.gpu

FORMATS = [(1, 3), (2, 4), (3, 4)]  # (SIFT_CUDA_PIXELS_*, channels)


@pytest.fixture(scope="module")
def sgb(built_lib):
    import sift_wgpu_gb300
    return sift_wgpu_gb300


@pytest.mark.parametrize("fmt,ch", FORMATS)
@pytest.mark.parametrize("shape", [(1, 1), (7, 13), (480, 641), (1080, 1920)])
def test_to_luma_kernel_matches_oracle(sgb, oracle_mod, fmt, ch, shape):
    import torch
    h, w = shape
    px = np.random.default_rng(h * 7 + w + fmt).integers(0, 256, size=(h, w, ch), dtype=np.uint8)
    stride = w * ch + 24  # a padded row
    buf = np.zeros((h, stride), np.uint8)
    buf[:, : w * ch] = px.reshape(h, w * ch)
    d_px = torch.from_numpy(buf).cuda()
    d_out = torch.full((h, w + 5), 77, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    L = sgb._capi.lib()
    rc = L.sift_cuda_to_luma(C.c_void_p(d_px.data_ptr()), w, h, stride, fmt, C.c_void_p(d_out.data_ptr()), w + 5,
                             None)
    assert rc == 0, L.sift_cuda_last_error()
    torch.cuda.synchronize()
    got = d_out.cpu().numpy()
    assert np.array_equal(got[:, :w], oracle_mod.luma_u8(px, fmt))
    assert np.all(got[:, w:] == 77)


@pytest.mark.parametrize("fmt,ch", FORMATS)
def test_colour_pipeline_equals_luma_pipeline(sgb, oracle_mod, fmt, ch):
    gray = synth_image(11, 640, 480)
    rng = np.random.default_rng(fmt)
    # a colour image whose channels differ, alpha random
    px = np.stack([gray, np.roll(gray, 3, axis=1), np.roll(gray, 5, axis=0)]
                  + ([rng.integers(0, 256, gray.shape, dtype=np.uint8)] if ch == 4 else []), axis=-1)
    with sgb.Engine(sgb.Sift.default()) as eng:
        k1, d1 = eng.detect_and_compute_pixels(px, fmt)
        k2, d2 = eng.detect_and_compute(oracle_mod.luma_u8(px, fmt))
        if fmt != 3:
            k3, d3 = eng.detect_and_compute(px)  # H x W x C arrays take the to_luma8 path
            assert k3.tobytes() == k1.tobytes() and d3.tobytes() == d1.tobytes()
    assert len(k1) > 0
    assert k1.tobytes() == k2.tobytes() and d1.tobytes() == d2.tobytes()
