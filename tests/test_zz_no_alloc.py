"""sift_cuda_gaussian_blur_u8_noalloc through the C ABI (GPU tests).

The blur that allocates nothing must give the levels the engine's own
pyramid holds: the base level of detect_and_compute (imageproc
gaussian_blur_f32 of the input, src/sift.rs:1200-1214) and each level blurred
from the one below it (src/sift.rs:129-177), u8 for u8 — on two calls in a
row. The file name sorts last so the tests also run after everything else in
the suite has used the device.
"""
import ctypes as C

import numpy as np
import pytest
from synthetic import synth_image

pytestmark = pytest.mark.gpu

ERR_UNSUPPORTED = 6


@pytest.fixture(scope="module")
def sgb(built_lib):
    import sift_wgpu_gb300
    return sift_wgpu_gb300


def blur_noalloc(lib, src, dst, w, h, sigma, src_stride=None, dst_stride=None):
    """One call on the default stream; src/dst are device tensors."""
    return lib.sift_cuda_gaussian_blur_u8_noalloc(C.c_void_p(src.data_ptr()), w, h, src_stride or w,
                                                  C.c_void_p(dst.data_ptr()), dst_stride or w, sigma, None)


def octave_levels(pyr, w, h, num_octaves, levels):
    """Split the STAGE_PYRAMID array into [octave][level] (h, w) planes."""
    out, off = [], 0
    for _ in range(num_octaves):
        n = w * h
        out.append([pyr[off + s * n: off + (s + 1) * n].reshape(h, w) for s in range(levels)])
        off += levels * n
        w, h = w // 2, h // 2
    return out


def test_base_level_matches_engine_twice(sgb, oracle_mod):
    import torch
    lib = sgb._capi.lib()
    w, h = 1920, 1080
    img = synth_image(1, w, h)
    eng = sgb.Engine(sgb.Sift.default())
    eng.detect_and_compute(img)
    level0 = eng.debug_stage(sgb.STAGE_PYRAMID)[: w * h].reshape(h, w)
    eng.close()
    sigma = float(oracle_mod.blur_sigmas(oracle_mod.params())[0])
    src = torch.from_numpy(img).cuda()
    for call in range(2):
        dst = torch.zeros_like(src)
        torch.cuda.synchronize()
        assert blur_noalloc(lib, src, dst, w, h, sigma) == 0, lib.sift_cuda_last_error()
        torch.cuda.synchronize()
        got = dst.cpu().numpy()
        assert np.array_equal(got, level0), f"call {call}: {np.count_nonzero(got != level0)} pixels differ"


def test_level_blurs_match_engine(sgb, oracle_mod):
    """Every non-copy level of three octaves, blurred from the level below it;
    octave 1 and 2 increments reach radii above 8 (the engine's two-pass
    path). Strided buffers; each level on two calls in a row."""
    import torch
    lib = sgb._capi.lib()
    w, h, O, S = 1024, 768, 3, 3
    img = synth_image(7, w, h)
    eng = sgb.Engine(sgb.Sift.new(1.6, O, S, 0.5, 0.04, 10.0))
    eng.detect_and_compute(img)
    pyr = octave_levels(eng.debug_stage(sgb.STAGE_PYRAMID), w, h, O, S + 3)
    eng.close()
    sig = oracle_mod.blur_sigmas(oracle_mod.params(1.6, O, S, 0.5, 0.04, 10.0))
    checked = 0
    for o in range(O):
        for s in range(1, S + 3):
            sigma = float(sig[1 + o * (S + 2) + (s - 1)])
            if sigma <= 0.0:
                continue
            below, want = pyr[o][s - 1], pyr[o][s]
            hh, ww = below.shape
            stride = ww + 40
            src = torch.zeros((hh, stride), dtype=torch.uint8, device="cuda")
            src[:, :ww] = torch.from_numpy(np.ascontiguousarray(below)).cuda()
            for call in range(2):
                dst = torch.full((hh, stride + 8), 7, dtype=torch.uint8, device="cuda")
                torch.cuda.synchronize()
                rc = blur_noalloc(lib, src, dst, ww, hh, sigma, stride, stride + 8)
                assert rc == 0, lib.sift_cuda_last_error()
                torch.cuda.synchronize()
                got = dst.cpu().numpy()
                assert np.array_equal(got[:, :ww], want), (o, s, call)
                assert np.all(got[:, ww:] == 7), "wrote past the row"
            checked += 1
    assert checked >= 10


def test_large_sigma_and_in_place_match_oracle(sgb, oracle_mod):
    import torch
    lib = sgb._capi.lib()
    w, h = 333, 217
    img = np.random.default_rng(3).integers(0, 256, size=(h, w), dtype=np.uint8)
    want = oracle_mod.gaussian_blur(img, 20.0)  # radius 40
    buf = torch.from_numpy(img).cuda()
    torch.cuda.synchronize()
    assert blur_noalloc(lib, buf, buf, w, h, 20.0) == 0, lib.sift_cuda_last_error()
    torch.cuda.synchronize()
    assert np.array_equal(buf.cpu().numpy(), want)


def test_rejects_requests_beyond_the_scratch(sgb):
    import torch
    lib = sgb._capi.lib()
    src = torch.zeros(16, dtype=torch.uint8, device="cuda")
    dst = torch.full((16,), 9, dtype=torch.uint8, device="cuda")
    # 3e9: a radius beyond int range, rejected on the host like any other
    for (w, h, sigma) in [(8193, 1, 1.0), (4096, 4097, 1.0), (4, 4, 40.0), (4, 4, 3e9)]:
        rc = blur_noalloc(lib, src, dst, w, h, sigma)
        assert rc == ERR_UNSUPPORTED
        msg = lib.sift_cuda_last_error().decode()
        assert "limit" in msg or "above 64" in msg, msg
    assert blur_noalloc(lib, src, dst, 4, 4, 0.0) == 1
    torch.cuda.synchronize()
    assert np.all(dst.cpu().numpy() == 9), "a rejected call launched work"
