"""The C-ABI library without a GPU: it loads, exports every entry point that
include/sift_cuda.h declares, and its host-only helpers behave (no kernel is
launched here)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    text = (ROOT / "include" / "sift_cuda.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sift_\w+)\s*\(", text)))


def test_header_symbols_exported(built_lib):
    lib = C.CDLL(str(built_lib))
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    from sift_wgpu_gb300 import _capi
    assert sorted(_capi.exported_symbols()) == names


def test_params_mirror_sift_new(built_lib):
    from sift_wgpu_gb300 import _capi
    L = _capi.lib()
    p = _capi.Params()
    L.sift_cuda_params_default(C.byref(p))
    assert (p.num_octaves, p.num_intervals, p.image_border_width) == (4, 3, 5)
    assert p.contrast_threshold == np.float32(0.04) / np.float32(3)
    L.sift_cuda_params_new(C.byref(p), 1.6, 6, 3, 0.5, 0.04, 10.0)
    assert p.num_octaves == 6 and p.contrast_threshold == np.float32(np.float32(0.04) / np.float32(3))
    from sift_wgpu_gb300 import Sift
    s = Sift.new(1.6, 6, 3, 0.5, 0.04, 10.0)
    assert s.contrast_threshold == p.contrast_threshold


def test_backend_from_str():
    from sift_wgpu_gb300 import SiftBackend, SiftError
    assert SiftBackend.from_str(" CUDA ") is SiftBackend.Cuda
    assert SiftBackend.from_str("gpu") is SiftBackend.WebGpu
    assert SiftBackend.from_str("v2") is SiftBackend.WebGpuV2
    assert SiftBackend.from_str("prefer-gpu") is SiftBackend.WebGpuWithCpuFallback
    assert SiftBackend.default() is SiftBackend.WebGpuWithCpuFallback
    with pytest.raises(SiftError):
        SiftBackend.from_str("opencl")


def test_other_backends_are_not_served_here(built_lib):
    from sift_wgpu_gb300 import Sift, SiftBackend, SiftError
    img = np.zeros((8, 8), np.uint8)
    for b in (SiftBackend.Cpu, SiftBackend.WebGpu, SiftBackend.WebGpuV2, SiftBackend.WebGpuWithCpuFallback):
        with pytest.raises(SiftError):
            Sift.default().detect_and_compute_with_backend(img, b)


def test_synth_is_seeded_and_dense():
    """The workload generator is seeded, dense, and loads no native code."""
    import synthetic
    a = synthetic.synth_image(0, 512, 512)
    b = synthetic.synth_image(0, 512, 512)
    c = synthetic.synth_image(1, 512, 512)
    assert a.dtype == np.uint8 and a.shape == (512, 512)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert 100 < a.mean() < 160 and a.std() > 10
    assert synthetic.density(1920, 1080) == (1582, 316)
    assert synthetic.density(4096, 4096) == (12800, 2560)
    assert synthetic.synth_image(3, 0, 0).shape == (0, 0)
    # draws of one stream do not depend on how they are split
    u = synthetic.uniforms(5, 3, 0, 1000)
    assert np.array_equal(u[400:], synthetic.uniforms(5, 3, 400, 600))
    assert 0.45 < u.mean() < 0.55 and u.min() >= 0.0 and u.max() < 1.0
    imports = re.findall(r"^\s*(?:import|from)\s+(\S+)", (ROOT / "synthetic.py").read_text(), flags=re.M)
    assert set(imports) <= {"numpy", "__future__"}, imports


def test_engine_errors_are_reported(built_lib):
    from sift_wgpu_gb300 import _capi
    L = _capi.lib()
    p = _capi.Params()
    L.sift_cuda_params_default(C.byref(p))
    p.num_octaves = 0
    h = C.c_void_p()
    rc = L.sift_cuda_create(C.byref(p), None, C.byref(h))
    assert rc == 1 and b"num_octaves" in L.sift_cuda_last_error()
    assert not h.value
    res = _capi.Result()
    rc = L.sift_cuda_detect_and_compute(None, None, 4, 4, 4, C.byref(res))
    assert rc == 1 and res.n == 0


def test_option_and_tuning_query_arguments_are_checked(built_lib):
    """Checked before any device call (no GPU needed): a fused level tile
    height other than 0, 32 or 64, and a tuning query without a server."""
    from sift_wgpu_gb300 import _capi
    L = _capi.lib()
    p = _capi.Params()
    L.sift_cuda_params_default(C.byref(p))
    o = _capi.Options()
    L.sift_cuda_options_default(C.byref(o))
    assert o.level_tile_rows == 0 and o.storage == _capi.STORAGE_U8
    o.level_tile_rows = 48
    h = C.c_void_p()
    rc = L.sift_cuda_create(C.byref(p), C.byref(o), C.byref(h))
    assert rc == 1 and b"level_tile_rows" in L.sift_cuda_last_error() and not h.value
    knobs = (C.c_int32 * 4)()
    assert L.sift_cuda_server_tuning_knobs(None, 1920, 1080, knobs, 4) == 1
    assert L.sift_cuda_server_tuning(None, 1920, 1080, knobs) == 1


def footprint_restated(S, O, w, h, es):
    """The admission estimate of a server slot, restated: the arena layout
    (pitch = width rounded to 32; S+3 Gaussian and S+3 u8 planes per octave,
    no DoG planes; horizontal-pass and resize scratch; two mask-word
    arrays) plus list capacities of 1/64 of the scanned positions (>= 1024)
    at 140 candidate-list bytes and 540 output bytes each, plus the padded
    image and 1 MiB of tables."""
    al = lambda v, a: (v + a - 1) // a * a
    g = u = tmpb = tmpo = lt = words = caps = 0
    ow, oh = w, h
    for o in range(O):
        pitch = al(max(ow, 1), 32)
        plane, nw = pitch * oh, (ow + 31) // 32
        g += plane * (S + 3) * es
        u += plane * (S + 3)
        tmpb = max(tmpb, plane)
        tmpo += al(plane, 256)
        if o + 1 < O:
            lt = max(lt, pitch * (oh // 2) * 4)
        wo = S * oh * nw
        words += wo * 8
        caps += min(max(wo * 32 // 64, 1024), 1 << 28)
        ow, oh = ow // 2, oh // 2
    return al(max(w, 1), 128) * h + g + u + tmpb + tmpo + lt + words + caps * 140 + caps * 540 + (1 << 20)


@pytest.mark.parametrize("shape", [(640, 480), (1920, 1080), (3840, 2160), (333, 217), (1, 1)])
def test_server_footprint_estimate(built_lib, shape):
    """Admission is by this estimate; it runs on the host (no GPU)."""
    import sift_wgpu_gb300 as sg
    w, h = shape
    s = sg.Sift.default()
    f32 = sg.footprint_bytes(s, w, h, "f32")
    f16 = sg.footprint_bytes(s, w, h, "f16")
    assert f32 == footprint_restated(3, 4, w, h, 4)
    assert f16 == footprint_restated(3, 4, w, h, 2)
    assert f16 < f32
