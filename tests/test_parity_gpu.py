"""CUDA engine vs the CPU oracle, through the C ABI (GPU tests).

Bit-exact bars: every Gaussian level, every DoG value, the candidate list and
the refined keypoints (x, y, response, octave, layer; size within 2 ulp, it is
the one value that goes through a transcendental). Tolerance bars for the
final keypoints and descriptors: tests/parity.py.
"""
import numpy as np
import pytest

from parity import DESC_RTOL, MATCH_RATE, match
from synthetic import synth_image

pytestmark = pytest.mark.gpu

CASES = [
    # (name, width, height, seed, sift_new args)
    ("512_default", 512, 512, 0, (1.6, 4, 3, 0.5, 0.04, 10.0)),
    ("1080p_default", 1920, 1080, 1, (1.6, 4, 3, 0.5, 0.04, 10.0)),
    ("odd_333x217", 333, 217, 5, (1.6, 4, 3, 0.5, 0.04, 10.0)),
    ("1024_6oct", 1024, 1024, 3, (1.6, 6, 3, 0.5, 0.04, 10.0)),
    ("640x480_s4", 640, 480, 9, (1.6, 5, 4, 0.5, 0.04, 10.0)),
    # the large-image workload: blur radii of octaves 4-5 (sigma ~49-99 px)
    # exceed the 256 x 256 and 128 x 128 octave sizes
    ("4096_6oct", 4096, 4096, 3, (1.6, 6, 3, 0.5, 0.04, 10.0)),
]


@pytest.fixture(scope="module")
def sgb(built_lib):
    import sift_wgpu_gb300
    return sift_wgpu_gb300


_engines = {}


def engine_for(sgb, args, storage="u8"):
    key = (args, storage)
    if key not in _engines:
        _engines[key] = sgb.Engine(sgb.Sift.new(*args), storage=storage)
    return _engines[key]


_oracle_cache = {}


def oracle_stages(oracle_mod, img, args, key):
    if key not in _oracle_cache:
        _oracle_cache[key] = oracle_mod.stages(img, oracle_mod.params(*args))
    return _oracle_cache[key]


def image(sgb, w, h, seed):
    return synth_image(seed, w, h)


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_stages_bit_exact(sgb, oracle_mod, case):
    name, w, h, seed, args = case
    img = image(sgb, w, h, seed)
    st = oracle_stages(oracle_mod, img, args, name)
    eng = engine_for(sgb, args)
    kps, desc = eng.detect_and_compute(img)
    pyr = eng.debug_stage(sgb.STAGE_PYRAMID)
    assert pyr.shape == st.pyramid.shape
    if not np.array_equal(pyr, st.pyramid):
        bad = np.nonzero(pyr != st.pyramid)[0]
        pytest.fail(f"pyramid differs at {len(bad)} of {pyr.size} values, first at {bad[:5]}")
    # DoG = G_{s+1}/255 - G_s/255 in f32 (src/sift.rs:92-124). No DoG plane
    # is stored; this read-back runs, on the device, the function through
    # which candidate emission and refinement read DoG (the u8 planes and the
    # v / 255 table in device memory), over every pixel. The extrema scan
    # stages DoG through its own tile loader, which the bit-identical
    # candidate list below checks.
    dog = eng.debug_stage(sgb.STAGE_DOG)
    off_g = off_d = 0
    L = st.levels
    for (ow, oh) in st.octave_dims:
        n = ow * oh
        lv = [st.pyramid[off_g + s * n: off_g + (s + 1) * n].astype(np.float32) / np.float32(255.0) for s in range(L)]
        for s in range(L - 1):
            ref = lv[s + 1] - lv[s]
            assert np.array_equal(dog[off_d + s * n: off_d + (s + 1) * n], ref)
        off_g += L * n
        off_d += (L - 1) * n
    cands = eng.debug_stage(sgb.STAGE_CANDIDATES)
    assert cands.tobytes() == st.candidates.tobytes(), f"{len(cands)} vs {len(st.candidates)} candidates"
    ref = eng.debug_stage(sgb.STAGE_REFINED)
    assert len(ref) == len(st.refined)
    for f in ("x", "y", "response", "octave", "layer", "angle"):
        assert np.array_equal(ref[f], st.refined[f]), f
    ulp = np.spacing(np.abs(st.refined["size"]))
    assert np.all(np.abs(ref["size"] - st.refined["size"]) <= 2 * ulp)


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_keypoints_and_descriptors_match(sgb, oracle_mod, case):
    name, w, h, seed, args = case
    img = image(sgb, w, h, seed)
    st = oracle_stages(oracle_mod, img, args, name)
    kps, desc = engine_for(sgb, args).detect_and_compute(img)
    m = match(st.keypoints, st.descriptors, kps, desc)
    print(name, m.summary())
    assert len(st.keypoints) > 0
    assert m.rate >= MATCH_RATE, m.summary()
    assert float(m.desc_err.max()) <= DESC_RTOL, m.summary()


def test_committed_fixture(sgb):
    """The CUDA path against the committed oracle fixture
    (tests/golden/oracle_256_seed0.npz)."""
    from pathlib import Path
    fx = np.load(Path(__file__).resolve().parent / "golden" / "oracle_256_seed0.npz")
    kps, desc = engine_for(sgb, (1.6, 4, 3, 0.5, 0.04, 10.0)).detect_and_compute(fx["image"])
    m = match(fx["keypoints"], fx["descriptors"], kps, desc)
    assert m.rate >= MATCH_RATE and m.same_order, m.summary()
    assert float(m.desc_err.max()) <= DESC_RTOL, m.summary()


def test_uniform_image_has_no_keypoints(sgb):
    """tests/integration_test.rs:205-226"""
    eng = engine_for(sgb, (1.6, 4, 3, 0.5, 0.04, 10.0))
    kps, desc = eng.detect_and_compute(np.full((100, 100), 128, np.uint8))
    assert len(kps) == 0 and desc.shape == (0, 128)


@pytest.mark.parametrize("shape", [(0, 0), (1, 1), (15, 20), (3, 64), (64, 3), (9, 9), (31, 33)])
def test_tiny_and_degenerate_images(sgb, oracle_mod, shape):
    """Empty octaves, images smaller than the border, kernels wider than the
    image: same result as the oracle."""
    h, w = shape
    if h == 15 and w == 20:
        img = np.tile((np.arange(20) * 10).astype(np.uint8), (15, 1))  # tests/integration_test.rs:166-203
    else:
        img = np.random.default_rng(h * 100 + w).integers(0, 256, size=(h, w), dtype=np.uint8)
    eng = engine_for(sgb, (1.6, 4, 3, 0.5, 0.04, 10.0))
    kps, desc = eng.detect_and_compute(img)
    rk, rd = oracle_mod.detect_and_compute(img)
    m = match(rk, rd, kps, desc)
    assert len(kps) == len(desc)
    assert len(m.unmatched_ref) == 0 and len(m.unmatched_got) == 0, m.summary()


def test_strided_input_and_determinism(sgb):
    """Determinism (tests/integration_test.rs:106-164): bit-identical keypoints
    and descriptors across calls, and a padded row stride changes nothing."""
    img = image(sgb, 700, 500, 21)
    padded = np.zeros((500, 768), np.uint8)
    padded[:, :700] = img
    view = padded[:, :700]
    eng = engine_for(sgb, (1.6, 4, 3, 0.5, 0.04, 10.0))
    k1, d1 = eng.detect_and_compute(img)
    k2, d2 = eng.detect_and_compute(view)
    k3, d3 = eng.detect_and_compute(img)
    assert k1.tobytes() == k2.tobytes() == k3.tobytes()
    assert d1.tobytes() == d2.tobytes() == d3.tobytes()


def test_image_in_place_and_copied_agree(sgb):
    """A pageable image that starts and strides on 16 bytes is read where it
    is on a GB300 (its Grace host memory is device-readable); a pinned image
    and one with a 1-byte wider stride are copied to the device first. All
    give the same keypoints and descriptors, pyramid included."""
    import torch
    img = image(sgb, 1280, 720, 33)
    eng = engine_for(sgb, (1.6, 4, 3, 0.5, 0.04, 10.0))
    k1, d1 = eng.detect_and_compute(img)
    in_place = eng.last_image_in_place
    p1 = eng.debug_stage(sgb.STAGE_PYRAMID)
    pinned = torch.from_numpy(img).pin_memory().numpy()
    k2, d2 = eng.detect_and_compute(pinned)
    assert not eng.last_image_in_place
    buf = np.zeros((720, 1281), np.uint8)
    buf[:, :1280] = img
    k3, d3 = eng.detect_and_compute(buf[:, :1280])
    assert not eng.last_image_in_place
    assert k1.tobytes() == k2.tobytes() == k3.tobytes()
    assert d1.tobytes() == d2.tobytes() == d3.tobytes()
    assert np.array_equal(eng.debug_stage(sgb.STAGE_PYRAMID), p1)
    k4, d4 = eng.detect_and_compute(img)  # back in place (the cell is rewritten)
    assert k4.tobytes() == k1.tobytes() and d4.tobytes() == d1.tobytes()
    if "GB300" in torch.cuda.get_device_name(0):
        assert in_place and eng.last_image_in_place


@pytest.mark.parametrize("storage", ["f32", "f16"])
def test_other_storage_modes_are_exact(sgb, storage):
    """u8-valued levels are exact in f32 (as v / 255) and in f16 (as v), the
    u8 default reads v / 255 through the IEEE quotient, and every mode forms
    DoG from the same u8 planes, so f32 and f16 storage give the u8 mode's
    output bit for bit, pyramid included."""
    args = (1.6, 4, 3, 0.5, 0.04, 10.0)
    img = image(sgb, 1920, 1080, 1)
    e8 = engine_for(sgb, args, "u8")
    k8, d8 = e8.detect_and_compute(img)
    p8 = e8.debug_stage(sgb.STAGE_PYRAMID)
    e = engine_for(sgb, args, storage)
    k, d = e.detect_and_compute(img)
    assert k.tobytes() == k8.tobytes()
    assert d.tobytes() == d8.tobytes()
    assert np.array_equal(e.debug_stage(sgb.STAGE_PYRAMID), p8)


@pytest.mark.parametrize("w,h,seed,args", [(1920, 1080, 1, (1.6, 4, 3, 0.5, 0.04, 10.0)),
                                            (333, 217, 2, (1.6, 4, 3, 0.5, 0.04, 10.0)),
                                            (1024, 1024, 5, (1.6, 6, 3, 0.5, 0.04, 10.0))])
def test_level_tile_rows_32_is_exact(sgb, w, h, seed, args):
    """The fused level kernel on 32-row tiles (an option and an autotuner
    knob) computes every level pixel with the same operations as on 64-row
    tiles: the pyramid, keypoints and descriptors are bit-identical, on a
    size whose last tile row is partial and with six octaves."""
    img = image(sgb, w, h, seed)
    e64 = engine_for(sgb, args, "u8")
    k64, d64 = e64.detect_and_compute(img)
    p64 = e64.debug_stage(sgb.STAGE_PYRAMID)
    with sgb.Engine(sgb.Sift.new(*args), level_tile_rows=32) as e32:
        k32, d32 = e32.detect_and_compute(img)
        assert np.array_equal(e32.debug_stage(sgb.STAGE_PYRAMID), p64)
    assert k32.tobytes() == k64.tobytes()
    assert d32.tobytes() == d64.tobytes()


def test_level_tile_rows_rejects_other_values(sgb):
    with pytest.raises(sgb.SiftCudaError):
        sgb.Engine(sgb.Sift.default(), level_tile_rows=48)


def test_high_contrast_threshold(sgb):
    """tests/integration_test.rs:228-281"""
    img = image(sgb, 512, 512, 0)
    k_def, _ = engine_for(sgb, (1.6, 4, 3, 0.5, 0.04, 10.0)).detect_and_compute(img)
    k_hi, d_hi = engine_for(sgb, (1.6, 4, 3, 0.5, 1.0, 10.0)).detect_and_compute(img)
    assert len(k_def) > 0 and (len(k_hi) < len(k_def) // 2 or len(k_hi) == 0)
    assert len(k_hi) == len(d_hi)


def test_detect_is_detect_and_compute_without_descriptors(sgb):
    """Sift::detect (src/sift.rs:846-886) = the keypoints of detect_and_compute."""
    img = image(sgb, 640, 480, 4)
    eng = engine_for(sgb, (1.6, 4, 3, 0.5, 0.04, 10.0))
    k, _ = eng.detect_and_compute(img)
    assert eng.detect(img).tobytes() == k.tobytes()


def test_sift_api_drop_in(sgb):
    """Sift::detect_and_compute_with_backend(img, SiftBackend::Cuda) returns
    Vec<KeyPoint> + Vec<Vec<f32>> with 128 floats each."""
    img = image(sgb, 320, 240, 2)
    s = sgb.Sift.default()
    kps, desc = s.detect_and_compute_with_backend(img, sgb.SiftBackend.from_str("cuda"))
    assert len(kps) == len(desc) > 0
    assert all(len(d) == 128 for d in desc)
    assert isinstance(kps[0], sgb.KeyPoint)


def test_large_6_octave_properties(sgb):
    """4096 x 4096, Sift::new(1.6, 6, 3, 0.5, 0.04, 10.0): size-independent
    properties at the full size (determinism, f16 == u8 == f32, unit-norm
    descriptors, keypoints inside the image)."""
    args = (1.6, 6, 3, 0.5, 0.04, 10.0)
    img = image(sgb, 4096, 4096, 3)
    e = engine_for(sgb, args)
    k1, d1 = e.detect_and_compute(img)
    k2, d2 = e.detect_and_compute(img)
    assert k1.tobytes() == k2.tobytes() and d1.tobytes() == d2.tobytes()
    assert len(k1) > 10000
    n = np.linalg.norm(d1, axis=1)
    assert np.all((np.abs(n - 1) < 1e-4) | (n == 0))
    assert np.all((k1["x"] >= -1) & (k1["x"] <= 4097) & (k1["y"] >= -1) & (k1["y"] <= 4097))
    for storage in ("f16", "f32"):
        ks, ds = engine_for(sgb, args, storage).detect_and_compute(img)
        assert ks.tobytes() == k1.tobytes() and ds.tobytes() == d1.tobytes(), storage


def test_all_call_forms_agree(sgb):
    """The copying call, the zero-copy view, the device-resident run (CUDA
    graph replay) and a profiled run (in-order launches with stage events)
    give bit-identical keypoints and descriptors."""
    import torch
    img = image(sgb, 800, 600, 31)
    eng = sgb.Engine(sgb.Sift.default())
    k1, d1 = eng.detect_and_compute(img)
    kv, dv = eng.detect_and_compute_view(img)
    assert kv.tobytes() == k1.tobytes() and dv.tobytes() == d1.tobytes()
    dimg = torch.from_numpy(img).cuda()
    torch.cuda.synchronize()
    eng.run_device(dimg.data_ptr(), 800, 600, 800)
    eng.synchronize()
    kd = eng.debug_stage(sgb.STAGE_KEYPOINTS)
    dd = eng.debug_stage(sgb.STAGE_DESCRIPTORS)
    assert kd.tobytes() == k1.tobytes() and dd.tobytes() == d1.tobytes()
    eng.profile(True)
    k2, d2 = eng.detect_and_compute(img)
    times, runs = eng.profile_read()
    eng.profile(False)
    assert runs == 1 and all(t > 0 for t in times.values())
    assert k2.tobytes() == k1.tobytes() and d2.tobytes() == d1.tobytes()
    # a different size re-captures; going back reuses a valid graph
    k3, _ = eng.detect_and_compute(image(sgb, 640, 480, 4))
    k4, d4 = eng.detect_and_compute(img)
    assert k4.tobytes() == k1.tobytes() and d4.tobytes() == d1.tobytes()
    eng.close()


def test_export_buffer_growth(sgb):
    """A host call writes descriptors below the export buffer's capacity into
    it from the descriptor stage and the rest to device memory. The first
    call of an engine on a 1080p frame has more keypoints than the initial
    buffer holds (the buffer grows, the head moves over from the old buffer,
    the tail comes from the device); later calls fit. Every form agrees, and
    the descriptor stage read back after a host call is the host result."""
    import torch
    w, h = 1920, 1080
    img = image(sgb, w, h, 1)
    eng = sgb.Engine(sgb.Sift.default())
    k1, d1 = eng.detect_and_compute(img)
    assert len(k1) > 3 * 4096
    assert eng.debug_stage(sgb.STAGE_DESCRIPTORS).tobytes() == d1.tobytes()
    k2, d2 = eng.detect_and_compute(img)
    assert k2.tobytes() == k1.tobytes() and d2.tobytes() == d1.tobytes()
    assert eng.debug_stage(sgb.STAGE_DESCRIPTORS).tobytes() == d1.tobytes()
    dimg = torch.from_numpy(img).cuda()
    torch.cuda.synchronize()
    eng.run_device(dimg.data_ptr(), w, h, w)
    eng.synchronize()
    assert eng.debug_stage(sgb.STAGE_KEYPOINTS).tobytes() == k1.tobytes()
    assert eng.debug_stage(sgb.STAGE_DESCRIPTORS).tobytes() == d1.tobytes()
    eng.close()
