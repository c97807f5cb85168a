"""The CPU oracle against the reference's own known-answer tests and
integration properties (CPU only, no GPU).

The oracle restates src/sift.rs; these tests pin it the way the reference pins
itself: the Cramer solve and bilinear sampler known answers
(src/sift.rs:1424-1525) and the integration properties of
tests/integration_test.rs on seeded synthetic images (the reference's JPEG
fixtures need a decoder this environment lacks).
"""
import json
import math
from pathlib import Path

import numpy as np
import pytest
from synthetic import synth_image

GOLDEN = Path(__file__).resolve().parent / "golden"
KAT = json.loads((GOLDEN / "reference_kat.json").read_text())


def check_properties(kps, w, h, S=3):
    """check_keypoint_properties (tests/integration_test.rs:13-62)."""
    pi = np.float32(math.pi)
    assert np.all(kps["x"] >= -1.0) and np.all(kps["x"] <= w + 1.0)
    assert np.all(kps["y"] >= -1.0) and np.all(kps["y"] <= h + 1.0)
    assert np.all(kps["size"] > 0.0)
    assert np.all(kps["angle"] >= -pi) and np.all(kps["angle"] <= pi)
    assert np.all(kps["octave"] >= 0)
    assert np.all(kps["layer"] >= -2) and np.all(kps["layer"] <= S + 4)


@pytest.mark.parametrize("case", KAT["solve_linear_system"])
def test_solve_linear_system_kat(oracle_mod, case):
    x = oracle_mod.solve3(case["a"], case["b"])
    if case["x"] is None:
        assert x is None
    else:
        assert x is not None
        assert np.allclose(x, case["x"], atol=case["tol"], rtol=0)


def test_bilinear_kat(oracle_mod):
    k = KAT["get_gauss_pixel_bilinear"]
    img = np.array(k["image"], dtype=np.uint8)
    for c in k["cases"]:
        v = oracle_mod.bilinear(img, c["x"], c["y"])
        assert abs(v - np.float32(c["v"]) / np.float32(255.0)) < k["tol"], c


def test_uniform_image_has_no_keypoints(oracle_mod):
    u = KAT["uniform_image"]
    img = np.full((u["height"], u["width"]), u["value"], dtype=np.uint8)
    kps, desc = oracle_mod.detect_and_compute(img)
    assert len(kps) == u["keypoints"] and len(desc) == 0


def test_small_gradient_properties(oracle_mod):
    img = np.tile((np.arange(20) * 10).astype(np.uint8), (15, 1))
    kps, desc = oracle_mod.detect_and_compute(img)
    assert len(kps) == len(desc)
    if len(kps):
        check_properties(kps, 20, 15)


def test_synthetic_properties_and_determinism(oracle_mod):
    img = synth_image(0, 512, 512)
    k1, d1 = oracle_mod.detect_and_compute(img, threads=4)
    k2, d2 = oracle_mod.detect_and_compute(img, threads=1)
    assert len(k1) > 0 and len(k1) == len(d1)
    check_properties(k1, 512, 512)
    # determinism (tests/integration_test.rs:106-164), across thread counts too
    assert k1.tobytes() == k2.tobytes()
    assert np.max(np.abs(d1 - d2)) < 1e-6
    norms = np.linalg.norm(d1, axis=1)
    assert np.all((np.abs(norms - 1.0) < 1e-4) | (norms == 0.0))


def test_high_contrast_threshold(oracle_mod):
    img = synth_image(0, 512, 512)
    k_def, _ = oracle_mod.detect_and_compute(img)
    k_hi, d_hi = oracle_mod.detect_and_compute(img, oracle_mod.params(contrast_threshold=1.0))
    assert len(k_def) > 0
    assert len(k_hi) < len(k_def) // 2 or len(k_hi) == 0
    assert len(k_hi) == len(d_hi)


def test_blur_sigmas_follow_reference_formula(oracle_mod):
    """generate_gaussian_pyramid increments (src/sift.rs:141-147): octave o is
    2^o times octave 0, base = sqrt(1.6^2 - 0.5^2)."""
    s = oracle_mod.blur_sigmas()
    base, rest = s[0], s[1:].reshape(4, 5)
    assert abs(base - math.sqrt(1.6 ** 2 - 0.25)) < 1e-5
    assert np.allclose(rest[0], [1.2262735, 1.5450078, 1.9465878, 2.452547, 3.0900155], rtol=1e-5)
    for o in range(4):
        assert np.array_equal(rest[o], rest[0] * np.float32(2 ** o))


def test_blur_matches_independent_python_restatement(oracle_mod):
    """imageproc gaussian_blur_f32 restated twice (C++ oracle vs float32
    numpy loops) must agree bit for bit, including clamp-to-edge when the
    kernel is wider than the image."""
    rng = np.random.default_rng(5)
    for (h, w, sigma) in [(9, 13, 1.3), (6, 5, 3.7), (17, 11, 0.6)]:
        img = rng.integers(0, 256, size=(h, w), dtype=np.uint8)
        k = oracle_mod.gaussian_kernel(sigma)
        r = (len(k) - 1) // 2
        assert r == math.ceil(2 * np.float32(sigma))

        def pass1d(a):
            out = np.empty_like(a)
            H, W = a.shape
            for y in range(H):
                for x in range(W):
                    acc = np.float32(0)
                    for i in range(len(k)):
                        xs = min(max(x + i - r, 0), W - 1)
                        acc = np.float32(acc + np.float32(a[y, xs]) * k[i])
                    out[y, x] = 255 if acc >= 255 else (0 if acc <= 0 else int(acc))
            return out

        ref = pass1d(pass1d(img).T.copy()).T
        assert np.array_equal(oracle_mod.gaussian_blur(img, sigma), ref)


def test_lanczos_uniform_and_shape(oracle_mod):
    img = np.full((37, 50), 77, dtype=np.uint8)
    out = oracle_mod.resize_lanczos3(img, 25, 18)
    assert out.shape == (18, 25) and np.all(out == 77)


def test_extrema_match_numpy_restatement(oracle_mod):
    """find_scale_space_extrema restated in numpy on the oracle's own pyramid:
    same candidates, same (octave, layer, y, x) order."""
    img = synth_image(11, 96, 80)
    st = oracle_mod.stages(img)
    rows = []
    for o, (w, h) in enumerate(st.octave_dims):
        g = [st.level(o, s).astype(np.float32) / np.float32(255.0) for s in range(st.levels)]
        d = [g[i + 1] - g[i] for i in range(len(g) - 1)]
        for s in range(1, 4):
            cube = np.stack(d[s - 1:s + 2])
            for y in range(5, h - 5):
                for x in range(5, w - 5):
                    v = cube[1, y, x]
                    nb = cube[:, y - 1:y + 2, x - 1:x + 2].ravel()
                    nb = np.delete(nb, 13)
                    if np.all(v > nb) or np.all(v < nb):
                        rows.append((o, s, y, x))
    got = [(int(k["octave"]), int(k["layer"]), int(k["y"] / 2 ** k["octave"]), int(k["x"] / 2 ** k["octave"]))
           for k in st.candidates]
    assert got == rows


def test_oracle_reproduces_committed_fixture(oracle_mod):
    """tests/golden/oracle_256_seed0.npz (make_oracle_fixtures.py): the oracle
    still gives the committed keypoints and descriptors."""
    from parity import match
    fx = np.load(GOLDEN / "oracle_256_seed0.npz")
    kps, desc = oracle_mod.detect_and_compute(fx["image"])
    m = match(fx["keypoints"], fx["descriptors"], kps, desc)
    assert len(kps) == len(fx["keypoints"]) and m.rate == 1.0 and m.same_order, m.summary()
    assert float(m.desc_err.max()) <= 1e-6, m.summary()


def test_fp64_model_is_the_reference_algorithm(oracle_mod):
    """oracle/ideal64.py with the reference's u8 rounding and f32 DoG put back
    reproduces the u8 oracle's pyramid, candidates and refined keypoints (up
    to the few pixels where float64 and f32 accumulation truncate differently),
    so the FP64 model of the precision statement differs from the reference
    path only by those roundings."""
    from oracle.ideal64 import Ideal64
    img = synth_image(0, 512, 512)
    m = Ideal64(quantize=True, dog_f32=True)
    pyr = m.pyramid(img)
    dog = m.dog(pyr)
    st = oracle_mod.stages(img, oracle_mod.params())
    off = diff = 0
    for lv in pyr:
        for g in lv:
            n = g.size
            diff += int(np.count_nonzero(st.pyramid[off: off + n].reshape(g.shape) != g))
            off += n
    assert diff < 1e-3 * off
    cands = m.extrema(dog)
    ref = {(int(k["octave"]), int(k["layer"]), float(k["x"]), float(k["y"])) for k in st.candidates}
    got = {(o, s, (x + 0.5) * 2.0 ** o, (y + 0.5) * 2.0 ** o) for (o, s, x, y) in cands}
    assert len(ref & got) >= 0.995 * len(ref)
    refined = m.refine(cands, dog)
    rx = np.array([k["x"] for k in refined])
    ry = np.array([k["y"] for k in refined])
    hit = 0
    for k in st.refined:
        d = np.hypot(rx - float(k["x"]), ry - float(k["y"]))
        hit += int(d.min() < 1e-3)
    assert hit >= 0.995 * len(st.refined)


def test_luma_restatements(oracle_mod):
    """Known answers of the two luma formulas (image 0.25.6 to_luma8 integer
    weights; src/wasm.rs:89-93 in f32)."""
    px = np.array([[[255, 255, 255, 0], [255, 0, 0, 9], [0, 255, 0, 9], [0, 0, 255, 9], [10, 20, 30, 0]]], np.uint8)
    assert oracle_mod.luma_u8(px, 2).tolist() == [[255, 54, 182, 18, 18]]
    f = np.float32
    want = [int(np.trunc((f(0.299) * f(r) + f(0.587) * f(g)) + f(0.114) * f(b))) for r, g, b, _ in px[0]]
    assert oracle_mod.luma_u8(px, 3).tolist() == [want]
    assert oracle_mod.luma_u8(px[..., :3], 1).tolist() == oracle_mod.luma_u8(px, 2).tolist()


def test_match_oracle_against_a_plain_loop():
    """oracle/match.py (the checker of sift_cuda_match) against a plain loop
    over every pair, with duplicate train rows (ties go to the lower index),
    a single train row and an empty train set."""
    import numpy as np
    from oracle.match import match
    rng = np.random.default_rng(3)
    q = rng.random((20, 128)).astype(np.float32)
    t = rng.random((30, 128)).astype(np.float32)
    t[7] = t[3]
    q[0] = t[3]
    i1, d1, i2, d2, third, _ = match(q, t)
    for a in range(len(q)):
        d = [float(((q[a].astype(np.float64) - t[b]) ** 2).sum()) for b in range(len(t))]
        order = sorted(range(len(t)), key=lambda b: (d[b], b))
        assert i1[a] == order[0] and i2[a] == order[1]
        assert abs(d1[a] ** 2 - d[order[0]]) < 1e-9 and abs(d2[a] ** 2 - d[order[1]]) < 1e-9
    assert i1[0] == 3 and i2[0] == 7
    i1, d1, i2, d2, third, _ = match(q[:2], t[:1])
    assert list(i1) == [0, 0] and list(i2) == [-1, -1] and np.all(np.isinf(d2))
    i1, d1, i2, d2, third, _ = match(q[:2], t[:0])
    assert list(i1) == [-1, -1] and np.all(np.isinf(d1))


def test_draw_oracle_shapes():
    """oracle/draw.py (the checker of sift_cuda_draw_keypoints): one keypoint
    gives the midpoint-circle disc of radius 6 (symmetric, 13 rows and columns
    wide), its orientation line and the centre dot, clipped at the border."""
    import numpy as np
    from oracle.draw import draw_keypoints_to_image
    from sift_wgpu_gb300._capi import KEYPOINT_DTYPE
    kp = np.zeros(1, KEYPOINT_DTYPE)
    kp["x"], kp["y"], kp["angle"] = 20.7, 20.2, 0.0
    img = draw_keypoints_to_image(np.zeros((41, 41), np.uint8), kp, (255, 0, 0))
    red = img[:, :, 0] == 255
    assert np.array_equal(red, red[::-1, :]) and np.array_equal(red, red[:, ::-1])
    ys, xs = np.nonzero(red)
    assert (ys.min(), ys.max(), xs.min(), xs.max()) == (14, 26, 14, 26)
    assert red[20, 14:27].all() and not red[20, 27]
    assert np.all(img[:, :, 1][red] == 0) and np.all(img[~red] == 0)
    kp["x"], kp["y"] = 1.5, 1.5
    img = draw_keypoints_to_image(np.full((10, 10), 7, np.uint8), kp, (0, 255, 0))
    assert (img[:, :, 1] == 255).sum() > 0 and img[9, 9, 1] == 7
