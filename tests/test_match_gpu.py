"""Descriptor matching on the GPU (sift_cuda_match, csrc/match.cu) against the
brute-force oracle (oracle/match.py), through the C ABI.

Indices must agree wherever the oracle's nearest (second-nearest) distance is
not tied with the next one within the f32 error of |q|^2 + |t|^2 - 2 q.t;
squared distances agree within 1e-5 (descriptors have unit norm, so squared
distances lie in [0, 4]).
"""
import ctypes as C

import numpy as np
import pytest
from synthetic import synth_image

pytestmark = pytest.mark.gpu

GAP = 1e-5


@pytest.fixture(scope="module")
def sgb(built_lib):
    import sift_wgpu_gb300
    return sift_wgpu_gb300


@pytest.fixture(scope="module")
def eng(sgb):
    e = sgb.Engine(sgb.Sift.default())
    yield e
    e.close()


def check(got, query, train):
    from oracle.match import match
    i1, d1, i2, d2, third, d2sq = match(query, train)
    assert len(got) == len(query)
    # with fewer than two (three) train descriptors a gap is inf - inf = nan:
    # not a sure ranking, so that row's index is not compared
    with np.errstate(invalid="ignore"):
        sure1 = (d2sq[:, 1] - d2sq[:, 0]) > GAP
        sure2 = sure1 & ((third - d2sq[:, 1]) > GAP)
    assert np.array_equal(got["train_idx"][sure1], i1[sure1])
    assert np.array_equal(got["second_idx"][sure2], i2[sure2])
    have1 = i1 >= 0
    assert np.all((got["train_idx"] >= 0) == have1) and np.all((got["second_idx"] >= 0) == (i2 >= 0))
    assert np.allclose(got["distance"][have1].astype(np.float64) ** 2, d2sq[have1, 0], atol=GAP, rtol=0)
    have2 = i2 >= 0
    assert np.allclose(got["second_distance"][have2].astype(np.float64) ** 2, d2sq[have2, 1], atol=GAP, rtol=0)
    assert np.all(np.isinf(got["distance"][~have1])) and np.all(np.isinf(got["second_distance"][~have2]))
    return sure1.mean()


def unit_rows(rng, n):
    x = np.abs(rng.standard_normal((n, 128))).astype(np.float32)
    x /= np.linalg.norm(x, axis=1, keepdims=True)
    return x


def test_real_descriptors_two_frames(sgb, eng):
    """Descriptors of a 1080p frame against those of the same scene shifted by
    a few pixels: the shifted keypoints find their originals."""
    img = synth_image(1, 1920, 1080)
    k1, d1 = eng.detect_and_compute(img)
    shifted = np.zeros_like(img)
    shifted[3:, 5:] = img[:-3, :-5]
    k2, d2 = eng.detect_and_compute(shifted)
    got = eng.match(d2, d1)
    assert check(got, d2, d1) > 0.99
    good = got["distance"] < 0.8 * got["second_distance"]  # Lowe's ratio test
    i = got["train_idx"][good]
    dx = k2["x"][good] - k1["x"][i]
    dy = k2["y"][good] - k1["y"][i]
    assert good.sum() > 1000
    assert np.median(dx) == pytest.approx(5.0, abs=0.2) and np.median(dy) == pytest.approx(3.0, abs=0.2)


@pytest.mark.parametrize("nq,nt", [(1, 1), (63, 65), (64, 64), (1000, 3001), (4097, 129), (200, 0), (10, 2)])
def test_random_unit_descriptors(eng, nq, nt):
    rng = np.random.default_rng(nq * 7 + nt)
    q, t = unit_rows(rng, nq), unit_rows(rng, nt)
    check(eng.match(q, t), q, t)


def test_ties_go_to_the_lower_index(eng):
    rng = np.random.default_rng(5)
    t = unit_rows(rng, 300)
    t[200] = t[17]  # duplicate of train 17
    t[250] = t[17]
    got = eng.match(t[[17, 200, 5]], t)
    assert list(got["train_idx"]) == [17, 17, 5]
    assert list(got["second_idx"][:2]) == [200, 200]
    assert got["distance"][0] == pytest.approx(0.0, abs=1e-3)


def test_empty_query(eng):
    got = eng.match(np.zeros((0, 128), np.float32), np.ones((5, 128), np.float32))
    assert len(got) == 0


def test_device_form_matches_host_form(sgb, eng):
    import torch
    rng = np.random.default_rng(9)
    q, t = unit_rows(rng, 777), unit_rows(rng, 1500)
    host = eng.match(q, t)
    lib = sgb._capi.lib()
    dq, dt = torch.from_numpy(q).cuda(), torch.from_numpy(t).cuda()
    out = torch.empty(len(q) * 4, dtype=torch.int32, device="cuda")
    scratch = torch.empty(lib.sift_cuda_match_scratch_bytes(len(q), len(t)), dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    rc = lib.sift_cuda_match_device(C.c_void_p(dq.data_ptr()), len(q), C.c_void_p(dt.data_ptr()), len(t),
                                    C.c_void_p(out.data_ptr()), C.c_void_p(scratch.data_ptr()), None)
    assert rc == 0, lib.sift_cuda_last_error()
    torch.cuda.synchronize()
    dev = out.cpu().numpy().view(sgb.MATCH_DTYPE)
    assert dev.tobytes() == host.tobytes()
    # misaligned descriptor arrays are refused
    rc = lib.sift_cuda_match_device(C.c_void_p(dq.data_ptr() + 4), 10, C.c_void_p(dt.data_ptr()), len(t),
                                    C.c_void_p(out.data_ptr()), C.c_void_p(scratch.data_ptr()), None)
    assert rc == 1
