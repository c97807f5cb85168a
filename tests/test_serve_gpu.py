"""The serving and batching forms against the plain per-image path (GPU).

Every request's keypoints and descriptors must be the same alone and in the
mix — bit for bit, since the server runs the same kernels on the same image,
only concurrently with other requests on other streams.
"""
import time

import numpy as np
import pytest
from synthetic import synth_image

pytestmark = pytest.mark.gpu

SIZES = [(640, 480), (1280, 720), (1920, 1080), (333, 217)]


@pytest.fixture(scope="module")
def sgb(built_lib):
    import sift_wgpu_gb300
    return sift_wgpu_gb300


@pytest.fixture(scope="module")
def images(sgb):
    return [synth_image(4_000_000 + i, w, h) for i, (w, h) in enumerate(SIZES)]


@pytest.fixture(scope="module")
def alone(sgb, images):
    with sgb.Engine(sgb.Sift.default()) as eng:
        return [eng.detect_and_compute(img) for img in images]


def same(a, b):
    return a[0].tobytes() == b[0].tobytes() and a[1].tobytes() == b[1].tobytes()


def test_mixed_requests_match_alone(sgb, images, alone):
    """24 requests of four sizes submitted back to back (copied and borrowed),
    up to 8 on the device at once."""
    with sgb.Server(max_inflight=8) as srv:
        order = [i % len(images) for i in range(24)]
        for k, i in enumerate(order):
            srv.submit(images[i], tag=k, borrow=bool(k % 2))
        got = {}
        while len(got) < len(order):
            r = srv.poll(timeout_s=60)
            assert r is not None, "server stalled"
            assert r.status == 0
            got[r.tag] = r
        for k, i in enumerate(order):
            assert same((got[k].keypoints, got[k].descriptors), alone[i]), f"request {k} (image {i}) differs"
        st = srv.stats()
        assert st["completed"] == len(order) and st["running"] == 0 and st["pending"] == 0
        assert st["slots"] >= len(images)


def test_batch_matches_per_image(sgb, images, alone):
    with sgb.Server(max_inflight=4) as srv:
        out = srv.detect_batch(images + images[::-1])
    for i, res in enumerate(out[: len(images)]):
        assert same(res, alone[i])
    for i, res in enumerate(out[len(images):]):
        assert same(res, alone[len(images) - 1 - i])


def test_batch_views_match_per_image(sgb, images, alone):
    """detect_batch(copy=False): views of the slots' host buffers, the same
    values; a second batch of the same sizes reuses the released slots."""
    with sgb.Server(max_inflight=4) as srv:
        batch = images + images[::-1]
        out = srv.detect_batch(batch, copy=False)
        for i, res in enumerate(out):
            assert not res[1].flags.owndata
            assert same(res, alone[i if i < len(images) else len(batch) - 1 - i])
        slots = srv.stats()["slots"]
        out = srv.detect_batch(batch, copy=False)
        assert same(out[0], alone[0])
        assert srv.stats()["slots"] == slots
        with pytest.raises(ValueError):  # views of a released request
            srv.poll(timeout_s=0, copy=False, release=True)


def test_small_arena_evicts_and_still_matches(sgb, images, alone):
    """A budget that holds about one 1080p slot: requests wait for memory,
    idle slots of other sizes are evicted, results unchanged."""
    budget = sgb.footprint_bytes(sgb.Sift.default(), 1920, 1080) + (64 << 20)
    with sgb.Server(arena_bytes=budget, max_inflight=4) as srv:
        order = [2, 0, 1, 2, 3, 0, 2, 1]
        for k, i in enumerate(order):
            srv.submit(images[i], tag=k)
        got = {}
        while len(got) < len(order):
            r = srv.poll(timeout_s=60)
            assert r is not None and r.status == 0
            got[r.tag] = r
        for k, i in enumerate(order):
            assert same((got[k].keypoints, got[k].descriptors), alone[i])
        st = srv.stats()
        assert st["evicted"] > 0
        assert st["device_bytes"] <= budget * 1.05


def test_oversize_request_fails_cleanly(sgb, images):
    with sgb.Server(arena_bytes=64 << 20) as srv:
        srv.submit(images[2], tag=7)
        r = srv.poll(timeout_s=60)
        assert r is not None and r.tag == 7 and r.status == 4  # SIFT_CUDA_ERR_CAPACITY


def test_autotune_keeps_results(sgb, images, alone):
    with sgb.Server(max_inflight=2, autotune=True) as srv:
        srv.submit(images[2], tag=0)
        r = srv.poll(timeout_s=120)
        assert r.status == 0
        assert same((r.keypoints, r.descriptors), alone[2])
        tuned, knobs = srv.tuning(1920, 1080)
        assert tuned
        assert knobs["fused_max_radius"] in (0, 4, 8) and knobs["level_tile_rows"] in (32, 64)
        assert knobs["ori_ctas_per_sm"] in (2, 4, 8) and knobs["desc_ctas_per_sm"] in (4, 8, 16)
        srv.submit(images[2], tag=1)
        r = srv.poll(timeout_s=60)
        assert same((r.keypoints, r.descriptors), alone[2])


def test_replay_served_and_plain(sgb, images, alone):
    """A short open-loop trace through both paths: every request completes
    with the keypoint count of its image, latencies are positive."""
    rng = np.random.default_rng(5)
    n = 60
    arrivals = np.cumsum(rng.exponential(1 / 400.0, size=n))
    idx = rng.integers(0, len(images), size=n)
    counts = np.array([len(a[0]) for a in alone])
    with sgb.Server(max_inflight=8) as srv:
        for img in images:
            srv.warm(img, 2)
        lat, nk, wall = sgb.replay(images, arrivals, idx, server=srv)
    assert np.array_equal(nk, counts[idx])
    assert np.all(lat > 0) and wall >= arrivals[-1]
    lat_p, nk_p, wall_p = sgb.replay(images, arrivals, idx, server=None)
    assert np.array_equal(nk_p, counts[idx])
    assert np.all(lat_p > 0)


def test_requests_submitted_while_others_run_start_early(sgb, images):
    """Continuous batching: a small request submitted while a large one runs
    finishes before the large one (it is not queued behind it)."""
    big = synth_image(77, 4096, 4096)
    with sgb.Server(max_inflight=4) as srv:
        srv.warm(big, 1)
        srv.warm(images[3], 1)
        srv.submit(big, tag=0, borrow=True)
        time.sleep(0.0002)
        srv.submit(images[3], tag=1, borrow=True)
        first = srv.poll(timeout_s=60)
        second = srv.poll(timeout_s=60)
        assert first.status == 0 and second.status == 0
        assert first.tag == 1 and second.tag == 0
        assert first.start_s < second.done_s


def test_batch64_sample_matches_oracle(sgb, oracle_mod):
    """Six images of the uneven 64-image batch (the smallest, the largest, the
    most elongated and three more) run together through detect_batch, each
    compared with the CPU oracle on its own: the same keypoints in the
    reference order within the tolerance bar, descriptors within 1e-3
    relative L2."""
    from parity import DESC_RTOL, MATCH_RATE, match
    import synthetic
    shapes = synthetic.batch64_shapes()
    area = [w * h for w, h in shapes]
    elong = [max(w / h, h / w) for w, h in shapes]
    pick = []
    for i in (int(np.argmin(area)), int(np.argmax(area)), int(np.argmax(elong)), 0, 1, 2):
        if i not in pick:
            pick.append(i)
    imgs = [synthetic.synth_image(1000 + i, *shapes[i]) for i in pick]
    with sgb.Server(max_inflight=8) as srv:
        out = srv.detect_batch(imgs)
    for i, img, (k, d) in zip(pick, imgs, out):
        rk, rd = oracle_mod.detect_and_compute(img)
        m = match(rk, rd, k, d)
        assert len(rk) > 0 and m.rate >= MATCH_RATE and m.same_order, f"image {i} {shapes[i]}: {m.summary()}"
        assert float(m.desc_err.max()) <= DESC_RTOL, f"image {i}: {m.summary()}"
