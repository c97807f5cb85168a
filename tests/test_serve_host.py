"""The batching logic of sift_wgpu_gb300.Server.detect_batch, checked on the
CPU against a fake server core (submit / poll / release): results in input
order, views held until the next call, owned copies released as they are
made, the arena check that turns a view batch into a copy, and failures."""
import ctypes as C

import numpy as np
import pytest

import sift_wgpu_gb300 as sg
from sift_wgpu_gb300 import serve


class FakeCore:
    """Finishes requests in reverse order; a request's results live in a
    buffer owned by its 'slot' until released (then the slot is reused and
    the buffer is overwritten)."""

    def __init__(self, fail_tag=None):
        self.pending, self.released, self.fail_tag = [], [], fail_tag
        self.buffers = {}
        self.next_ticket = 1

    def submit(self, img, tag=0, borrow=False):
        t = self.next_ticket
        self.next_ticket += 1
        n = int(img[0, 0])  # the image's first pixel says how many keypoints
        kps = np.zeros(n, sg.KEYPOINT_DTYPE)
        kps["x"] = np.arange(n) + tag
        desc = np.full((n, sg.DESC_LEN), float(tag), np.float32)
        self.buffers[t] = (kps, desc)
        self.pending.append((t, tag))
        return t

    def poll(self, timeout_s=None, release=None, copy=True):
        t, tag = self.pending.pop()  # reverse order
        kps, desc = self.buffers[t]
        status = 5 if tag == self.fail_tag else 0
        if copy:
            kps, desc = kps.copy(), desc.copy()
        return serve.Served(t, tag, status, kps, desc, 0.0, 0.0, 0.0)

    def release(self, ticket):
        self.released.append(ticket)
        kps, desc = self.buffers.pop(ticket)
        kps["x"] = -1  # the slot's buffer is reused
        desc[:] = -1


def fake_server(core, arena=40 << 30):
    srv = object.__new__(sg.Server)
    srv._h = C.c_void_p()
    srv._borrowed, srv._held, srv._pool = {}, [], None
    srv.sift, srv._storage, srv._arena = sg.Sift.default(), "f32", arena
    srv.submit, srv.poll, srv.release = core.submit, core.poll, core.release
    return srv


def images(counts):
    return [np.full((16, 16), c, np.uint8) for c in counts]


@pytest.mark.parametrize("copy", [True, False])
def test_results_in_input_order(copy):
    core = FakeCore()
    srv = fake_server(core)
    out = srv.detect_batch(images([3, 0, 5, 2]), copy=copy)
    assert [len(k) for k, _ in out] == [3, 0, 5, 2]
    for tag, (k, d) in enumerate(out):
        assert np.array_equal(k["x"], np.arange(len(k)) + tag) and np.all(d == tag)
    if srv._pool is not None:
        srv._pool.shutdown()


def test_owned_copies_are_released_and_survive_slot_reuse():
    core = FakeCore()
    srv = fake_server(core)
    out = srv.detect_batch(images([4, 4]), copy=True)
    assert sorted(core.released) == [1, 2] and srv._held == []
    assert np.array_equal(out[1][0]["x"], np.arange(4) + 1)  # unaffected by the release
    srv._pool.shutdown()


def test_views_are_held_until_the_next_call():
    core = FakeCore()
    srv = fake_server(core)
    out = srv.detect_batch(images([4, 4]), copy=False)
    assert core.released == [] and sorted(srv._held) == [1, 2]
    assert np.array_equal(out[0][0]["x"], np.arange(4))  # still the slot's data
    srv.detect_batch(images([1]), copy=False)
    assert sorted(core.released) == [1, 2] and srv._held == [3]


def test_view_batch_larger_than_the_arena_is_copied():
    core = FakeCore()
    one = sg.footprint_bytes(sg.Sift.default(), 16, 16)
    srv = fake_server(core, arena=one)  # room for one slot, not two
    srv.detect_batch(images([2, 2]), copy=False)
    assert sorted(core.released) == [1, 2] and srv._held == []
    srv._pool.shutdown()


@pytest.mark.parametrize("copy", [True, False])
def test_a_failed_request_raises_after_the_batch_is_drained(copy):
    core = FakeCore(fail_tag=1)
    srv = fake_server(core)
    with pytest.raises(sg._capi.SiftCudaError):
        srv.detect_batch(images([2, 2, 2]), copy=copy)
    assert core.pending == []  # every request was polled
    assert 2 in core.released  # the failed one is released
    if srv._pool is not None:
        srv._pool.shutdown()


def test_poll_refuses_released_views():
    srv = fake_server(FakeCore())
    srv.poll = sg.Server.poll.__get__(srv)  # the real poll: checks its arguments first
    with pytest.raises(ValueError):
        srv.poll(timeout_s=0, copy=False, release=True)


def test_host_view_is_a_view():
    buf = (C.c_uint8 * 64)()
    v = serve._host_view(C.addressof(buf), 64)
    buf[3] = 7
    assert v[3] == 7 and not v.flags.owndata
    assert serve._host_view(0, 0).size == 0
