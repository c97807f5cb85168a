"""Serving and batching forms of the CUDA engine (the sift_cuda_server_* and
sift_cuda_replay entry points of include/sift_cuda.h).

``Server`` keeps resident engines ("slots") per image size, admits requests by
their device footprint against a memory budget and runs several at once on
separate streams (continuous batching). ``Server.detect_batch`` is the batched
form: every image of a batch is submitted at once and the results come back
in input order. ``replay`` drives the server, or the plain one-call-per-image
path, with an open-loop arrival trace and returns per-request latencies.
Results are bit-identical to ``Engine.detect_and_compute`` on the same image.
"""
from __future__ import annotations

import ctypes as C
import os
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass

import numpy as np

from . import _capi
from ._capi import DESC_LEN, KEYPOINT_DTYPE
from .sift import Sift, _as_gray

_STORAGE = {"f32": _capi.STORAGE_F32, "f16": _capi.STORAGE_F16, "u8": _capi.STORAGE_U8}


@dataclass
class Served:
    ticket: int
    tag: int
    status: int
    keypoints: np.ndarray
    descriptors: np.ndarray
    submit_s: float
    start_s: float
    done_s: float

    @property
    def latency_s(self) -> float:
        return self.done_s - self.submit_s


def footprint_bytes(sift: Sift, width: int, height: int, storage: str = "u8") -> int:
    """Device bytes of one slot for a width x height image (admission estimate)."""
    p = sift.to_c()
    return int(_capi.lib().sift_cuda_footprint_bytes(C.byref(p), _STORAGE[storage], width, height))


def _host_view(addr: int, nbytes: int) -> np.ndarray:
    """A uint8 view of library-owned host memory (no copy, no ownership)."""
    if not nbytes:
        return np.empty(0, np.uint8)
    return np.ctypeslib.as_array((C.c_uint8 * nbytes).from_address(addr))


def _c_image(img: np.ndarray):
    img = _as_gray(img)
    if img.strides[1] != 1:
        img = np.ascontiguousarray(img)
    return img, img.shape[1], img.shape[0], img.strides[0]


class Server:
    """A continuous-batching SIFT server on one GPU."""

    def __init__(self, sift: Sift | None = None, device: int = 0, storage: str = "u8",
                 arena_bytes: int = 40 << 30, max_inflight: int = 8, autotune: bool = False):
        L = _capi.lib()
        self.sift = sift or Sift.default()
        p = self.sift.to_c()
        o = _capi.ServerOptions()
        L.sift_cuda_server_options_default(C.byref(o))
        o.device, o.storage = device, _STORAGE[storage]
        o.arena_bytes, o.max_inflight, o.autotune = arena_bytes, max_inflight, int(autotune)
        h = C.c_void_p()
        _capi.check(L.sift_cuda_server_create(C.byref(p), C.byref(o), C.byref(h)))
        self._h = h
        self._storage, self._arena = storage, arena_bytes
        self._borrowed = {}  # ticket -> array kept alive while borrowed
        self._held = []      # tickets whose results detect_batch(copy=False) returned as views
        self._pool = None    # copy threads of detect_batch(copy=True)

    def close(self) -> None:
        if getattr(self, "_h", None):
            if self._pool is not None:
                self._pool.shutdown(wait=True)
                self._pool = None
            _capi.lib().sift_cuda_server_destroy(self._h)
            self._h = C.c_void_p()
            self._borrowed.clear()
            self._held.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, img, tag: int = 0, borrow: bool = False) -> int:
        """Queues one image; returns its ticket. borrow=True skips the copy:
        the array must stay unchanged until its result is polled."""
        if self._held:
            self._release_held()
        img, w, h, stride = _c_image(img)
        t = C.c_uint64()
        _capi.check(_capi.lib().sift_cuda_server_submit(self._h, img.ctypes.data, w, h, stride, tag,
                                                        _capi.SUBMIT_BORROW if borrow else 0, C.byref(t)))
        if borrow:
            self._borrowed[t.value] = img
        return t.value

    def poll(self, timeout_s: float | None = None, release: bool | None = None,
             copy: bool = True) -> Served | None:
        """The next finished request, or None on timeout. copy=True copies the
        keypoints and descriptors out and (by default) releases the request's
        slot; copy=False returns views of the slot's host buffers, which stay
        valid until release(ticket) (the default then is not to release)."""
        if release is None:
            release = copy
        if release and not copy:
            raise ValueError("views of a released request would dangle: pass copy=True or release=False")
        sv = _capi.Served()
        us = -1 if timeout_s is None else int(timeout_s * 1e6)
        if _capi.lib().sift_cuda_server_poll(self._h, C.byref(sv), us) != 1:
            return None
        n = sv.n if sv.status == 0 else 0
        if copy:
            kps = np.empty(n, dtype=KEYPOINT_DTYPE)
            desc = np.empty((n, DESC_LEN), dtype=np.float32)
            if n:
                C.memmove(kps.ctypes.data, sv.kps, n * KEYPOINT_DTYPE.itemsize)
                C.memmove(desc.ctypes.data, sv.desc, n * DESC_LEN * 4)
        else:
            kps = _host_view(sv.kps or 0, n * KEYPOINT_DTYPE.itemsize).view(KEYPOINT_DTYPE)
            desc = _host_view(sv.desc or 0, n * DESC_LEN * 4).view(np.float32).reshape(n, DESC_LEN)
        out = Served(sv.ticket, sv.tag, sv.status, kps, desc, sv.submit_s, sv.start_s, sv.done_s)
        self._borrowed.pop(sv.ticket, None)
        if release:
            self.release(sv.ticket)
        return out

    def release(self, ticket: int) -> None:
        _capi.check(_capi.lib().sift_cuda_server_release(self._h, ticket))

    def warm(self, img, count: int = 1) -> None:
        """Creates up to `count` slots for this image's size (untimed)."""
        img, w, h, stride = _c_image(img)
        _capi.check(_capi.lib().sift_cuda_server_warm(self._h, img.ctypes.data, w, h, stride, count))

    def stats(self) -> dict:
        s = _capi.ServerStats()
        _capi.check(_capi.lib().sift_cuda_server_stats(self._h, C.byref(s)))
        return {f: getattr(s, f) for f, _ in _capi.ServerStats._fields_ if f != "reserved"}

    def tuning(self, width: int, height: int) -> tuple[bool, dict]:
        k = (C.c_int32 * 4)()
        tuned = _capi.lib().sift_cuda_server_tuning_knobs(self._h, width, height, k, 4) == 1
        return tuned, {"fused_max_radius": k[0], "level_tile_rows": k[1], "ori_ctas_per_sm": k[2],
                       "desc_ctas_per_sm": k[3]}

    def _copy_out(self, r: Served):
        kps, desc = r.keypoints.copy(), r.descriptors.copy()
        self.release(r.ticket)
        return r.tag, kps, desc

    def _release_held(self) -> None:
        held, self._held = self._held, []
        for t in held:
            self.release(t)

    def detect_batch(self, images, borrow: bool = False, copy: bool = True) -> list[tuple[np.ndarray, np.ndarray]]:
        """The batched form: all images in flight at once; results in input
        order. borrow=True skips the copy into pinned memory (pass pinned
        arrays for the fastest host-to-device copies).

        copy=True returns arrays the caller owns; they are copied out of the
        slots' host buffers by a pool of threads while the GPU runs the rest
        of the batch. copy=False returns views of those buffers (the GPU
        writes its results there): valid until the next detect_batch, submit
        or close on this server. Held views keep their slots busy, so a batch
        whose slots together exceed the server's arena (where requests would
        wait for slots that only the next call frees) is copied instead."""
        self._release_held()
        if not copy:
            need = 0
            for img in images:
                g = _as_gray(img)
                need += footprint_bytes(self.sift, g.shape[1], g.shape[0], self._storage)
            copy = need > self._arena
        for i, img in enumerate(images):
            self.submit(img, tag=i, borrow=borrow)
        out = [None] * len(images)
        if copy:
            if self._pool is None:
                self._pool = ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1))
            futs = []
            failed = None
            for _ in range(len(images)):
                r = self.poll(copy=False)
                if r.status:
                    self.release(r.ticket)
                    failed = failed or r
                    continue
                futs.append(self._pool.submit(self._copy_out, r))
            for f in futs:
                tag, kps, desc = f.result()
                out[tag] = (kps, desc)
            if failed is not None:
                raise _capi.SiftCudaError(failed.status, f"request {failed.tag} failed")
            return out
        failed = None
        for _ in range(len(images)):
            r = self.poll(copy=False)
            if r.status:
                self.release(r.ticket)
                failed = failed or r
                continue
            self._held.append(r.ticket)
            out[r.tag] = (r.keypoints, r.descriptors)
        if failed is not None:
            raise _capi.SiftCudaError(failed.status, f"request {failed.tag} failed")
        return out


def replay(images: list, arrivals_s, image_index, server: Server | None = None, sift: Sift | None = None,
           storage: str = "u8", device: int = 0) -> tuple[np.ndarray, np.ndarray, float]:
    """Open-loop replay. Request i (image images[image_index[i]]) is due at
    arrivals_s[i] after the start; returns (latency_s per request, keypoint
    count per request, wall seconds). server=None replays the plain path:
    one synchronous call per request on an engine per image size."""
    L = _capi.lib()
    imgs = [_c_image(im) for im in images]
    keep = []
    try:
        import torch
        pinned = []
        for img, w, h, stride in imgs:
            t = torch.empty((h, w), dtype=torch.uint8).pin_memory()
            t.numpy()[:] = img
            pinned.append((t.numpy(), w, h, w))
            keep.append(t)
        imgs = pinned
    except Exception:
        pass
    cimgs = (_capi.ReplayImage * len(imgs))()
    for k, (img, w, h, stride) in enumerate(imgs):
        cimgs[k].data, cimgs[k].width, cimgs[k].height, cimgs[k].stride = img.ctypes.data, w, h, stride
    n = len(arrivals_s)
    reqs = (_capi.ReplayRequest * n)()
    for i, (t, k) in enumerate(zip(arrivals_s, image_index)):
        reqs[i].arrival_s, reqs[i].image = float(t), int(k)
    res = (_capi.ReplayResult * n)()
    wall = C.c_double()
    sift = sift or (server.sift if server else Sift.default())
    p = sift.to_c()
    o = _capi.Options()
    L.sift_cuda_options_default(C.byref(o))
    o.device, o.storage = device, _STORAGE[storage]
    _capi.check(L.sift_cuda_replay(server._h if server else None, C.byref(p), C.byref(o), cimgs, len(imgs), reqs, n,
                                   res, C.byref(wall)))
    lat = np.array([r.latency_s for r in res])
    nk = np.array([r.n for r in res], dtype=np.int64)
    st = np.array([r.status for r in res])
    if np.any(st != 0):
        raise _capi.SiftCudaError(int(st[st != 0][0]), "a replayed request failed")
    del keep
    return lat, nk, wall.value
