#!/usr/bin/env python
"""Benchmark of the GB300 SIFT engine on the 1080p workload.

One step = one full detect_and_compute (pyramid + DoG, extrema + refinement,
orientation, descriptors) of one 1920x1080 u8 synthetic frame (seed 1,
Sift::default()), the configuration the headline metric "1080p images/s" is
quoted on. Prints one JSON line.

  value   images/s with the image already resident in HBM, device time of K
          steps from CUDA events on the engine's stream; the L2 is flushed
          (256 MiB write) before every step, outside the timed events.
  e2e     images/s through the C ABI with a pinned host image
          (sift_cuda_detect_and_compute_view): host->device copy, the pipeline
          and the device->host copy of keypoints and descriptors into host
          memory inside the timed region (wall clock).
  roofline  the dominant stage, timed live with CUDA events in the timed
          region; algorithmic bytes per run: pyramid_bytes() below for the
          pyramid stage, keypoint and descriptor bytes for the gather stages.
  cpu_baseline  the C++ restatement of the reference CPU path (oracle/) on the
          host cores, bounded sample of the same frame.

  serving  the continuous-batching server (sift_wgpu_gb300.Server) against
          the plain one-call-per-image path on the same open-loop Poisson
          trace of mixed resolutions (40% 640x480, 30% 1280x720, 20% 1920x1080,
          10% 3840x2160): p50/p99 latency per offered rate, and the saturated
          images/s of both (all requests due at once).

--workload batch64 prints the batched form (64 images of uneven sizes in
flight at once, results as views of the host buffers the GPU wrote; the
owned-copy form beside it) against the plain path; --workload serve prints the full
serving sweep (20000 requests per offered rate, 500-8000 req/s).

--impl reference times that CPU path alone (the reference crate itself cannot
be built here: no Rust toolchain), with the same metric and workload.
Multi-GPU (torchrun): independent replicas, one engine per rank, no
collective on the data path; value = all ranks' images / max rank time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOADS = {
    # name: (width, height, seed, Sift::new args)
    "1080p": (1920, 1080, 1, (1.6, 4, 3, 0.5, 0.04, 10.0)),
    "512": (512, 512, 0, (1.6, 4, 3, 0.5, 0.04, 10.0)),
    "4096": (4096, 4096, 3, (1.6, 6, 3, 0.5, 0.04, 10.0)),
}
METRIC = "1080p images/s"
STORED_BYTES = {"f32": 4, "f16": 2, "u8": 0}  # per pixel of a stored level, beside its u8 plane
FLUSH_BYTES = 256 << 20


def pyramid_bytes(w: int, h: int, octaves: int, S: int, b: int) -> int:
    """Algorithmic bytes of the pyramid stage as stored here: the u8 input
    read once, every octave base read once (as its u8 plane), S+3 Gaussian
    levels written once as u8 planes (1 byte) plus, in the f32 and f16 modes,
    the stored level (b = 4 or 2 bytes; 0 in u8 storage). No DoG plane is
    written: extrema and refinement form DoG from the u8 planes."""
    total = w * h  # u8 input
    ow, oh = w, h
    for o in range(octaves):
        n = ow * oh
        if o > 0:
            total += n
        total += n * (S + 3) * (b + 1)
        ow, oh = ow // 2, oh // 2
    return total


def blur_radii(octaves: int, S: int, sigma: float = 1.6, assumed_blur: float = 0.5):
    """(base radius, [[radius of level s = 1..S+2] per octave]) of the
    pyramid's Gaussian blurs: the increments of generate_gaussian_pyramid
    (src/sift.rs:141-147) in f32 and imageproc's radius ceil(2 sigma)."""
    f = np.float32
    sg, ab = f(sigma), f(assumed_blur)
    base = np.sqrt(sg * sg - ab * ab) if sg > ab else f(0)
    k = f(2.0) ** (f(1.0) / f(S))
    target = [sg * f(k) ** s for s in range(S + 3)]
    out = []
    for o in range(octaves):
        scale = f(2.0 ** o)
        prev = sg * scale
        row = []
        for s in range(1, S + 3):
            t = f(target[s] * scale)
            b = np.sqrt(t * t - prev * prev)
            row.append(int(np.ceil(f(2.0) * b)) if b >= f(1e-4) else 0)
            prev = t
        out.append(row)
    return (int(np.ceil(f(2.0) * base)) if base > f(1e-4) else 0), out


def pyramid_fp32_ops(w: int, h: int, octaves: int, S: int, sigma: float = 1.6, assumed_blur: float = 0.5) -> int:
    """Separately rounded f32 multiplies and adds the pyramid stage needs (the
    reference's tap order forbids fusing them): two passes of 2r + 1 taps per
    pixel for every Gaussian level, and the 2x Lanczos3 resize between octaves
    (12 taps per output in each pass: the vertical pass over the source width,
    the horizontal over the destination). Halo recomputation is not counted."""
    r0, radii = blur_radii(octaves, S, sigma, assumed_blur)
    taps = 0
    ow, oh = w, h
    for o in range(octaves):
        n = ow * oh
        if n == 0:
            break
        if o == 0 and r0:
            taps += n * 2 * (2 * r0 + 1)
        for r in radii[o]:
            if r:
                taps += n * 2 * (2 * r + 1)
        if o + 1 < octaves and ow // 2 and oh // 2:
            taps += 12 * ow * (oh // 2) + 12 * (ow // 2) * (oh // 2)
        ow, oh = ow // 2, oh // 2
    return 2 * taps


FP32_LANES_PER_SM = 128
N_SMS = 152


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def traffic_from_profiles(workload: str, stage: str, kind: str = "dram_bytes"):
    """A per-run figure of one stage from profiles/traffic.json (scoped ncu
    captures): kind "dram_bytes" (DRAM read + write bytes) or "inst" (warp
    instructions); None where nothing was captured."""
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists():
        return None
    try:
        return json.loads(p.read_text()).get(kind, {}).get(workload, {}).get(stage)
    except (ValueError, OSError, AttributeError):
        return None


def issue_roofline(inst, ms: float, sm_mhz):
    """Instruction issue as the roofline of an issue-bound stage: warp
    instructions per run (ncu) over the stage time, against 152 SMs x 4
    schedulers x one warp instruction per clock at the sampled SM clock."""
    if not inst or not ms or not sm_mhz:
        return None
    peak = 152 * 4 * float(sm_mhz) * 1e6 / 1e9
    achieved = inst / (ms / 1e3) / 1e9
    return {"bound": "issue", "achieved": achieved, "peak": peak, "unit": "G warp instructions/s",
            "frac": achieved / peak, "inst_per_run": inst, "peak_kind": "152 SMs x 4 schedulers x sampled SM clock"}


def measured_peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    try:
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    except (OSError, ValueError, KeyError):
        return 6800.0, "fallback"


def cpu_baseline(img, args, budget_s: float = 15.0) -> dict:
    from oracle import oracle

    threads = os.cpu_count() or 1
    p = oracle.params(*args)
    oracle.detect_and_compute(img, p, threads)  # warm-up
    times = []
    t_end = time.perf_counter() + budget_s
    while len(times) < 3 or (time.perf_counter() < t_end and len(times) < 50):
        t0 = time.perf_counter()
        oracle.detect_and_compute(img, p, threads)
        times.append(time.perf_counter() - t0)
    med = statistics.median(times)
    return {"value": 1.0 / med, "unit": "images/s", "cores": threads, "kind": "port",
            "sample": f"{len(times)} runs of the same {img.shape[1]}x{img.shape[0]} frame, median; "
                      f"C++ restatement of src/sift.rs (blur/resize sequential as in the reference, "
                      f"rayon axes on {threads} threads)"}


SERVE_MIX = [((640, 480), 0.4), ((1280, 720), 0.3), ((1920, 1080), 0.2), ((3840, 2160), 0.1)]


def serve_pool(per_size: int = 4):
    """Images of the serving mix: per_size distinct seeded frames per
    resolution (seeds 4000000 + k), at the 512x512 density."""
    from synthetic import synth_image
    images, size_of = [], []
    for si, ((w, h), _) in enumerate(SERVE_MIX):
        for j in range(per_size):
            images.append(synth_image(4_000_000 + si * per_size + j, w, h))
            size_of.append(si)
    return images, np.array(size_of)


def serve_trace(n: int, rate: float, size_of, seed: int = 4):
    """Poisson arrivals at `rate` req/s; each request draws a resolution from
    the mix and one of that resolution's pooled images."""
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=n)) if rate > 0 else np.zeros(n)
    probs = np.array([p for _, p in SERVE_MIX])
    sizes = rng.choice(len(SERVE_MIX), size=n, p=probs)
    idx = np.empty(n, dtype=np.int64)
    for si in range(len(SERVE_MIX)):
        pool = np.nonzero(size_of == si)[0]
        m = sizes == si
        idx[m] = rng.choice(pool, size=int(m.sum()))
    return arrivals, idx, sizes


def lat_summary(lat, sizes=None):
    ms = np.asarray(lat) * 1e3
    out = {"p50_ms": float(np.percentile(ms, 50)), "p99_ms": float(np.percentile(ms, 99)),
           "mean_ms": float(ms.mean())}
    if sizes is not None:
        m = sizes == 2  # 1920x1080
        if m.any():
            out["p50_1080p_ms"] = float(np.percentile(ms[m], 50))
            out["p99_1080p_ms"] = float(np.percentile(ms[m], 99))
    return out


def serving_report(n_req: int, rates, max_inflight: int = 8, autotune: bool = False, device: int = 0) -> dict:
    """Served vs plain on the same traces (both warmed, untimed)."""
    import sift_wgpu_gb300 as sg
    images, size_of = serve_pool()
    rep = {"mix": "40% 640x480, 30% 1280x720, 20% 1920x1080, 10% 3840x2160; 4 pooled seeded frames per "
                  "resolution; Poisson arrivals (seed 4); latency from due time to results in host memory",
           "requests_per_rate": n_req, "max_inflight": max_inflight, "autotune": autotune, "rates": []}
    with sg.Server(device=device, max_inflight=max_inflight, autotune=autotune) as srv:
        for si in range(len(SERVE_MIX)):
            srv.warm(images[int(np.nonzero(size_of == si)[0][0])], max_inflight)
        # saturation: every request due at once
        arr0, idx0, sz0 = serve_trace(n_req, 0, size_of)
        lat, nk, wall = sg.replay(images, arr0, idx0, server=srv, device=device)
        served_sat = n_req / wall
        for rate in rates:
            arr, idx, sz = serve_trace(n_req, rate, size_of)
            lat, nk, wall = sg.replay(images, arr, idx, server=srv, device=device)
            rep["rates"].append({"offered_req_s": rate, "served": dict(lat_summary(lat, sz),
                                                                       images_s=n_req / wall)})
        rep["server_stats"] = srv.stats()
    lat, nk, wall = sg.replay(images, arr0, idx0, server=None, device=device)
    plain_sat = n_req / wall
    for k, rate in enumerate(rates):
        arr, idx, sz = serve_trace(n_req, rate, size_of)
        lat, nk, wall = sg.replay(images, arr, idx, server=None, device=device)
        rep["rates"][k]["plain"] = dict(lat_summary(lat, sz), images_s=n_req / wall)
    rep["saturated_images_s"] = {"served": served_sat, "plain": plain_sat, "ratio": served_sat / plain_sat}
    return rep


def batch64_images():
    """64 images, width and height uniform over the multiples of 16 in
    [320, 2560] (seed 2), image i made with seed 1000 + i."""
    from synthetic import batch64_images as make
    return make()


def run_batch64(args, world, rank, local):
    import sift_wgpu_gb300 as sg
    import torch
    images = []
    for im in batch64_images():  # pinned host images, borrowed by the server
        t = torch.from_numpy(im).pin_memory()
        images.append(t.numpy())
    px = sum(im.size for im in images)
    with sg.Server(device=local, max_inflight=args.inflight, autotune=args.autotune) as srv:
        srv.detect_batch(images, borrow=True)  # creates and captures a slot per size
        for _ in range(max(0, args.warmup - 1)):
            srv.detect_batch(images, borrow=True)
        # results as views of the slots' host buffers (the GPU writes them
        # there), and as arrays the caller owns (copied by a thread pool while
        # the rest of the batch runs)
        t, tc = [], []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            out = srv.detect_batch(images, borrow=True, copy=False)
            t.append(time.perf_counter() - t0)
        nk = sum(len(k) for k, _ in out)
        for _ in range(args.steps):
            t0 = time.perf_counter()
            srv.detect_batch(images, borrow=True, copy=True)
            tc.append(time.perf_counter() - t0)
        stats = srv.stats()
    # the flattened batch: one run, every stage one launch over all 64 images
    with sg.Batch(sg.Sift.default(), device=local) as fb:
        for _ in range(max(1, args.warmup)):
            fb.detect_and_compute(images, copy=False)
        tf, tdev = [], []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            fout = fb.detect_and_compute(images, copy=False)
            tf.append(time.perf_counter() - t0)
            tdev.append(fb.last_device_ms / 1e3)
        flat_launches = fb.last_launch_count
        nk_flat = sum(len(k) for k, _ in fout)
    zero = np.zeros(len(images))
    idx = np.arange(len(images))
    sg.replay(images, zero, idx, server=None, device=local)  # warm the plain engines
    tp = []
    for _ in range(args.steps):
        _, _, wall = sg.replay(images, zero, idx, server=None, device=local)
        tp.append(wall)
    served = len(images) / statistics.median(t)
    flat = len(images) / statistics.median(tf)
    plain = len(images) / statistics.median(tp)
    value = flat
    if rank == 0:
        print(json.dumps({
            "metric": "batch64 images/s", "value": value, "unit": "images/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.median(tf),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": "64 u8 images, W,H uniform multiples of 16 in [320, 2560], seeds 1000+i, "
                                   "Sift::default()", "megapixels": px / 1e6, "keypoints": int(nk_flat),
                       "form": "flattened batch: one run, each stage one launch over all images, one CUDA graph",
                       "max_inflight": args.inflight, "autotune": bool(args.autotune)},
            "e2e": {"value": value, "unit": "images/s", "h2d_bytes_per_step": int(px),
                    "d2h_bytes_per_step": int(nk_flat * (28 + 512))},
            "gpu_launches": flat_launches * args.steps,
            "keypoints_per_s": value * int(nk_flat) / 64,
            "flat_over_plain": flat / plain,
            "flat_device_images_s": len(images) / statistics.median(tdev),
            "served_concurrent_graphs_images_s": served, "served_owned_copy_images_s": len(images) / statistics.median(tc),
            "plain_images_s": plain, "served_over_plain": served / plain, "server_stats": stats,
        }), flush=True)


def run_match(args, world, rank, local):
    """Descriptor matching (sift_cuda_match_device on resident descriptors;
    the host form for e2e): the 1080p frame's descriptors as train set, those
    of the same scene shifted by (5, 3) pixels as queries; pairs/s = queries x
    train descriptors compared per second."""
    import ctypes as C
    import torch
    import sift_wgpu_gb300 as sg
    from synthetic import synth_image
    img = synth_image(1, 1920, 1080)
    shifted = np.zeros_like(img)
    shifted[3:, 5:] = img[:-3, :-5]
    torch.cuda.set_device(local)
    with sg.Engine(sg.Sift.default(), device=local) as eng:
        _, dt = eng.detect_and_compute(img)
        _, dq = eng.detect_and_compute(shifted)
        nq, nt = len(dq), len(dt)
        lib = sg._capi.lib()
        q, t = torch.from_numpy(dq).cuda(), torch.from_numpy(dt).cuda()
        out = torch.empty(nq * 4, dtype=torch.int32, device="cuda")
        scratch = torch.empty(lib.sift_cuda_match_scratch_bytes(nq, nt), dtype=torch.uint8, device="cuda")
        stream = torch.cuda.current_stream()
        launch = lambda: lib.sift_cuda_match_device(C.c_void_p(q.data_ptr()), nq, C.c_void_p(t.data_ptr()), nt,
                                                    C.c_void_p(out.data_ptr()), C.c_void_p(scratch.data_ptr()),
                                                    C.c_void_p(stream.cuda_stream))
        for _ in range(args.warmup):
            assert launch() == 0, lib.sift_cuda_last_error()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(args.steps):
            launch()
        b.record(stream)
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / args.steps
        for _ in range(max(1, args.warmup)):
            eng.match(dq, dt)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            m = eng.match(dq, dt)
        e2e_s = (time.perf_counter() - t0) / args.steps
        good = int((m["distance"] < 0.8 * m["second_distance"]).sum())
    pairs = float(nq) * nt
    if rank == 0:
        print(json.dumps({
            "metric": "descriptor pairs/s", "value": pairs / (ms / 1e3), "unit": "pairs/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "match: 1080p frame seed 1 (train) vs the same scene shifted by (5, 3) px (queries)",
                       "queries": nq, "train": nt, "ratio_test_0.8_matches": good},
            "tflops_dot": 2.0 * pairs * 128 / (ms / 1e3) / 1e12,
            "e2e": {"value": pairs / e2e_s, "unit": "pairs/s", "h2d_bytes_per_step": (nq + nt) * 512,
                    "d2h_bytes_per_step": nq * 16},
        }), flush=True)


def run_serve(args, world, rank, local):
    rep = serving_report(args.requests, [500, 1000, 2000, 4000, 8000], max_inflight=args.inflight,
                         autotune=args.autotune, device=local)
    if rank == 0:
        best = min(rep["rates"], key=lambda r: r["served"]["p99_ms"])
        print(json.dumps({
            "metric": "served images/s (mixed-resolution Poisson stream)", "value": rep["saturated_images_s"]["served"],
            "unit": "images/s", "n_gpus": world, "steps": args.requests, "warmup": 1, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "serving mix, 20000 requests per offered rate"}, "serving": rep,
            "best_p99_ms": best["served"]["p99_ms"],
        }), flush=True)


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(world, v: float) -> float:
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args, world, rank):
    """The reference CPU path (its C++ restatement) on the host cores."""
    if rank != 0:
        return
    from synthetic import synth_image
    from oracle import oracle
    w, h, seed, sargs = WORKLOADS.get(args.workload, WORKLOADS["1080p"])
    img = synth_image(seed, w, h)
    threads = os.cpu_count() or 1
    p = oracle.params(*sargs)
    for _ in range(args.warmup):
        oracle.detect_and_compute(img, p, threads)
    # bounded: at most ~150 s of timed work whatever K is
    times = []
    t_start = time.perf_counter()
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.detect_and_compute(img, p, threads)
        times.append(time.perf_counter() - t0)
        if time.perf_counter() - t_start > 150.0:
            break
    total = sum(times)
    value = len(times) / total
    line = {
        "impl": "reference", "metric": METRIC if args.workload == "1080p" else f"{args.workload} images/s",
        "value": value, "unit": "images/s", "n_gpus": args.gpus, "steps": len(times), "warmup": args.warmup,
        "ms_per_step": 1000.0 * total / len(times), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{w}x{h} u8 synthetic frame, seed {seed}, Sift::new{sargs}", "storage": "u8 levels",
                   "steps_requested": args.steps},
        "cpu_baseline": {"value": value, "unit": "images/s", "cores": threads, "kind": "port",
                         "sample": f"{len(times)} detect_and_compute runs of the frame (C++ restatement of "
                                   f"src/sift.rs; the Rust crate cannot be built: no cargo)"},
        "e2e": {"value": value, "unit": "images/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def fp32_roofline(ops: int, ms: float, sm_mhz) -> dict:
    """The pyramid stage against the FP32 pipe: its separately rounded
    multiplies and adds over the stage time, as a fraction of 152 SMs x 128
    f32 lanes x the SM clock sampled during the timed region."""
    mhz = float(sm_mhz) if sm_mhz else 2070.0
    peak = N_SMS * FP32_LANES_PER_SM * mhz * 1e6
    ach = ops / (ms / 1e3)
    return {"bound": "fp32", "ops": int(ops), "achieved_tops": ach / 1e12, "peak_tops": peak / 1e12,
            "unit": "Tops/s", "frac": ach / peak, "sm_mhz": mhz,
            "peak_kind": "152 SMs x 128 f32 lanes x sampled SM clock"}


def pyramid_section(workload: str, local: int, storage: str, steps: int, warmup: int, sm_mhz) -> dict:
    """The pyramid stage of one workload, launched in stage order with CUDA
    events at the stage boundaries (no overlap with the other stages), after
    an L2 flush: HBM and FP32-pipe rooflines."""
    import torch
    import sift_wgpu_gb300 as sg
    from synthetic import synth_image
    w, h, seed, sargs = WORKLOADS[workload]
    img = synth_image(seed, w, h)
    d_img = torch.from_numpy(img).to(f"cuda:{local}")
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device=f"cuda:{local}")
    with sg.Engine(sg.Sift.new(*sargs), device=local, storage=storage) as eng:
        stream = torch.cuda.ExternalStream(eng.stream, device=torch.device("cuda", local))
        torch.cuda.synchronize()
        eng.profile(True)
        with torch.cuda.stream(stream):
            for _ in range(max(1, warmup)):
                eng.run_device(d_img.data_ptr(), w, h, w)
        torch.cuda.synchronize()
        eng.profile_read()
        with torch.cuda.stream(stream):
            for _ in range(steps):
                flush.zero_()
                eng.run_device(d_img.data_ptr(), w, h, w)
        torch.cuda.synchronize()
        stage_ms, runs = eng.profile_read()
        eng.profile(False)
        nk = len(eng.debug_stage(sg.STAGE_KEYPOINTS))
    per_run = {k: v / max(runs, 1) for k, v in stage_ms.items()}
    peak, peak_kind = measured_peaks()
    octs, S = sargs[1], sargs[2]
    b = pyramid_bytes(w, h, octs, S, STORED_BYTES[storage])
    ms = per_run["pyramid_dog"]
    gbs = b / (ms / 1e3) / 1e9
    return {"workload": f"{w}x{h} u8 synthetic frame, seed {seed}, Sift::new{sargs}", "storage": storage,
            "runs": runs, "stages_ms": per_run, "keypoints": nk,
            "hbm": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                    "algorithmic_bytes": b, "ms": ms, "peak_kind": peak_kind,
                    "traffic": traffic_from_profiles(workload, "pyramid_dog")},
            "fp32_pipe": fp32_roofline(pyramid_fp32_ops(w, h, octs, S, sargs[0], sargs[3]), ms, sm_mhz)}


def run_cuda(args, world, rank, local):
    import torch

    import sift_wgpu_gb300 as sg

    w, h, seed, sargs = WORKLOADS[args.workload]
    torch.cuda.set_device(local)
    from synthetic import synth_image
    img = synth_image(seed, w, h)
    eng = sg.Engine(sg.Sift.new(*sargs), device=local, storage=args.storage, level_tile_rows=args.level_tile_rows)
    stream = torch.cuda.ExternalStream(eng.stream, device=torch.device("cuda", local))
    d_img = torch.from_numpy(img).to(f"cuda:{local}")
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device=f"cuda:{local}")
    torch.cuda.synchronize()

    # correctness of what is timed: the device path returns what the host call returns
    kps_ref, desc_ref = eng.detect_and_compute(img)

    for _ in range(args.warmup):
        eng.run_device(d_img.data_ptr(), w, h, w)
    eng.synchronize()
    launches_per_step = eng.last_launch_count

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    sampler = ClockSampler(local)
    barrier(world)
    torch.cuda.synchronize()
    sampler.start()
    t_wall0 = time.perf_counter()
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.zero_()
            ev[k][0].record(stream)
            eng.run_device(d_img.data_ptr(), w, h, w)
            ev[k][1].record(stream)
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall0
    barrier(world)
    clocks = sampler.stop()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    dev_s = sum(step_ms) / 1000.0
    dev_s_max = allreduce_max(world, dev_s)
    value = world * args.steps / dev_s_max

    # Stage breakdown: a second timed region of the same K steps with per-stage
    # CUDA events (in-order launches instead of the graph's two-stream DAG, so
    # each stage has a start and an end).
    eng.profile(True)
    eng.profile_read()
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.zero_()
            eng.run_device(d_img.data_ptr(), w, h, w)
    torch.cuda.synchronize()
    stage_ms, runs = eng.profile_read()
    eng.profile(False)

    # the timed device runs produced what the host call returns
    kps_dev = eng.debug_stage(sg.STAGE_REFINED)
    if len(kps_ref) == 0 or len(kps_dev) == 0:
        raise SystemExit("bench: the workload produced no keypoints")

    # e2e through the C ABI with host buffers (pinned)
    pinned = torch.from_numpy(img).pin_memory()
    host_img = pinned.numpy()
    for _ in range(max(1, args.warmup)):
        eng.detect_and_compute_view(host_img)
    barrier(world)
    e2e_n = args.steps
    t0 = time.perf_counter()
    nk = 0
    for _ in range(e2e_n):
        kk, dd = eng.detect_and_compute_view(host_img)
        nk = len(kk)
    e2e_s = time.perf_counter() - t0
    e2e_s = allreduce_max(world, e2e_s)
    e2e_value = world * e2e_n / e2e_s
    d2h = 16 + nk * (28 + 512)

    # the drop-in call: a pageable image, results in arrays the caller owns
    # (sift_cuda_detect_and_compute copies them out of the engine's buffers)
    pageable = np.array(img, copy=True)
    for _ in range(max(1, args.warmup)):
        eng.detect_and_compute(pageable)
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(e2e_n):
        kk, dd = eng.detect_and_compute(pageable)
    dropin_s = allreduce_max(world, time.perf_counter() - t0)
    dropin_value = world * e2e_n / dropin_s

    # roofline of the dominant stage
    per_run = {k: v / max(runs, 1) for k, v in stage_ms.items()}
    dominant = max(per_run, key=per_run.get)
    peak, peak_kind = measured_peaks()
    octs, S = sargs[1], sargs[2]
    b_pyr = pyramid_bytes(w, h, octs, S, STORED_BYTES[args.storage])
    pyr_gbs = b_pyr / (per_run["pyramid_dog"] / 1e3) / 1e9
    roof_pyr = {"stage": "pyramid_dog", "bound": "hbm", "achieved": pyr_gbs, "peak": peak, "unit": "GB/s",
                "frac": pyr_gbs / peak, "traffic": traffic_from_profiles(args.workload, "pyramid_dog"),
                "algorithmic_bytes": b_pyr, "ms": per_run["pyramid_dog"], "peak_kind": peak_kind,
                "fp32_pipe": fp32_roofline(pyramid_fp32_ops(w, h, octs, S, sargs[0], sargs[3]), per_run["pyramid_dog"],
                                           clocks.get("sm_mhz"))}
    if dominant == "pyramid_dog":
        roof = dict(roof_pyr)
    else:
        # the gather stages read the pyramid levels they sample and write their
        # outputs; DRAM bytes are the bound that the schema tracks
        if dominant == "descriptor":
            alg = nk * (28 + 512)
        elif dominant == "orientation":
            alg = nk * 28 * 2
        else:
            alg = b_pyr
        gbs = alg / (per_run[dominant] / 1e3) / 1e9
        roof = {"stage": dominant, "bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s",
                "frac": gbs / peak, "traffic": traffic_from_profiles(args.workload, dominant),
                "algorithmic_bytes": alg, "ms": per_run[dominant], "peak_kind": peak_kind,
                "issue_slots": issue_roofline(traffic_from_profiles(args.workload, dominant, "inst"),
                                              per_run[dominant], clocks.get("sm_mhz")),
                "note": ("issue-bound gather stage: its DRAM bytes are small, so the HBM fraction is low by "
                         "nature; issue_slots is the roofline that binds it (warp instructions from a scoped ncu "
                         "capture, profiles/); roofline_pyramid_dog is the HBM roofline of the pyramid stage")}

    out = None
    if rank == 0:
        out = {
            "metric": METRIC if args.workload == "1080p" else f"{args.workload} images/s",
            "value": value, "unit": "images/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": statistics.mean(step_ms), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"{w}x{h} u8 synthetic frame, seed {seed}, Sift::new{sargs}",
                       "storage": args.storage, "level_tile_rows": args.level_tile_rows or 64,
                       "parallelism": f"replicas x{world}",
                       "l2": "256 MiB flush before every step", "keypoints": int(nk)},
            "e2e": {"value": e2e_value, "unit": "images/s", "h2d_bytes_per_step": w * h, "d2h_bytes_per_step": d2h,
                    "form": "sift_cuda_detect_and_compute_view, pinned host image, results read in place"},
            "e2e_dropin": {"value": dropin_value, "unit": "images/s", "h2d_bytes_per_step": w * h,
                           "d2h_bytes_per_step": d2h,
                           "form": "pageable host image through sift_cuda_detect_and_compute: the library copies "
                                   "keypoints and descriptors into arrays the caller owns (and frees)"},
            "keypoints_per_s": {"device": value * int(nk), "e2e": e2e_value * int(nk)},
            "roofline": roof,
            "roofline_pyramid_dog": roof_pyr,
            "stages_ms": per_run,
            "gpu_launches": launches_per_step * args.steps,
            "clocks": clocks,
            "wall_s_timed": t_wall,
        }
        if world == 1 and not args.no_cpu_baseline:
            out["cpu_baseline"] = cpu_baseline(img, sargs, args.cpu_budget)
    eng.close()
    if args.workload == "1080p" and not args.no_4096:
        sec = pyramid_section("4096", local, args.storage, 2, 1, clocks.get("sm_mhz"))
        if rank == 0:
            out["pyramid_4096"] = sec
    if not args.no_serving:
        srv = serving_report(args.serve_requests, [1000, 2000, 4000], max_inflight=args.inflight, device=local)
        if rank == 0:
            out["serving"] = srv
    if rank == 0:
        print(json.dumps(out), flush=True)
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["cuda", "reference"], default="cuda")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + ["batch64", "serve", "match"], default="1080p")
    ap.add_argument("--storage", choices=["f32", "f16", "u8"], default="u8")
    ap.add_argument("--level-tile-rows", type=int, choices=[0, 32, 64], default=0,
                    help="rows of the fused level kernel's tiles (0: the default, 64)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-serving", action="store_true", help="skip the served-vs-plain section")
    ap.add_argument("--no-4096", action="store_true", help="skip the 4096x4096 pyramid section")
    ap.add_argument("--serve-requests", type=int, default=2000)
    ap.add_argument("--requests", type=int, default=20000, help="requests per rate (--workload serve)")
    ap.add_argument("--inflight", type=int, default=8, help="server: requests on the device at once")
    ap.add_argument("--autotune", action="store_true", help="server: tune launch shapes per image size")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "cuda" else args.warmup
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.workload == "batch64":
        run_batch64(args, world, rank, local)
    elif args.workload == "serve":
        run_serve(args, world, rank, local)
    elif args.workload == "match":
        run_match(args, world, rank, local)
    else:
        run_cuda(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
