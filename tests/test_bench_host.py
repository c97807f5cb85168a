"""Host-side logic of bench.py, checked on the CPU: the pyramid's algorithmic
bytes (the roofline numerator), the clock-sample parsing that decides whether
a run throttled, the seeded serving trace and the latency summaries."""
import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
import bench  # noqa: E402


def pyramid_bytes_restated(w, h, octaves, S, b):
    """u8 input once; octave o >= 1 reads its base as its u8 plane; every
    octave writes S+3 levels as u8 planes plus b bytes each (f32 4, f16 2,
    u8 storage 0)."""
    total, ow, oh = w * h, w, h
    for o in range(octaves):
        n = ow * oh
        total += (n if o else 0) + n * (S + 3) * b + n * (S + 3)
        ow, oh = ow // 2, oh // 2
    return total


@pytest.mark.parametrize("w,h,octs,b", [(1920, 1080, 4, 4), (4096, 4096, 6, 4), (4096, 4096, 6, 2), (512, 512, 4, 4),
                                        (333, 217, 4, 4), (4096, 4096, 6, 0)])
def test_pyramid_bytes(w, h, octs, b):
    assert bench.pyramid_bytes(w, h, octs, 3, b) == pyramid_bytes_restated(w, h, octs, 3, b)


def test_pyramid_bytes_headline_values():
    assert bench.pyramid_bytes(1920, 1080, 4, 3, 4) == 85_374_000
    assert bench.pyramid_bytes(4096, 4096, 6, 3, 4) == 693_288_960
    assert bench.pyramid_bytes(4096, 4096, 6, 3, 0) == 156_549_120


def test_fp32_ops_and_radii():
    """The blur radii follow the reference's 2^o-scaled increments, and the
    operation count is two per tap."""
    r0, radii = bench.blur_radii(6, 3)
    assert r0 == 4 and radii[0] == [3, 4, 4, 5, 7] and radii[5] == [79, 99, 125, 157, 198]
    n = 512 * 512
    taps = n * 2 * (9 + 7 + 9 + 9 + 11 + 15)
    assert bench.pyramid_fp32_ops(512, 512, 1, 3) == 2 * taps


class _DoneProc:
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


def _stopped(lines):
    s = bench.ClockSampler(0)
    s.proc, s.lines = _DoneProc(), lines
    return s.stop()


def test_clock_samples_parse(monkeypatch):
    monkeypatch.setattr(bench.time, "sleep", lambda s: None)
    idle = "Not Active"
    r = _stopped([f"2070, 2070, 900.5, 0x0, {idle}, {idle}, {idle}, {idle}",
                  f"2055, 2070, 1100.0, 0x4, {idle}, {idle}, {idle}, Active",
                  "garbage line",
                  f"2070, 2070, 1200.0, 0x0, {idle}, {idle}, {idle}, {idle}"])
    assert r["samples"] == 3 and r["sm_mhz"] == 2070.0 and r["sm_max_mhz"] == 2070.0
    assert r["reasons"] == ["sw_power_cap"]
    r = _stopped([f"1500, 2070, 1390.0, 0x40, {idle}, Active, {idle}, {idle}"])
    assert r["reasons"] == ["hw_thermal_slowdown"]


def test_clock_sampler_without_nvidia_smi():
    s = bench.ClockSampler(0)
    assert s.stop() == {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}


def test_serve_trace_is_seeded_and_consistent():
    size_of = np.repeat(np.arange(len(bench.SERVE_MIX)), 4)  # a pool of 4 images per resolution
    a1, i1, s1 = bench.serve_trace(5000, 1000.0, size_of)
    a2, i2, s2 = bench.serve_trace(5000, 1000.0, size_of)
    assert np.array_equal(a1, a2) and np.array_equal(i1, i2) and np.array_equal(s1, s2)
    assert np.all(np.diff(a1) >= 0) and abs(a1[-1] - 5.0) < 0.5  # Poisson at 1000/s
    assert np.array_equal(size_of[i1], s1)  # each request uses an image of its resolution
    share = np.bincount(s1, minlength=len(bench.SERVE_MIX)) / len(s1)
    assert np.allclose(share, [p for _, p in bench.SERVE_MIX], atol=0.03)
    a0, _, _ = bench.serve_trace(100, 0.0, size_of)  # all due at once
    assert np.all(a0 == 0)


def test_latency_summary():
    lat = np.arange(1, 101) / 1e3  # 1..100 ms
    sizes = np.where(np.arange(100) % 2 == 0, 2, 0)  # even requests are 1920x1080
    r = bench.lat_summary(lat, sizes)
    assert r["p50_ms"] == pytest.approx(50.5) and r["p99_ms"] == pytest.approx(99.01)
    assert r["mean_ms"] == pytest.approx(50.5)
    assert r["p50_1080p_ms"] == pytest.approx(np.percentile(np.arange(1, 101, 2), 50))


def test_measured_peaks_come_from_the_measured_file():
    peak, kind = bench.measured_peaks()
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        assert kind == "measured" and peak == float(json.loads(p.read_text())["hbm_gbs"])
    else:
        assert kind == "fallback"


def test_traffic_figures_exist_for_the_bench_workloads():
    # figures come from scoped ncu captures; a stage that was not captured
    # reports null, the dominant stage of both workloads must be there
    for kind in ("dram_bytes", "inst"):
        for wl in ("1080p", "4096"):
            for stage in ("pyramid_dog", "extrema_refine", "orientation", "descriptor"):
                t = bench.traffic_from_profiles(wl, stage, kind)
                assert t is None or (isinstance(t, int) and t > 0), (kind, wl, stage)
    assert bench.traffic_from_profiles("1080p", "descriptor") > 0
    assert bench.traffic_from_profiles("1080p", "descriptor", "inst") > 0
    assert bench.traffic_from_profiles("4096", "descriptor", "inst") > 0


def test_issue_roofline():
    r = bench.issue_roofline(1.258e9, 2.0, 2070.0)  # 1.258 G warp instructions in 2 ms
    assert r["bound"] == "issue" and r["peak"] == pytest.approx(152 * 4 * 2.07)
    assert r["achieved"] == pytest.approx(629.0) and r["frac"] == pytest.approx(629.0 / (152 * 4 * 2.07))
    assert bench.issue_roofline(None, 2.0, 2070.0) is None and bench.issue_roofline(1e9, 2.0, None) is None
