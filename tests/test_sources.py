"""Structure of the pipeline's CUDA sources, checked on the CPU.

The pipeline's kernels are launched with programmatic stream serialization
(launch_chained): a kernel may be scheduled before the previous kernel in its
stream has finished, so each one must start with chain_wait() before it reads
or writes anything. A kernel that missed the wait, or a pipeline launch that
bypassed launch_chained, would race or lose the overlap without any visible
error, so both are pinned here.
"""
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "sift_wgpu_gb300" / "csrc"
PIPELINE = ["convert.cu", "pyramid.cu", "detect.cu", "scan.cu", "describe.cu", "export.cu"]


def kernels(src: str):
    """(name, first statement of the body) for every __global__ function."""
    for m in re.finditer(r"__global__\s+void\s+(?:__launch_bounds__\([^)]*\)\s+)?(\w+)\s*\(", src):
        # the signature's closing parenthesis: the first ") {" after the name
        close = src.index(") {", m.end())
        stmt = src[close + 3:].lstrip().split(";", 1)[0]
        yield m.group(1), stmt.strip()


def test_the_kernel_scan_sees_a_missing_wait():
    src = "__global__ void __launch_bounds__(256) k_a(int* p) {\n    chain_wait();\n    *p = 1;\n}\n" \
          "__global__ void k_b(int* p) {\n    *p = 2;\n}\n"
    assert list(kernels(src)) == [("k_a", "chain_wait()"), ("k_b", "*p = 2")]


def test_every_pipeline_kernel_waits_first():
    seen = 0
    for f in PIPELINE:
        src = (CSRC / f).read_text()
        for name, first in kernels(src):
            seen += 1
            assert first == "chain_wait()", f"{f}: {name} starts with `{first}`, not chain_wait()"
    assert seen >= 17


def test_pipeline_launches_are_chained():
    for f in PIPELINE:
        src = (CSRC / f).read_text()
        assert "<<<" not in src, f"{f}: a launch bypasses launch_chained"
        assert "launch_chained(" in src, f


def test_no_kernel_releases_dependents_early():
    """Released at their start, dependents of one octave's chain held SM
    slots that other octaves' kernels needed; nothing signals it now."""
    for f in PIPELINE + ["sift_internal.cuh"]:
        src = (CSRC / f).read_text()
        code = "\n".join(l.split("//")[0] for l in src.splitlines())
        assert "launch_dependents" not in code, f
