"""In-tree build of libsiftcuda.so for sm_103a.

Each translation unit is compiled in parallel (nvcc for .cu, g++ for host-only
.cpp) and linked into ``sift_wgpu_gb300/libsiftcuda.so`` with the CUDA runtime
linked statically. The whole library is built with ``--fmad=false`` and
``-ffp-contract=off``: the pyramid and refinement stages reproduce the
reference CPU path bit for bit only when no multiply-add is fused.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libsiftcuda.so"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

CU_SOURCES = ["scan.cu", "pyramid.cu", "detect.cu", "describe.cu", "engine.cu", "server.cu", "convert.cu", "export.cu", "noalloc.cu", "match.cu", "draw.cu", "batch.cu"]
CPP_SOURCES = ["tables.cpp"]
HEADERS = ["sift_internal.cuh", "tables.h", "engine.h"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsiftcuda.so")


def _fingerprint() -> str:
    h = hashlib.sha256()
    h.update(ARCH.encode())
    for name in CU_SOURCES + CPP_SOURCES + HEADERS:
        h.update(name.encode())
        h.update((CSRC / name).read_bytes())
    h.update((PKG.parent / "include" / "sift_cuda.h").read_bytes())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile libsiftcuda.so if its sources changed; returns its path."""
    BUILD.mkdir(exist_ok=True)
    stamp = BUILD / "stamp"
    fp = _fingerprint()
    if not force and LIB.exists() and stamp.exists() and stamp.read_text() == fp:
        return LIB
    nvcc = _nvcc()
    inc = str(PKG.parent / "include")
    cu_flags = [ARCH, "-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-I", inc,
                "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr"]
    if verbose:
        cu_flags += ["-Xptxas", "-v"]
    cxx = shutil.which("g++") or "c++"
    jobs = []
    objs = []
    for src in CU_SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        jobs.append([nvcc, *cu_flags, "-c", str(CSRC / src), "-o", str(obj)])
    for src in CPP_SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        jobs.append([cxx, "-O2", "-fPIC", "-ffp-contract=off", "-std=c++17", "-I", inc,
                     "-c", str(CSRC / src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        list(ex.map(_run, jobs))
    tmp = BUILD / "libsiftcuda.so.tmp"
    _run([nvcc, ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs)])
    os.replace(tmp, LIB)
    stamp.write_text(fp)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
