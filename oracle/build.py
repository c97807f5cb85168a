"""Builds oracle/_build/libsiftoracle.so (test infrastructure only).

Same recipe as oracle/Makefile, callable from Python without make.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libsiftoracle.so"
FLAGS = ["-O2", "-fPIC", "-ffp-contract=off", "-std=c++17", "-pthread", "-shared"]


def build(force: bool = False) -> Path:
    src = HERE / "sift_oracle.cpp"
    hdr = HERE / "sift_oracle.h"
    fp = hashlib.sha256(src.read_bytes() + hdr.read_bytes() + " ".join(FLAGS).encode()
                        + os.uname().machine.encode()).hexdigest()
    stamp = HERE / "_build" / "stamp"
    if not force and LIB.exists() and stamp.exists() and stamp.read_text() == fp:
        return LIB
    LIB.parent.mkdir(exist_ok=True)
    cxx = shutil.which("g++") or "c++"
    tmp = LIB.with_suffix(".so.tmp")
    r = subprocess.run([cxx, *FLAGS, "-o", str(tmp), str(src)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    stamp.write_text(fp)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
