"""Build the GB300 library in-tree: nvcc for sm_103a, one object per translation unit
(compiled in parallel), linked into curvami_gb300/libcurvami_gb300.so.

    python curvami-official_gb300/build.py [--force]
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "curvami_gb300")
LIB = os.path.join(OUT_DIR, "libcurvami_gb300.so")
PEAKS = os.path.join(OUT_DIR, "libcgb_peaks.so")
OBJ = os.path.join(HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
UNITS = ["shape", "pattern", "assemble", "capi", "noalloc", "batch"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(INCLUDE, "curvami_gb300.h"))
    return max(os.path.getmtime(f) for f in files)


def build(force: bool = False) -> str:
    if not force and all(os.path.exists(p) and os.path.getmtime(p) >= _deps() for p in (LIB, PEAKS)):
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    nvcc = _nvcc()
    procs = []
    for u in UNITS:
        obj = os.path.join(OBJ, u + ".o")
        cmd = [nvcc] + ARCH + FLAGS + ["-c", os.path.join(CSRC, u + ".cu"), "-o", obj]
        procs.append((u, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for u, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append(u)
            sys.stderr.write(out.decode(errors="replace"))
    if failed:
        raise RuntimeError(f"nvcc failed for: {', '.join(failed)}")
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + [os.path.join(OBJ, u + ".o") for u in UNITS]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    # The FMA-throughput probe used as the compute roofline denominator (benchmark only).
    tmp = PEAKS + ".tmp"
    subprocess.check_call([nvcc] + ARCH + FLAGS + ["-shared", "-o", tmp, os.path.join(CSRC, "pipe_peaks.cu")])
    os.replace(tmp, PEAKS)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
