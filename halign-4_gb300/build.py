"""Build the GB300 library ``_build/libhalign_gb300.so`` from ``csrc/``.

nvcc compiles every translation unit for sm_103a only (one -gencode, in
parallel) and links one shared library exporting the C ABI of
include/halign_gb300.h and the C++ drop-in surface of include/*.h.
"""
from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIB = BUILD / "libhalign_gb300.so"
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3", "-Xcompiler", "-fopenmp",
         f"-I{ROOT / 'include'}"]


def _sources():
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _headers():
    return sorted(CSRC.glob("*.cuh")) + sorted((ROOT / "include").glob("*.h"))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(map(str, cmd)) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(force: bool = False, verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    srcs = _sources()
    hdr_t = max((p.stat().st_mtime for p in _headers()), default=0)
    jobs = []
    for s in srcs:
        o = BUILD / (s.stem + ".o")
        stale = force or not o.exists() or o.stat().st_mtime < max(s.stat().st_mtime, hdr_t)
        if stale:
            extra = ["-Xptxas", "-v"] if verbose else []
            jobs.append([NVCC, *ARCH, *FLAGS, *extra, "-c", str(s), "-o", str(o)])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        logs = list(ex.map(_run, jobs))
    if verbose:
        for lg in logs:
            print(lg)
    objs = [str(BUILD / (s.stem + ".o")) for s in srcs]
    if jobs or not LIB.exists():
        _run([NVCC, *ARCH, "-shared", "-o", str(LIB), *objs, "-lcudart", "-lgomp"])
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
