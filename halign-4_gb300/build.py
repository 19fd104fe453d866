"""Build the GB300 libraries.

* ``_build/libhalign_gb300.so`` from ``csrc/``: nvcc compiles every
  translation unit for sm_103a only (one -gencode, in parallel) and links one
  shared library exporting the C ABI of include/halign_gb300.h.
* ``_build/libhalign4_dropin.so`` from ``dropin/hg_shim.cpp``: g++ builds
  HAlign-4's C++ call surface (include/halign4/*.h) over that C ABI; it
  links libhalign_gb300.so and finds it next to itself.
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
DROPIN = BUILD / "libhalign4_dropin.so"
DROPIN_SRC = HERE / "dropin" / "hg_shim.cpp"
CXX = os.environ.get("CXX", "g++")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3", "-Xcompiler", "-fopenmp",
         f"-I{ROOT / 'include'}"]


def _sources():
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _headers():
    return sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted((ROOT / "include").glob("*.h"))


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
    build_dropin(force)
    return LIB


def build_dropin(force: bool = False) -> Path:
    """The C++ drop-in library over the C ABI (host code only)."""
    deps = [DROPIN_SRC, LIB, *sorted((ROOT / "include" / "halign4").glob("*.h")), ROOT / "include" / "halign_gb300.h"]
    if force or not DROPIN.exists() or DROPIN.stat().st_mtime < max(p.stat().st_mtime for p in deps):
        _run([CXX, "-std=c++17", "-O2", "-fPIC", "-shared", "-Wall", f"-I{ROOT / 'include'}", str(DROPIN_SRC),
              "-o", str(DROPIN), f"-L{BUILD}", "-lhalign_gb300", "-Wl,-rpath,$ORIGIN"])
    return DROPIN


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
