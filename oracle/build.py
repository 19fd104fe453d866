"""Build recipe for the test oracle.

TEST INFRASTRUCTURE ONLY: builds the checker, never the product.

* ``build_oracle()`` compiles the C restatement ``oracle/halign_oracle.c``
  into ``oracle/_build/libhalign_oracle.so`` (portable C11 + OpenMP; builds on
  x86-64 and aarch64 alike).
* ``build_ref()`` compiles the UNMODIFIED HAlign-4 sources of the
  align-to-center path directly with g++/gcc (no CMake) together with
  ``oracle/ref_harness.cpp`` into ``oracle/_ref/libhalign_ref.so`` and links
  the reference CLI into ``oracle/_ref/halign4``.  It needs the reference tree
  (``REF_ROOT``, default ``/root/reference``) and an x86-64 host, because the
  reference's KSW2 kernel (src/align/ksw2_extz2_sse.c) only compiles under
  ``__SSE2__``.  When the tree is absent it does nothing.
"""
from __future__ import annotations

import os
import platform
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
REF_ROOT = Path(os.environ.get("HALIGN_REF_ROOT", "/root/reference"))

# Reference translation units on the align-to-center path (+ what they pull in
# for linking: file/seq I/O for consensus.cpp, the CLI driver for the golden
# end-to-end FASTA).
REF_LIB_CPP = [
    "seed/minimizer.cpp",
    "seed/anchor.cpp",
    "align/align.cpp",
    "align/cigar.cpp",
    "consensus/consensus.cpp",
    "utils/file_io.cpp",
    "utils/seq_io.cpp",
    "mash/mash.cpp",
    "mash/hash.cpp",
]
REF_CLI_CPP = [
    "halign4.cpp",
    "align/ref_aligner.cpp",
    "utils/preprocess.cpp",
    "utils/cmd.cpp",
    "consensus/selector.cpp",
]
REF_C = ["align/ksw2_extz2_sse.c", "mash/xxhash.c"]


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _newer(out: Path, inputs: list[Path]) -> bool:
    if not out.exists():
        return False
    t = out.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in inputs)


def build_oracle(force: bool = False) -> Path:
    """Compile the C restatement; returns the shared-library path."""
    BUILD.mkdir(exist_ok=True)
    out = BUILD / "libhalign_oracle.so"
    srcs = [HERE / "halign_oracle.c", HERE / "halign_oracle.h"]
    if force or not _newer(out, srcs):
        # -O3 as the reference's own build; -ffp-contract=off: the chain-score
        # penalty is float arithmetic that the reference evaluates without
        # fused multiply-add.
        _run(["gcc", "-std=c11", "-O3", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
              "-o", str(out), str(HERE / "halign_oracle.c"), "-lm"])
    return out


def ref_available() -> bool:
    return (REF_ROOT / "src" / "align" / "ksw2_extz2_sse.c").exists() and platform.machine() in ("x86_64", "AMD64")


def build_ref(force: bool = False) -> Path | None:
    """Compile the reference's own sources into oracle/_ref; None if unavailable."""
    if not ref_available():
        return None
    obj = REF_OUT / "obj"
    obj.mkdir(parents=True, exist_ok=True)
    lib = REF_OUT / "libhalign_ref.so"
    cli = REF_OUT / "halign4"
    src = REF_ROOT / "src"
    inc = [f"-I{REF_ROOT / 'include'}", f"-I{REF_ROOT / 'extern/CLI11/include'}",
           f"-I{REF_ROOT / 'extern/spdlog/include'}", f"-I{REF_ROOT / 'extern/cereal/include'}",
           f"-I{REF_ROOT / 'extern/WFA2-lib'}"]
    # The reference CLI is built with -O3 and no -march=native (its CMake
    # default), i.e. SSE2 only and no FMA contraction.
    jobs = []
    for rel in REF_LIB_CPP + REF_CLI_CPP:
        o = obj / (Path(rel).stem + ".o")
        jobs.append((["g++", "-std=c++20", "-O3", "-fPIC", "-fopenmp", *inc, "-c", str(src / rel), "-o", str(o)],
                     o, [src / rel]))
    for rel in REF_C:
        o = obj / (Path(rel).stem + ".o")
        jobs.append((["gcc", "-O3", "-fPIC", *inc, "-c", str(src / rel), "-o", str(o)], o, [src / rel]))
    h = obj / "ref_harness.o"
    jobs.append((["g++", "-std=c++20", "-O3", "-fPIC", "-fopenmp", *inc, "-c", str(HERE / "ref_harness.cpp"),
                  "-o", str(h)], h, [HERE / "ref_harness.cpp"]))
    todo = [j for j in jobs if force or not _newer(j[1], j[2])]
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(lambda j: _run(j[0]), todo))
    names = lambda rels: [str(obj / (Path(r).stem + ".o")) for r in rels]  # noqa: E731
    lib_objs = [str(h)] + names(REF_LIB_CPP) + [str(obj / "ksw2_extz2_sse.o"), str(obj / "xxhash.o")]
    if force or todo or not lib.exists():
        _run(["g++", "-shared", "-fopenmp", "-o", str(lib), *lib_objs, "-lz"])
    if force or todo or not cli.exists():
        _run(["g++", "-fopenmp", "-o", str(cli), *lib_objs, *names(REF_CLI_CPP), "-lz"])
    return lib


if __name__ == "__main__":
    print(build_oracle())
    print(build_ref())
