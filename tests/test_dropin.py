"""HAlign-4's C++ call surface (include/halign4/*.h) through the drop-in
library libhalign4_dropin.so.

CPU: the library exports every function the headers declare, and the C++
test program compiles against the headers alone.  GPU: the program runs the
reference's known answers and the reference-generated golden cases
(tests/golden/dropin_cases.txt, the consensus files) through the library and
prints the single-call latency."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
BUILD = ROOT / "halign-4_gb300" / "_build"
SRC = ROOT / "tests" / "dropin" / "test_dropin.cpp"

# demangled names the drop-in library must define (the reference functions it replaces)
EXPORTS = [
    "minimizer::extractMinimizer(", "minimizer::collect_anchors(", "anchor::chainAnchors(",
    "anchor::compute_occ_cutoff_top_frac(", "anchor::compute_ref_occ_threshold(",
    "align::globalAlignKSW2(", "align::extendAlignKSW2(", "align::globalAlignMM2(",
    "cigar::cigarToInt(", "cigar::intToCigar(", "cigar::hasInsertion(", "cigar::cigarToString",
    "cigar::stringToCigar(", "cigar::padQueryToRefByCigar(", "cigar::delQueryToRefByCigar(",
    "cigar::appendCigar(", "cigar::getRefLength(", "cigar::getQueryLength(",
    "consensus::pickConsensusChar(", "consensus::writeConsensusFasta(", "consensus::writeCountsJson(",
    "consensus::generateConsensusSequence(", "ksw_extz2_sse",
    "mash::sketchFromSequence(", "mash::jaccard(", "mash::mashDistanceFromJaccard(", "mash::aniFromJaccard(",
    "mash::aniFromMashDistance(", "mash::intersectionSizeSortedUnique(",
]


def _binary(tmp: Path) -> Path:
    exe = tmp / "test_dropin"
    cxx = os.environ.get("CXX", "g++")
    subprocess.run([cxx, "-std=c++17", "-O1", f"-I{ROOT / 'include' / 'halign4'}", f"-I{ROOT / 'include'}",
                    str(SRC), "-o", str(exe), f"-L{BUILD}", "-lhalign4_dropin", "-lhalign_gb300",
                    f"-Wl,-rpath,{BUILD}"], check=True, capture_output=True, text=True)
    return exe


def test_dropin_library_exports_the_call_surface(native):
    lib = BUILD / "libhalign4_dropin.so"
    assert lib.exists()
    nm = shutil.which("nm")
    if nm is None:
        pytest.skip("nm not available")
    out = subprocess.run([nm, "-D", "-C", "--defined-only", str(lib)], check=True, capture_output=True,
                         text=True).stdout
    missing = [e for e in EXPORTS if e not in out]
    assert not missing, missing


def test_dropin_program_compiles_against_the_headers(native, tmp_path):
    assert _binary(tmp_path).exists()


@pytest.mark.gpu
def test_dropin_reference_answers_on_gpu(gpu, tmp_path):
    exe = _binary(tmp_path)
    scratch = tmp_path / "scratch"
    scratch.mkdir()
    r = subprocess.run([str(exe), str(ROOT / "tests" / "golden"), str(scratch)], capture_output=True, text=True,
                       timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "failed 0" in r.stdout


# the reference sources whose definitions the drop-in library replaces
REPLACED = ["minimizer", "anchor", "align", "cigar", "ksw2_extz2_sse", "consensus", "mash"]
# the rest of the reference CLI, linked unchanged
KEPT = ["halign4", "ref_aligner", "preprocess", "cmd", "selector", "seq_io", "file_io", "hash", "xxhash"]


def test_reference_cli_links_against_the_dropin(native, tmp_path):
    """The reference's own CLI objects (compiled from the unmodified sources
    by oracle/build.py, where the reference tree exists) link with
    libhalign4_dropin.so standing in for the seven replaced sources: every
    symbol the reference's callers need is defined by the drop-in."""
    obj = ROOT / "oracle" / "_ref" / "obj"
    if not all((obj / f"{n}.o").exists() for n in KEPT):
        pytest.skip("reference objects not built on this host")
    exe = tmp_path / "halign4_dropin"
    r = subprocess.run([os.environ.get("CXX", "g++"), "-fopenmp", "-o", str(exe), *[str(obj / f"{n}.o") for n in KEPT],
                        f"-L{BUILD}", "-lhalign4_dropin", "-lhalign_gb300", f"-Wl,-rpath,{BUILD}", "-lz"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    # and none of the replaced sources' objects was needed
    nm = subprocess.run(["nm", "-C", "--defined-only", str(exe)], capture_output=True, text=True).stdout
    for sym in ("minimizer::extractMinimizer(", "anchor::chainAnchors(", "align::globalAlignMM2(",
                "mash::sketchFromSequence(", "consensus::generateConsensusSequence("):
        assert sym not in nm, sym
