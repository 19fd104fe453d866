"""The serving loop's request-byte ring (halign-4_gb300/csrc/hg_ring.h) on
CPU: tests/ring_sim.cpp drives it the way hg_serve.cpp does - one writer
reserving, copying and publishing bursts; micro-batches reading the oldest
queued requests as runs of contiguous memory; batches finishing in any
order - and checks that no request wraps, every batch's runs hold exactly
its requests' bytes, no live byte is overwritten and an empty ring always
takes a request of half its size."""
import os
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def ring_sim(tmp_path_factory):
    exe = tmp_path_factory.mktemp("ring") / "ring_sim"
    cxx = os.environ.get("CXX", "g++")
    subprocess.run([cxx, "-std=c++17", "-O1", f"-I{ROOT / 'halign-4_gb300' / 'csrc'}", str(ROOT / "tests" / "ring_sim.cpp"),
                    "-o", str(exe)], check=True, capture_output=True, text=True)
    return exe


@pytest.mark.parametrize("seed", [1, 2, 3, 4, 5, 6])
def test_ring_keeps_live_requests_and_batch_runs(ring_sim, seed):
    r = subprocess.run([str(ring_sim), str(seed), "40000"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 failures" in r.stdout
