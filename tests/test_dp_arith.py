"""The small-tier DP's int32 lane arithmetic equals the reference's SSE2 byte
sequence on every in-band cell (tests/dp_arith_equiv.c, compiled with gcc)."""
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent


def test_int32_lanes_equal_sse2_bytes(tmp_path):
    exe = tmp_path / "dp_arith_equiv"
    subprocess.run(["gcc", "-O2", "-o", str(exe), str(HERE / "dp_arith_equiv.c")], check=True)
    r = subprocess.run([str(exe), "20000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches=0" in r.stdout
