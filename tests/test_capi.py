"""C ABI checks that need no GPU: the library builds for sm_103a, exports every
entry point include/halign_gb300.h declares, packs inputs losslessly on the
host, and fails loudly (no CPU fallback) when no GPU is visible."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def _declared():
    text = (ROOT / "include" / "halign_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(hg_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(native):
    declared = _declared()
    assert len(declared) >= 20
    lib_path = Path(native._name)
    out = subprocess.run(["nm", "-D", "--defined-only", str(lib_path)], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (hg_[a-z0-9_]+)", out))
    missing = [s for s in declared if s not in exported]
    assert not missing, missing
    for s in declared:
        getattr(native, s)  # resolvable through ctypes


def test_library_is_built_for_sm103a(native):
    out = subprocess.run(["/usr/local/cuda/bin/cuobjdump", "--list-elf", native._name], capture_output=True,
                         text=True)
    if out.returncode != 0:
        pytest.skip("cuobjdump unavailable")
    assert "sm_103a" in out.stdout


def test_pack_roundtrip_and_exceptions(pkg, native):
    seqs = [b"ACGTACGTAC", b"", b"NNNNACGTnnU--ACGT", b"A" * 33, b"acgt", b"ACGTRYKM"]
    blob = b"".join(seqs)
    offs = np.concatenate([[0], np.cumsum([len(s) for s in seqs])]).astype(np.int64)
    p = pkg.pack(blob, offs)
    assert p.n == len(seqs)
    assert all(int(o) % 16 == 0 for o in p.poff)
    runs = p.exc.reshape(-1, 3)
    for i, s in enumerate(seqs):
        out = bytearray()
        for j in range(len(s)):
            out.append(b"ACGT"[(p.packed[p.poff[i] + j // 4] >> (2 * (j % 4))) & 3])
        for r in runs[p.exc_off[i]:p.exc_off[i + 1]]:
            out[r[0]:r[0] + r[1]] = bytes([r[2]]) * int(r[1])
        assert bytes(out) == s, i


def test_pack_single_pass_matches_sizing_protocol(pkg, native):
    """hg_pack with a packed buffer and no exception list packs in one pass and
    reports the run count through HG_ERR_CAPACITY; the sized second call and
    the sizing-first protocol give the same bytes and runs."""
    L = native
    rng = np.random.default_rng(3)
    seqs = []
    for i in range(200):  # >= 64 queries: the OpenMP loops run
        s = bytearray(rng.choice(list(b"ACGT"), int(rng.integers(0, 300))).astype(np.uint8).tobytes())
        if i % 5 == 0 and len(s) > 12:
            s[3:7] = b"NNNN"
            s[10] = ord("n")
        seqs.append(bytes(s))
    blob = b"".join(seqs)
    offs = np.concatenate([[0], np.cumsum([len(s) for s in seqs])]).astype(np.int64)
    buf = np.frombuffer(blob, np.uint8)
    n = len(seqs)
    P = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    pb, ne = C.c_int64(0), C.c_int64(0)
    assert L.hg_pack(P(buf), P(offs), n, None, 0, None, None, 0, None, C.byref(pb), C.byref(ne)) == 0
    assert ne.value > 0
    ref_packed = np.zeros(pb.value, np.uint8)
    ref_poff, ref_eoff = np.zeros(n, np.int64), np.zeros(n + 1, np.int64)
    ref_exc = np.zeros(3 * ne.value, np.int32)
    assert L.hg_pack(P(buf), P(offs), n, P(ref_packed), pb.value, P(ref_poff), P(ref_exc), ne.value, P(ref_eoff),
                     None, None) == 0
    packed = np.zeros(pb.value, np.uint8)
    poff, eoff = np.zeros(n, np.int64), np.zeros(n + 1, np.int64)
    ne1 = C.c_int64(0)
    assert L.hg_pack(P(buf), P(offs), n, P(packed), pb.value, P(poff), None, 0, P(eoff), None,
                     C.byref(ne1)) == 4  # HG_ERR_CAPACITY: runs present, no list given
    assert ne1.value == ne.value
    assert np.array_equal(packed, ref_packed) and np.array_equal(poff, ref_poff) and np.array_equal(eoff, ref_eoff)
    exc = np.zeros(3 * ne1.value, np.int32)
    assert L.hg_pack(P(buf), P(offs), n, P(packed), pb.value, P(poff), P(exc), ne1.value, P(eoff), None, None) == 0
    assert np.array_equal(exc, ref_exc)
    p = pkg.pack(blob, offs)  # the Python wrapper takes the single-pass route
    assert np.array_equal(p.packed[: pb.value], ref_packed) and np.array_equal(p.exc, ref_exc)
    assert np.array_equal(p.exc_off, ref_eoff)
    clean = np.concatenate([[0], np.cumsum([len(s) for s in seqs if b"N" not in s and b"n" not in s])])
    cblob = b"".join(s for s in seqs if b"N" not in s and b"n" not in s)
    q = pkg.pack(cblob, clean.astype(np.int64))
    assert q.exc_off[-1] == 0


def test_calls_fail_loudly_without_gpu(pkg, native):
    if pkg.device_count() > 0:
        pytest.skip("a GPU is visible")
    with pytest.raises(pkg.HalignError):
        pkg.Index(b"ACGT" * 100)
    with pytest.raises(pkg.HalignError):
        pkg.extract_minimizer(b"ACGT" * 100)
    with pytest.raises(pkg.HalignError):
        pkg.global_align_ksw2(b"ACGTACGT", b"ACGTACG")


def test_bad_arguments_rejected_on_host(pkg, native):
    L = native
    h = C.c_void_p()
    assert L.hg_index_create(b"ACGT", 4, 0, 10, None, C.byref(h)) == 2
    assert L.hg_index_create(b"ACGT", 4, 15, 300, None, C.byref(h)) == 2
    assert L.hg_ctx_create(None, 1, 1, C.byref(h)) == 2
    ez = np.zeros(10, np.int32)
    # a symbol outside the alphabet is refused before any device work
    bad = np.array([0, 1, 7, 2], np.uint8)
    r = L.hg_ksw_extz2(4, bad.ctypes.data, 4, np.zeros(4, np.uint8).ctypes.data, 5,
                       np.zeros(25, np.int8).ctypes.data, 6, 2, -1, -1, 0, 0x02, ez.ctypes.data, None, 0)
    assert r == -2
    assert b"symbol >= m" in L.hg_last_error()
    # hg_align_ascii: no context, missing buffers, or a negative query length
    offs = np.array([0, 8, 4], np.int64)
    seqs = np.frombuffer(b"ACGTACGT", np.uint8)
    out = np.zeros(64, np.uint32)
    coff = np.zeros(3, np.int64)
    assert L.hg_align_ascii(None, seqs.ctypes.data, offs.ctypes.data, 2, out.ctypes.data, 64, coff.ctypes.data,
                            None, None, 0, None) == 2
    assert L.hg_align_ascii(None, None, None, -1, None, 0, None, None, None, 0, None) == 2


def test_auto_band_matches_oracle(oracle):
    import itertools
    from tests.pkgload import load_package
    load_package()
    for a, b in itertools.product([1, 2, 7, 50, 199, 200, 201, 333, 1000, 5000, 16569], repeat=2):
        # the band formula is shared by the DP kernels (hg_common.cuh) and the host wrapper
        d = abs(a - b)
        mx = max(a, b)
        want = -1 if d / mx > 0.5 else 200 + int(0.1 * (a + b // 2))
        assert oracle.auto_band(a, b) == want
