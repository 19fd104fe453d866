"""Multi-reference mode on the GPU: device MinHash sketches equal the oracle's
(and the reference's golden vectors), the device selection picks the
oracle's best reference, alignment to it (and the consensus re-check) gives
the oracle's CIGARs and rows, and the streamed FASTA of a multi-reference
run equals the reference CLI's byte for byte."""
import hashlib

import numpy as np
import pytest

from tests.test_mash_oracle import _ragged, multiref_fasta

pytestmark = pytest.mark.gpu


def _pack_list(gpu, seqs):
    offs = np.zeros(len(seqs) + 1, np.int64)
    np.cumsum([len(s) for s in seqs], out=offs[1:])
    return gpu.pack(b"".join(seqs), offs)


def test_sketch_batch_golden(gpu, golden):
    z = golden.load("mash_sketch.npz")
    for i, (k, sz, nc, sd) in enumerate(z["params"]):
        b = _pack_list(gpu, [_ragged(z, "seq", i).tobytes()])
        got = gpu.sketch_batch(b, int(k), int(sz), bool(nc), int(sd))[0]
        assert np.array_equal(got, _ragged(z, "sketch", i)), i


@pytest.mark.parametrize("k,sz,nc", [(15, 2000, True), (21, 500, True), (15, 2000, False), (9, 8192, True),
                                     (31, 1, True), (32, 100, True), (5, 2000, True)])
def test_sketch_batch_vs_oracle(gpu, oracle, k, sz, nc):
    rng = np.random.default_rng(k * 31 + sz)
    alpha = np.frombuffer(b"ACGTACGTACGTACGTNacgtUu", np.uint8)
    seqs = []
    for t in range(60):
        n = int(rng.choice([0, 4, k - 1, k, k + 3, 300, 2047, 2048, 2049, 5000, 16569, 29903]))
        n = max(n, 0)
        s = (alpha if t % 2 else alpha[:4])[rng.integers(0, len(alpha) if t % 2 else 4, n)].tobytes()
        if t % 6 == 0:
            s = (b"ACGTTGCAAG" * (n // 10 + 1))[:n]  # few distinct k-mers: the unlimited second sweep
        if t % 9 == 0 and n > 500:
            a = int(rng.integers(0, n - 300))
            s = s[:a] + b"N" * 250 + s[a + 250:]
        seqs.append(s)
    got = gpu.sketch_batch(_pack_list(gpu, seqs), k, sz, nc, 42)
    for i, s in enumerate(seqs):
        assert np.array_equal(got[i], oracle.sketch(s, k, sz, nc, 42)), i


def test_sketch_batch_rejects_oversize(gpu):
    b = _pack_list(gpu, [b"ACGT" * 100])
    with pytest.raises(gpu.HalignError):
        gpu.sketch_batch(b, 15, gpu.SKETCH_MAX + 1)


@pytest.fixture(scope="module")
def mr(gpu):
    from tests.pkgload import load_package
    w = load_package().synth.multiref(200)
    rs = gpu.RefSet(w.refs, max_queries=256, max_bases=4_000_000)
    return w, rs


def test_reference_sketches_and_consensus(gpu, oracle, mr):
    w, rs = mr
    for r, ref in enumerate(w.refs):
        assert np.array_equal(rs.sketch(r), oracle.sketch(ref))
    rows = np.frombuffer(b"".join(w.refs), np.uint8).reshape(len(w.refs), -1)
    cnt = oracle.count_rows(rows)
    cons = bytes(ord(oracle.pick_consensus(cnt[c])) for c in range(rows.shape[1]))
    assert rs.consensus() == cons


def test_select_vs_oracle_and_cli(gpu, oracle, golden, mr):
    w, rs = mr
    best, jac = rs.select(gpu.pack(w.seqs, w.offsets))
    sks = [oracle.sketch(r) for r in w.refs]
    for i in range(w.n):
        b, j = oracle.best_reference(oracle.sketch(w.query(i)), sks)
        assert best[i] == b and jac[i] == j, i
    assert best.tolist() == golden.meta["multiref200_best_ref"]


def test_select_ties_take_the_first_reference(gpu):
    from tests.pkgload import load_package
    w = load_package().synth.multiref(30, n_refs=3)
    refs = [w.refs[0], w.refs[1], w.refs[0]]  # references 0 and 2 identical
    rs = gpu.RefSet(refs, max_queries=64, max_bases=1_000_000)
    best, _ = rs.select(gpu.pack(w.seqs, w.offsets))
    assert 2 not in set(best.tolist())
    rs.close()


def test_align_keep_length_vs_oracle(gpu, oracle, mr):
    w, rs = mr
    res = rs.align(gpu.pack(w.seqs, w.offsets), keep_length=True)
    mz = [oracle.extract_minimizer(r) for r in w.refs]
    for i in range(w.n):
        b = int(res.best[i])
        c = oracle.align_query(w.refs[b], mz[b][0], mz[b][1], w.query(i))
        assert np.array_equal(res.cigar_of(i), c), i
        assert bool(res.has_ins[i]) == oracle.has_insertion(c)
        L = len(w.refs[b])
        assert res.rows[i, :L].tobytes() == oracle.del_query(w.query(i), c), i


def test_align_consensus_recheck_vs_oracle(gpu, oracle, mr):
    w, rs = mr
    cons = rs.consensus()
    res = rs.align(gpu.pack(w.seqs, w.offsets), keep_length=False, rows=False)
    cx, cy = oracle.extract_minimizer(cons)
    for i in range(0, w.n, 3):
        c = oracle.align_query(cons, cx, cy, w.query(i))
        assert np.array_equal(res.cigar_of(i), c), i


def test_align_fasta_multiref_equals_reference_cli(gpu, pkg, golden, oracle, tmp_path):
    w = pkg.synth.multiref(200)
    pkg.synth.write_refs_fasta(str(tmp_path / "refs.fa"), w.refs)
    pkg.synth.write_fasta(str(tmp_path), "unused", b"A", w)
    for chunk in (200, 37):
        out = tmp_path / f"out{chunk}.fa"
        n = gpu.align_fasta(tmp_path / "refs.fa", tmp_path / "queries.fa", out, chunk_queries=chunk)
        assert n == w.n
        data = out.read_bytes()
        assert len(data) == golden.meta["multiref200_cli_fasta_bytes"], chunk
        assert hashlib.sha256(data).hexdigest() == golden.meta["multiref200_cli_fasta_sha256"], chunk


def test_align_fasta_rejects_references_of_different_lengths(gpu, pkg, tmp_path):
    w = pkg.synth.multiref(5)
    pkg.synth.write_refs_fasta(str(tmp_path / "refs.fa"), [w.refs[0], w.refs[1][:-7]])
    pkg.synth.write_fasta(str(tmp_path), "unused", b"A", w)
    with pytest.raises(gpu.HalignError):
        gpu.align_fasta(tmp_path / "refs.fa", tmp_path / "queries.fa", tmp_path / "o.fa")


def test_build_center_and_align_equal_reference_cli(gpu, pkg, golden, oracle, tmp_path):
    """The CLI run without a center file: Top-K of the 40 longest queries,
    their consensus on the device, every query aligned to it; the FASTA
    equals the reference CLI's."""
    from tests.test_center_oracle import built_center
    w = pkg.synth.center_build()
    pkg.synth.write_fasta(str(tmp_path), "unused", b"A", w)
    assert gpu.build_center(tmp_path / "queries.fa", 40) == built_center(oracle, w, 40)
    for chunk in (200, 33):
        out = tmp_path / f"c{chunk}.fa"
        assert gpu.align_fasta_consensus(tmp_path / "queries.fa", out, cons_n=40, chunk_queries=chunk) == w.n
        data = out.read_bytes()
        assert len(data) == golden.meta["center_build_cli_fasta_bytes"], chunk
        assert hashlib.sha256(data).hexdigest() == golden.meta["center_build_cli_fasta_sha256"], chunk
    # a selection of records of different lengths needs the external MSA
    with pytest.raises(gpu.HalignError):
        gpu.build_center(tmp_path / "queries.fa", 41)
