"""Multi-reference mode in the oracle against the reference: MinHash sketches,
getHash2bit and jaccard against vectors made by the unmodified reference
(tests/golden/make_golden.py --mash), and the whole multi-reference
--keep-length run against the reference CLI's aligned FASTA.  CPU only."""
import hashlib

import numpy as np
import pytest


def _ragged(z, name, i):
    off = z[name + "_off"]
    return z[name][off[i]:off[i + 1]]


def test_hash2bit_golden(oracle, golden):
    z = golden.load("mash_sketch.npz")
    for c, row in zip(z["codes"], z["hashes"]):
        for sd, h in zip((42, 0, 7, 2**31 - 1), row):
            assert oracle.hash2bit(int(c), sd) == int(h)


def test_sketch_golden(oracle, golden):
    z = golden.load("mash_sketch.npz")
    for i, (k, sz, nc, sd) in enumerate(z["params"]):
        got = oracle.sketch(_ragged(z, "seq", i).tobytes(), int(k), int(sz), bool(nc), int(sd))
        assert np.array_equal(got, _ragged(z, "sketch", i)), i


def test_jaccard_golden(oracle, golden):
    z = golden.load("mash_sketch.npz")
    m = len(z["jac_sk_off"]) - 1
    for a in range(m):
        for b in range(m):
            assert oracle.jaccard(_ragged(z, "jac_sk", a), _ragged(z, "jac_sk", b)) == z["jaccard"][a, b]


def test_best_reference_first_of_ties(oracle):
    r = [np.array([1, 5, 9], np.uint64), np.array([1, 5, 9], np.uint64), np.array([2, 5], np.uint64)]
    assert oracle.best_reference(np.array([1, 5, 9], np.uint64), r) == (0, 1.0)
    assert oracle.best_reference(np.array([2, 5], np.uint64), r) == (2, 1.0)
    # an empty query sketch matches only an empty reference sketch
    assert oracle.best_reference(np.zeros(0, np.uint64), r + [np.zeros(0, np.uint64)]) == (3, 1.0)


def test_sketch_matches_reference_fuzz(oracle, reference):
    rng = np.random.default_rng(5)
    alpha = np.frombuffer(b"ACGTACGTACGTNacgtUuRY", np.uint8)
    for t in range(120):
        n = int(rng.integers(0, 4000))
        s = alpha[rng.integers(0, len(alpha), n)].tobytes()
        k = int(rng.choice([1, 9, 15, 24, 31, 32, 33]))
        sz = int(rng.choice([0, 1, 64, 2000, 6000]))
        nc = bool(t % 3)
        assert np.array_equal(oracle.sketch(s, k, sz, nc, 42), reference.sketch(s, k, sz, nc, 42)), t


def _clean(s: bytes) -> bytes:
    t = bytearray(b"N" * 256)
    for c in b"ACGTU":
        t[c] = c
        t[c + 32] = c
    t[ord("-")] = ord("-")
    return s.translate(bytes(t))


def multiref_fasta(oracle, w):
    """The multi-reference --keep-length output as the oracle computes it:
    the references (clean_table), then the rows with an insertion, then the
    others; each row projected onto the query's best reference."""
    sks = [oracle.sketch(r) for r in w.refs]
    mz = [oracle.extract_minimizer(r) for r in w.refs]
    ins, non, best = [], [], []
    for i in range(w.n):
        q = w.query(i)
        b, _ = oracle.best_reference(oracle.sketch(q), sks)
        c = oracle.align_query(w.refs[b], mz[b][0], mz[b][1], q)
        rec = b">" + w.names[i].encode() + b"\n" + oracle.del_query(q, c) + b"\n"
        (ins if oracle.has_insertion(c) else non).append(rec)
        best.append(b)
    hdr = b"".join(b">ref%d reference %d\n" % (r, r) + _clean(s) + b"\n" for r, s in enumerate(w.refs))
    return hdr + b"".join(ins) + b"".join(non), best


def test_multiref_fasta_identical_to_reference_cli(oracle, golden, pkg):
    w = pkg.synth.multiref(200)
    fa, best = multiref_fasta(oracle, w)
    assert best == golden.meta["multiref200_best_ref"]
    assert len(fa) == golden.meta["multiref200_cli_fasta_bytes"]
    assert hashlib.sha256(fa).hexdigest() == golden.meta["multiref200_cli_fasta_sha256"]
