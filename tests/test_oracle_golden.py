"""The oracle against the reference: golden vectors produced by the unmodified
reference (tests/golden/make_golden.py) and the known answers of the
reference's own unit tests (test/test_anchor.cpp, test/test_align.cpp,
test/test_consensus.cpp), restated here.  CPU only."""
import hashlib

import numpy as np
import pytest

from oracle.oracle import ANCHOR_DTYPE

MAT = np.array([5, -4, -4, -4, 0, -4, 5, -4, -4, 0, -4, -4, 5, -4, 0, -4, -4, -4, 5, 0, 0, 0, 0, 0, 0], np.int8)


def _ragged(z, name, i):
    off = z[name + "_off"]
    return z[name][off[i]:off[i + 1]]


def test_log2_table_matches_double_rounding(oracle):
    import math
    t = oracle.log2_table()
    for i in range(1, 513):
        assert np.float32(math.log2(i)) == t[i], i


def test_extz2_golden_vectors(oracle, golden):
    z = golden.load("ksw_extz2.npz")
    for i in range(len(z["params"])):
        w, zdrop, eb, flag = (int(x) for x in z["params"][i])
        ez, cig = oracle.ksw_extz2(_ragged(z, "q", i), _ragged(z, "t", i), 5, MAT, 6, 2, w, zdrop, eb, flag)
        assert np.array_equal(ez, z["ez"][i]), i
        assert np.array_equal(cig, _ragged(z, "cigar", i)), i


def test_stage_dumps_golden(oracle, golden, pkg):
    z = golden.load("mito_stages.npz")
    w = pkg.synth.mito(3)
    cx, cy = oracle.extract_minimizer(w.center)
    assert np.array_equal(cx, z["center_x"]) and np.array_equal(cy, z["center_y"])
    for j in range(3):
        qx, qy = oracle.extract_minimizer(w.query(j))
        assert np.array_equal(qx, z[f"q{j}_x"]) and np.array_equal(qy, z[f"q{j}_y"])
        a = oracle.collect_anchors(cx, cy, qx, qy)
        assert np.array_equal(a, z[f"q{j}_anchors"].astype(ANCHOR_DTYPE))
        srt, ch = oracle.chain_anchors(a)
        assert np.array_equal(srt, z[f"q{j}_sorted"].astype(ANCHOR_DTYPE))
        assert np.array_equal(ch, z[f"q{j}_chain"].astype(ANCHOR_DTYPE))


@pytest.mark.parametrize("name,n", [("mito", 1000), ("divergent", 40), ("uneven", 400), ("serve", 20)])
def test_workload_cigars_golden(oracle, golden, pkg, name, n):
    w = getattr(pkg.synth, name)(n)
    cx, cy = oracle.extract_minimizer(w.center)
    z = golden.load(f"{name}_cigars.npz")
    for j, i in enumerate(z["idx"]):
        got = oracle.align_query(w.center, cx, cy, w.query(int(i)))
        assert np.array_equal(got, _ragged(z, "cigar", j)), (name, int(i))


def test_aligned_fasta_identical_to_reference_cli(oracle, golden, pkg):
    w = pkg.synth.mito(1000)
    _, cigs = oracle.align_batch(w.center, w.center, w.seqs, w.offsets, nthreads=4)
    hdr = b">" + golden.meta["center_header"].encode() + b"\n" + w.center + b"\n"
    ins, non = [], []
    for i in range(w.n):
        rec = b">" + w.names[i].encode() + b"\n" + oracle.del_query(w.query(i), cigs[i]) + b"\n"
        (ins if oracle.has_insertion(cigs[i]) else non).append(rec)
    fa = hdr + b"".join(ins) + b"".join(non)
    assert len(fa) == golden.meta["mito1000_cli_fasta_bytes"]
    assert hashlib.sha256(fa).hexdigest() == golden.meta["mito1000_cli_fasta_sha256"]


# ---- known answers of the reference's unit tests (restated) ----

def _hit(h, pos, rid=0, strand=False, span=15):
    x = (h << 8) | span
    y = ((rid | (0x80000000 if strand else 0)) << 32) | pos
    return np.uint64(x), np.uint64(y)


def _hits(lst):
    xs = np.array([h[0] for h in lst], np.uint64)
    ys = np.array([h[1] for h in lst], np.uint64)
    return xs, ys


NOFILTER = (0.0, 10, 1000000, 0.0, 500)


def test_anchor_known_answers(oracle):
    rx, ry = _hits([_hit(0x123456, 100, span=20)])
    qx, qy = _hits([_hit(0x123456, 50, span=20)])
    a = oracle.collect_anchors(rx, ry, qx, qy, NOFILTER)
    assert len(a) == 1 and a[0]["pos_ref"] == 100 and a[0]["pos_qry"] == 50 and a[0]["span"] == 20
    assert a[0]["is_rev"] == 0 and a[0]["hash"] == 0x123456
    # strand XOR
    rx, ry = _hits([_hit(0xABCDEF, 200)])
    qx, qy = _hits([_hit(0xABCDEF, 80, strand=True)])
    assert oracle.collect_anchors(rx, ry, qx, qy, NOFILTER)[0]["is_rev"] == 1
    # one-to-many expansion
    rx, ry = _hits([_hit(0x555555, p) for p in (100, 200, 300)])
    qx, qy = _hits([_hit(0x555555, 50)])
    a = oracle.collect_anchors(rx, ry, qx, qy, NOFILTER)
    assert sorted(a["pos_ref"].tolist()) == [100, 200, 300] and set(a["pos_qry"].tolist()) == {50}
    # q_occ filter: 50 of 100 query hits share a hash, limit 10%
    rx, ry = _hits([_hit(0x888888, 100)])
    qx, qy = _hits([_hit(0x888888, i) for i in range(50)] + [_hit(0x999900 + i, i) for i in range(50)])
    assert len(oracle.collect_anchors(rx, ry, qx, qy, (0.0, 10, 1000000, 0.10, 500))) == 0
    # span = min, rid pass-through
    rx, ry = _hits([_hit(0xAAAAAA, 100, span=30)])
    qx, qy = _hits([_hit(0xAAAAAA, 50, span=20)])
    assert oracle.collect_anchors(rx, ry, qx, qy, NOFILTER)[0]["span"] == 20
    rx, ry = _hits([_hit(0xBBBBBB, 100, rid=2)])
    qx, qy = _hits([_hit(0xBBBBBB, 50, rid=3)])
    a = oracle.collect_anchors(rx, ry, qx, qy, NOFILTER)[0]
    assert a["rid_ref"] == 2 and a["rid_qry"] == 3
    # empty inputs
    e = np.zeros(0, np.uint64)
    assert len(oracle.collect_anchors(e, e, qx, qy)) == 0 and len(oracle.collect_anchors(rx, ry, e, e)) == 0


def _anchors(rows):
    a = np.zeros(len(rows), ANCHOR_DTYPE)
    for i, (h, r, q, rid, rev, span) in enumerate(rows):
        a[i] = (h, rid, r, 0, q, span, rev)
    return a


def test_chain_known_answers(oracle):
    base = [5000, 5000, 500, 25, 5000]
    _, ch = oracle.chain_anchors(_anchors([(1, 100, 50, 0, 0, 20)]), base + [1, 10])
    assert len(ch) == 1 and ch[0]["span"] == 20
    _, ch = oracle.chain_anchors(_anchors([(1, 100, 50, 0, 0, 20), (2, 150, 100, 0, 0, 20)]), base + [2, 30])
    assert len(ch) == 2 and ch[0]["pos_ref"] < ch[1]["pos_ref"]
    rows = [(1, 100, 50, 0, 0, 20), (2, 150, 100, 0, 0, 20), (5, 200, 150, 0, 0, 20),
            (3, 200, 150, 1, 0, 15), (4, 250, 200, 1, 0, 15)]
    _, ch = oracle.chain_anchors(_anchors(rows), base + [2, 20])
    assert ch[0]["rid_ref"] == 0 and len(ch) >= 2
    rows = [(1, 100, 50, 0, 0, 20), (2, 150, 100, 0, 0, 20), (6, 200, 150, 0, 0, 20),
            (3, 300, 250, 0, 1, 15), (4, 350, 300, 0, 1, 15)]
    _, ch = oracle.chain_anchors(_anchors(rows), base + [2, 20])
    assert ch[0]["is_rev"] == 0 and len(ch) >= 2
    _, ch = oracle.chain_anchors(_anchors([(1, 100, 50, 0, 0, 20), (2, 6000, 5500, 0, 0, 20)]), base + [1, 10])
    assert len(ch) == 1
    _, ch = oracle.chain_anchors(_anchors([(1, 100, 50, 0, 0, 20), (2, 250, 150, 0, 0, 20)]),
                                 [5000, 5000, 30, 25, 5000, 1, 10])
    assert len(ch) == 1
    rows = [(1, 100, 50, 0, 0, 20), (2, 150, 100, 0, 0, 20), (3, 200, 150, 0, 0, 20),
            (4, 10000, 5000, 0, 0, 15), (5, 10100, 5100, 0, 0, 15)]
    assert len(oracle.chain_anchors(_anchors(rows), base + [2, 20])[1]) == 3
    assert len(oracle.chain_anchors(_anchors([(1, 100, 50, 0, 0, 15), (2, 150, 100, 0, 0, 15)]),
                                    base + [3, 10])[1]) == 0
    assert len(oracle.chain_anchors(_anchors([(1, 100, 50, 0, 0, 5), (2, 150, 100, 0, 0, 5)]),
                                    base + [2, 50])[1]) == 0
    _, ch = oracle.chain_anchors(_anchors([(1, 100, 50, 0, 0, 20), (2, 200, 150, 0, 0, 25)]), base + [2, 30])
    assert ch["pos_ref"].tolist() == [100, 200] and ch["pos_qry"].tolist() == [50, 150]
    assert len(oracle.chain_anchors(np.zeros(0, ANCHOR_DTYPE))[1]) == 0


def test_align_and_cigar_known_answers(oracle):
    c = oracle.global_align_ksw2(b"ACGTACGTACGT", b"ACGTACGTACGT")
    assert oracle.cigar_str(c) == "12M"
    assert oracle.cigar_str(oracle.global_align_ksw2(b"", b"ACG")) == "3I"
    assert oracle.cigar_str(oracle.global_align_ksw2(b"ACGT", b"")) == "4D"
    assert len(oracle.global_align_ksw2(b"", b"")) == 0
    # projection: I removed, D becomes '-', M copies
    cig = np.array([3 << 4 | 0, 2 << 4 | 1, 2 << 4 | 2, 1 << 4 | 0], np.uint32)
    assert oracle.del_query(b"ACGTTA", cig) == b"ACG--A"
    assert oracle.has_insertion(cig) and not oracle.has_insertion(cig[[0, 2, 3]])


def test_consensus_known_answers(oracle):
    def pick(s):
        rows = np.frombuffer(b"".join(s), np.uint8).reshape(len(s), -1)
        cnt = oracle.count_rows(rows)
        return "".join(oracle.pick_consensus(cnt[c]) for c in range(rows.shape[1]))
    assert pick([b"ACGTA", b"ACGTA", b"-CGTA"]) == "ACGTA"      # gap majority ignored
    assert pick([b"A", b"C", b"G", b"T"]) == "A"                # tie -> A > C > G > T
    assert pick([b"---", b"---"]) == "AAA"                      # all gaps -> A
    assert pick([b"ACGTACGT"]) == "ACGTACGT"
    assert pick([b"U", b"U", b"A"]) == "U"
    assert pick([b"C", b"C", b"a"]) == "C" and pick([b"N", b"n", b"A"]) == "A"


def test_oracle_extz2_match_mismatch_golden(oracle, golden):
    """extz2 without KSW_EZ_GENERIC_SC (extendAlignKSW2's scoring) against the
    reference's own outputs: the 16-byte score blocks reach past the band end
    into the target copy's padding and the reversed query."""
    z = golden.load("ksw_extz2_ng.npz")
    bad = []
    for i in range(len(z["params"])):
        w, zdrop, eb, flag = (int(x) for x in z["params"][i])
        q = z["q"][z["q_off"][i]:z["q_off"][i + 1]]
        t = z["t"][z["t_off"][i]:z["t_off"][i + 1]]
        ez, cig = oracle.ksw_extz2(q, t, 5, MAT, 6, 2, w, zdrop, eb, flag)
        if not (np.array_equal(ez, z["ez"][i]) and np.array_equal(cig, z["cigar"][z["cigar_off"][i]:z["cigar_off"][i + 1]])):
            bad.append(i)
    assert not bad, f"{len(bad)} of {len(z['params'])} differ, first {bad[:5]}"
