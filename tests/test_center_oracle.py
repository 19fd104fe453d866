"""Center construction (the reference CLI run without a center file): the
oracle's Top-K selection, consensus and alignment against that center give
the reference CLI's aligned FASTA byte for byte.  CPU only."""
import hashlib

import numpy as np

from tests.test_mash_oracle import _clean


def topk_longest(lens, k):
    """TopKLongestSelector (src/consensus/selector.cpp): the k longest
    records, ties to the earlier one, longest first."""
    return sorted(range(len(lens)), key=lambda i: (-lens[i], i))[:k]


def built_center(oracle, w, cons_n):
    sel = topk_longest([len(w.query(i)) for i in range(w.n)], cons_n)
    rows = np.stack([np.frombuffer(_clean(w.query(i)), np.uint8) for i in sel])
    cnt = oracle.count_rows(rows)
    return bytes(ord(oracle.pick_consensus(cnt[c])) for c in range(rows.shape[1]))


def center_fasta(oracle, w, cons_n):
    cons = built_center(oracle, w, cons_n)
    cx, cy = oracle.extract_minimizer(cons)
    ins, non = [], []
    for i in range(w.n):
        c = oracle.align_query(cons, cx, cy, w.query(i))
        rec = b">" + w.names[i].encode() + b"\n" + oracle.del_query(w.query(i), c) + b"\n"
        (ins if oracle.has_insertion(c) else non).append(rec)
    return b">consensus\n" + cons + b"\n" + b"".join(ins) + b"".join(non)


def test_topk_selects_the_longest_records(pkg):
    w = pkg.synth.center_build()
    sel = topk_longest([len(w.query(i)) for i in range(w.n)], 40)
    assert {len(w.query(i)) for i in sel} == {len(w.center)}


def test_center_build_fasta_identical_to_reference_cli(oracle, golden, pkg):
    w = pkg.synth.center_build()
    fa = center_fasta(oracle, w, 40)
    assert len(fa) == golden.meta["center_build_cli_fasta_bytes"]
    assert hashlib.sha256(fa).hexdigest() == golden.meta["center_build_cli_fasta_sha256"]
