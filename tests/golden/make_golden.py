"""Generate the golden fixtures in tests/golden from the UNMODIFIED reference.

Run here (where /root/reference exists and is x86-64):
    python tests/golden/make_golden.py

It builds oracle/_ref (the reference's own sources compiled by oracle/build.py),
runs the reference functions through oracle/ref_harness.cpp and the reference
CLI (oracle/_ref/halign4), and writes small .npz / .json fixtures.  The tests
replay them against the oracle and the GPU path where the reference is absent
(for example on the GPU host).
"""
from __future__ import annotations

import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from tests.pkgload import load_package  # noqa: E402

synth = load_package().synth
from oracle.oracle import Reference  # noqa: E402

OUT = Path(__file__).resolve().parent
MAT = np.array([5, -4, -4, -4, 0, -4, 5, -4, -4, 0, -4, -4, 5, -4, 0, -4, -4, -4, 5, 0, 0, 0, 0, 0, 0], np.int8)


def ragged(arrs, dtype):
    off = np.zeros(len(arrs) + 1, np.int64)
    np.cumsum([len(a) for a in arrs], out=off[1:])
    flat = np.concatenate([np.asarray(a, dtype) for a in arrs]) if arrs else np.zeros(0, dtype)
    return flat, off


def ksw_vectors(R: Reference, n=600, seed=11):
    rng = np.random.default_rng(seed)
    qs, ts, ezs, cigs, prm = [], [], [], [], []
    for it in range(n):
        ql = int(rng.integers(1, 160))
        tl = int(rng.integers(1, 160))
        q = rng.integers(0, 5 if it % 3 == 0 else 4, ql).astype(np.uint8)
        if it % 2 == 0:
            t = np.resize(q, tl).copy()
            m = rng.random(tl) < 0.1
            t[m] = rng.integers(0, 4, int(m.sum()))
        else:
            t = rng.integers(0, 4, tl).astype(np.uint8)
        w = int(rng.choice([-1, 0, 1, 3, 5, 10, 17, 30, 200]))
        flag = int(rng.choice([0x04, 0x06, 0x05, 0x07, 0x0C, 0x0E, 0x46, 0x44, 0x86, 0x1E]))
        zdrop = int(rng.choice([-1, -1, 10, 50]))
        eb = int(rng.choice([0, 5]))
        ez, c = R.ksw_extz2(q, t, 5, MAT, 6, 2, w, zdrop, eb, flag)
        qs.append(q), ts.append(t), ezs.append(ez), cigs.append(c), prm.append([w, zdrop, eb, flag])
    qf, qo = ragged(qs, np.uint8)
    tf, to = ragged(ts, np.uint8)
    cf, co = ragged(cigs, np.uint32)
    np.savez_compressed(OUT / "ksw_extz2.npz", q=qf, q_off=qo, t=tf, t_off=to, cigar=cf, cigar_off=co,
                        ez=np.array(ezs, np.int32), params=np.array(prm, np.int32))


def workload_cigars(R: Reference, name: str, w, idx):
    cigs, mx, my = [], [], []
    for i in idx:
        cigs.append(R.align_query_full(w.center, w.query(int(i))))
    cf, co = ragged(cigs, np.uint32)
    np.savez_compressed(OUT / f"{name}_cigars.npz", idx=np.asarray(idx, np.int64), cigar=cf, cigar_off=co)


def stages(R: Reference, w, idx):
    cx, cy = R.extract_minimizer(w.center)
    rec = {"center_x": cx, "center_y": cy}
    for j, i in enumerate(idx):
        q = w.query(int(i))
        qx, qy = R.extract_minimizer(q)
        a = R.collect_anchors(cx, cy, qx, qy)
        srt, ch = R.chain_anchors(a)
        rec[f"q{j}_x"], rec[f"q{j}_y"] = qx, qy
        rec[f"q{j}_anchors"] = a
        rec[f"q{j}_sorted"] = srt
        rec[f"q{j}_chain"] = ch
    rec["idx"] = np.asarray(idx, np.int64)
    np.savez_compressed(OUT / "mito_stages.npz", **rec)


def ksw_nongeneric_vectors(R: Reference, n=400, seed=12):
    """extz2 without KSW_EZ_GENERIC_SC (match/mismatch scoring, symbol m-1 the
    wildcard): the scoring extendAlignKSW2 uses."""
    rng = np.random.default_rng(seed)
    qs, ts, ezs, cigs, prm = [], [], [], [], []
    for it in range(n):
        ql = int(rng.integers(1, 200))
        tl = int(rng.integers(1, 200))
        q = rng.integers(0, 5 if it % 3 == 0 else 4, ql).astype(np.uint8)
        if it % 2 == 0:
            t = np.resize(q, tl).copy()
            m = rng.random(tl) < 0.12
            t[m] = rng.integers(0, 5, int(m.sum()))
        else:
            t = rng.integers(0, 4, tl).astype(np.uint8)
        w = int(rng.choice([-1, 0, 1, 3, 5, 10, 17, 30, 200]))
        flag = int(rng.choice([0x00, 0x02, 0x01, 0x40, 0x42, 0x52, 0x08, 0x82, 0x12]))
        zdrop = int(rng.choice([-1, -1, 10, 50, 200]))
        eb = int(rng.choice([0, 5, 50]))
        ez, c = R.ksw_extz2(q, t, 5, MAT, 6, 2, w, zdrop, eb, flag)
        qs.append(q), ts.append(t), ezs.append(ez), cigs.append(c), prm.append([w, zdrop, eb, flag])
    qf, qo = ragged(qs, np.uint8)
    tf, to = ragged(ts, np.uint8)
    cf, co = ragged(cigs, np.uint32)
    np.savez_compressed(OUT / "ksw_extz2_ng.npz", q=qf, q_off=qo, t=tf, t_off=to, cigar=cf, cigar_off=co,
                        ez=np.array(ezs, np.int32), params=np.array(prm, np.int32))


def _seq(rng, n, noisy=True):
    s = np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, n)].copy()
    if noisy and n:
        m = rng.random(n) < 0.02
        s[m] = np.frombuffer(b"NacgtU", np.uint8)[rng.integers(0, 6, int(m.sum()))]
    return s.tobytes()


def _mutate(rng, src: bytes, p=0.02):
    out = bytearray()
    for c in src:
        r = rng.random()
        if r < p / 2:
            continue
        if r < p:
            out += bytes([c]) + _seq(rng, int(rng.integers(1, 4)), False)
            continue
        out.append(c if rng.random() > p else b"ACGT"[int(rng.integers(0, 4))])
    return bytes(out)


def dropin_cases(R: Reference):
    """Inputs and the reference's outputs of the C++ call surface
    (include/halign4/*.h) for tests/dropin/test_dropin.cpp: one case per line,
    space-separated fields, integer lists as a count followed by the values,
    sequences as raw bytes.  The aligned FASTA and the consensus outputs of
    generateConsensusSequence are written next to it."""
    rng = np.random.default_rng(77)
    L = []
    arr = lambda v: " ".join([str(len(v))] + [str(int(x)) for x in v])  # noqa: E731

    def anchors_line(a):
        cols = [a[f] for f in ("hash", "rid_ref", "pos_ref", "rid_qry", "pos_qry", "span", "is_rev")]
        return str(len(a)) + "".join(" " + " ".join(str(int(c[i])) for c in cols) for i in range(len(a)))

    # extractMinimizer
    for it in range(8):
        s = _seq(rng, int(rng.integers(0, 3000)))
        k, w = int(rng.choice([15, 11, 21, 31])), int(rng.choice([10, 40, 16]))
        nc = int(it % 2 == 0)
        x, y = R.extract_minimizer(s, k, w, bool(nc))
        L.append(f"MZ {k} {w} {nc} {len(s)} {s.decode() if s else '-'} {arr(x)} {arr(y)}")
    # collect_anchors + chainAnchors on hits with several ids and both strands
    for it in range(5):
        ref = _seq(rng, int(rng.integers(2000, 6000)), False)
        qry = _mutate(rng, ref[int(rng.integers(0, 500)):])
        rx, ry = R.extract_minimizer(ref, 15, 10, True)
        qx, qy = R.extract_minimizer(qry, 15, 10, True)
        if it % 2:  # a second reference id and reverse strands on part of the hits
            ry = ry.copy()
            flip = rng.random(len(ry)) < 0.3
            ry[flip] ^= np.uint64(1) << np.uint64(63)
            ry[rng.random(len(ry)) < 0.2] += np.uint64(1) << np.uint64(32)
        fp = [float(rng.choice([2e-4, 0.05])), int(rng.choice([1, 10])), int(rng.choice([2, 1000000])),
              float(rng.choice([0.01, 0.0, 0.002])), int(rng.choice([500, 0, 3]))]
        a = R.collect_anchors(rx, ry, qx, qy, fp)
        L.append(f"CA {' '.join(repr(v) for v in fp)} {arr(rx)} {arr(ry)} {arr(qx)} {arr(qy)} {anchors_line(a)}")
        ip = [5000, 5000, int(rng.choice([500, 50])), int(rng.choice([25, 2])), int(rng.choice([5000, 30])),
              int(rng.choice([3, 1])), int(rng.choice([40, 10]))]
        fpp = [float(rng.choice([0.01, 0.05])), 0.01]
        srt, ch = R.chain_anchors(a, ip, fpp)
        L.append(f"CH {' '.join(map(str, ip))} {fpp[0]!r} {fpp[1]!r} {anchors_line(a)} {anchors_line(srt)} "
                 f"{anchors_line(ch)}")
        # globalAlignMM2 with these anchors (general shape) and with the
        # align-to-center shape
        c = R.global_align_mm2(ref, qry, a)
        L.append(f"MM {ref.decode()} {qry.decode()} {anchors_line(a)} {arr(c)}")
        a2 = R.collect_anchors(*R.extract_minimizer(ref), qx, qy)
        c2 = R.global_align_mm2(ref, qry, a2)
        L.append(f"MM {ref.decode()} {qry.decode()} {anchors_line(a2)} {arr(c2)}")
        # projections of the query by that CIGAR
        L.append(f"DQ {qry.decode()} {arr(c2)} {R.del_query(qry, c2).decode()}")
        L.append(f"PQ {qry.decode()} {arr(c2)} {R.pad_query(qry, c2).decode()}")
    # ksw_extz2_sse, generic and match/mismatch scoring
    for it in range(60):
        ql, tl = int(rng.integers(1, 300)), int(rng.integers(1, 300))
        q = rng.integers(0, 5, ql).astype(np.uint8)
        t = np.resize(q, tl).copy()
        m = rng.random(tl) < 0.1
        t[m] = rng.integers(0, 5, int(m.sum()))
        w = int(rng.choice([-1, 5, 30, 120]))
        flag = int(rng.choice([0x04, 0x06, 0x46, 0x00, 0x02, 0x52, 0x05]))
        zdrop = int(rng.choice([-1, 40]))
        eb = int(rng.choice([0, 50]))
        ez, c = R.ksw_extz2(q, t, 5, MAT, 6, 2, w, zdrop, eb, flag)
        L.append(f"KS {w} {zdrop} {eb} {flag} {arr(q)} {arr(t)} {arr(ez)} {arr(c)}")
    # globalAlignKSW2 (default and caller flags) and extendAlignKSW2
    for it in range(12):
        ref = _seq(rng, int(rng.integers(0, 400)))
        qry = _mutate(rng, ref) if it % 3 else _seq(rng, int(rng.integers(0, 300)))
        flag = int(rng.choice([-1, 0x04, 0x06]))
        c = R.global_align_ksw2(ref, qry, flag)
        L.append(f"GK {flag} {ref.decode() or '-'} {qry.decode() or '-'} {arr(c)}")
        if ref and qry:
            zd = int(rng.choice([200, 20]))
            L.append(f"EX {zd} {ref.decode()} {qry.decode()} {arr(R.extend_align_ksw2(ref, qry, zd))}")
    # CIGAR strings
    for it in range(6):
        c = R.global_align_ksw2(_seq(rng, 200), _seq(rng, 180))
        L.append(f"CS {arr(c)} {R.cigar_str(c)}")
    # mash::sketchFromSequence and jaccard (own generator: the cases above stay as they were)
    rs = np.random.default_rng(78)
    sks = []
    for it in range(10):
        s = _seq(rs, int(rs.choice([0, 20, 800, 3000])), noisy=it % 2 == 0)
        k, sz, nc, sd = int(rs.choice([15, 21, 32])), int(rs.choice([2000, 50, 1])), int(it % 3 != 2), int(
            rs.choice([42, 0]))
        h = R.sketch(s, k, sz, bool(nc), sd)
        L.append(f"SK {k} {sz} {nc} {sd} {len(s)} {s.decode() if s else '-'} {arr(h)}")
        if k == 15 and nc and sz == 2000 and sd == 42:
            sks.append(h)
    base = R.sketch(_seq(rs, 2500, False))
    for o in sks + [base[:300], np.zeros(0, np.uint64)]:
        L.append(f"JC 15 {arr(base)} {arr(o)} {R.jaccard(base, o)!r}")
    (OUT / "dropin_cases.txt").write_text("\n".join(L) + "\n")
    # generateConsensusSequence: batches of 3 (the reference skips one record
    # between full batches) and a record limit
    alpha = np.frombuffer(b"ACGTACGTACGTacgtUuNn-.XR", np.uint8)
    with open(OUT / "dropin_aln.fa", "wb") as f:
        for i in range(13):
            row = alpha[rng.integers(0, len(alpha), 41)].tobytes()
            f.write(b">r%d sample\n" % i + row[:25] + b"\n" + row[25:] + b"\n")
    for tag, limit, bs in (("b3", 0, 3), ("l5", 5, 4096)):
        R.generate_consensus(OUT / "dropin_aln.fa", OUT / f"dropin_cons_{tag}.fa", OUT / f"dropin_cons_{tag}.json",
                             limit, bs)


def mash_vectors(R: Reference, seed=21):
    """mash::sketchFromSequence / getHash2bit / jaccard outputs of the
    reference on sequences with N, lowercase and U, repetitive and short
    ones, several k, sketch sizes and seeds."""
    rng = np.random.default_rng(seed)
    seqs, prm, sks = [], [], []
    for it in range(48):
        n = int(rng.choice([0, 3, 14, 15, 40, 700, 2500, 9000]))
        s = _seq(rng, n, noisy=it % 2 == 0)
        if it % 5 == 0:
            s = (b"ACGTTGCAAG" * (n // 10 + 1))[:n]  # few distinct k-mers
        if it % 7 == 0 and n > 100:  # an N-run
            a = int(rng.integers(0, n - 60))
            s = s[:a] + b"N" * 50 + s[a + 50:]
        k = int(rng.choice([15, 15, 21, 5, 31, 32, 1]))
        sz = int(rng.choice([2000, 2000, 10, 1, 300, 8192]))
        nc = int(it % 4 != 3)
        sd = int(rng.choice([42, 0, 7]))
        seqs.append(np.frombuffer(s, np.uint8)), prm.append([k, sz, nc, sd]), sks.append(R.sketch(s, k, sz, bool(nc), sd))
    sf, so = ragged(seqs, np.uint8)
    kf, ko = ragged(sks, np.uint64)
    codes = rng.integers(0, 2**62, 64, dtype=np.int64).astype(np.uint64)
    hashes = np.array([[R.hash2bit(int(c), sd) for sd in (42, 0, 7, 2**31 - 1)] for c in codes], np.uint64)
    # jaccard over default sketches (one empty) and truncated ones
    base = [R.sketch(_seq(rng, 3000, False)) for _ in range(3)]
    base.append(R.sketch(b""))
    pairs = base + [base[0][:100], base[1][50:2000]]
    jf, jo = ragged(pairs, np.uint64)
    jac = np.array([[R.jaccard(a, b) for b in pairs] for a in pairs], np.float64)
    np.savez_compressed(OUT / "mash_sketch.npz", seq=sf, seq_off=so, params=np.array(prm, np.int64), sketch=kf,
                        sketch_off=ko, codes=codes, hashes=hashes, jac_sk=jf, jac_sk_off=jo, jaccard=jac)


def multiref_cli_digest(w):
    """The reference CLI in multi-reference mode (several records in -c) with
    --keep-length and an MSA command that copies its input."""
    d = Path(tempfile.mkdtemp(prefix="halign_golden_mr_"))
    try:
        synth.write_refs_fasta(str(d / "refs.fa"), w.refs)
        synth.write_fasta(str(d), "unused", b"A", w)
        cmd = [str(ROOT / "oracle/_ref/halign4"), "-i", str(d / "queries.fa"), "-o", str(d / "out.fa"), "-c",
               str(d / "refs.fa"), "--keep-length", "-p", "cp {input} {output}", "-t", "1",
               "--kmer-size", "15", "--kmer-window", "10", "-w", str(d / "wd"), "--save-workdir"]
        subprocess.run(cmd, check=True, capture_output=True)
        data = (d / "out.fa").read_bytes()
        # the reference each query was aligned to, from the SAM records' RNAME
        rname = {}
        for sam in ("thread0.sam", "thread0_insertion.sam"):
            for line in (d / "wd" / "result" / sam).read_text().splitlines():
                if line and not line.startswith("@"):
                    f = line.split("\t")
                    rname[f[0]] = int(f[2][3:])
        best = [rname[nm] for nm in w.names]
        return hashlib.sha256(data).hexdigest(), len(data), data.count(b"\n") // 2, best
    finally:
        shutil.rmtree(d, ignore_errors=True)


def center_cli_digest(w, cons_n=40):
    """The reference CLI without a center file (it builds the center from
    the --cons-n longest queries) with --keep-length and an MSA command that
    copies its input."""
    d = Path(tempfile.mkdtemp(prefix="halign_golden_cc_"))
    try:
        synth.write_fasta(str(d), "unused", b"A", w)
        cmd = [str(ROOT / "oracle/_ref/halign4"), "-i", str(d / "queries.fa"), "-o", str(d / "out.fa"),
               "--keep-length", "-p", "cp {input} {output}", "-t", "1", "--kmer-size", "15", "--kmer-window", "10",
               "--cons-n", str(cons_n), "-w", str(d / "wd")]
        subprocess.run(cmd, check=True, capture_output=True)
        data = (d / "out.fa").read_bytes()
        return hashlib.sha256(data).hexdigest(), len(data), data.count(b"\n") // 2
    finally:
        shutil.rmtree(d, ignore_errors=True)


def center_fixtures():
    w = synth.center_build()
    digest, nbytes, nrec = center_cli_digest(w)
    meta = json.loads((OUT / "meta.json").read_text())
    meta.update({"center_build_cli_fasta_sha256": digest, "center_build_cli_fasta_bytes": nbytes,
                 "center_build_cli_records": nrec,
                 "center_build_cli": "halign4 -i queries.fa -o out.fa --keep-length -p 'cp {input} {output}' -t 1 "
                                     "--kmer-size 15 --kmer-window 10 --cons-n 40 (no -c)"})
    (OUT / "meta.json").write_text(json.dumps(meta, indent=1) + "\n")


def mash_fixtures(R: Reference):
    mash_vectors(R)
    w = synth.multiref(200)
    digest, nbytes, nrec, best = multiref_cli_digest(w)
    meta = json.loads((OUT / "meta.json").read_text())
    meta.update({"multiref200_cli_fasta_sha256": digest, "multiref200_cli_fasta_bytes": nbytes,
                 "multiref200_cli_records": nrec, "multiref200_best_ref": best,
                 "multiref_cli": "halign4 -i queries.fa -o out.fa -c refs.fa --keep-length -p 'cp {input} {output}' "
                                 "-t 1 --kmer-size 15 --kmer-window 10 (four references of one length)"})
    (OUT / "meta.json").write_text(json.dumps(meta, indent=1) + "\n")


def cli_fasta_digest(w, threads=1):
    d = Path(tempfile.mkdtemp(prefix="halign_golden_"))
    try:
        synth.write_fasta(str(d), "center", w.center, w, "synthetic mito center seed0")
        cmd = [str(ROOT / "oracle/_ref/halign4"), "-i", str(d / "queries.fa"), "-o", str(d / "out.fa"), "-c",
               str(d / "center.fa"), "--keep-length", "-p", "cp {input} {output}", "-t", str(threads),
               "--kmer-size", "15", "--kmer-window", "10", "-w", str(d / "wd")]
        subprocess.run(cmd, check=True, capture_output=True)
        data = (d / "out.fa").read_bytes()
        return hashlib.sha256(data).hexdigest(), len(data), data.count(b"\n") // 2
    finally:
        shutil.rmtree(d, ignore_errors=True)


def main():
    R = Reference()
    if sys.argv[1:] == ["--dropin"]:  # only the C++-surface fixtures
        ksw_nongeneric_vectors(R)
        dropin_cases(R)
        return
    if sys.argv[1:] == ["--mash"]:  # only the multi-reference fixtures
        mash_fixtures(R)
        return
    if sys.argv[1:] == ["--center"]:  # only the center-construction fixture
        center_fixtures()
        return
    ksw_vectors(R)
    ksw_nongeneric_vectors(R)
    dropin_cases(R)
    mito = synth.mito(1000)
    workload_cigars(R, "mito", mito, np.arange(0, 1000, 10))
    stages(R, mito, [0, 1, 2])
    div = synth.divergent(40)
    workload_cigars(R, "divergent", div, np.arange(40))
    une = synth.uneven(400)
    # every query with an N-run plus a spread of the rest
    has_n = [i for i in range(une.n) if b"N" in une.query(i)]
    idx = sorted(set(has_n) | set(range(0, une.n, 20)))
    workload_cigars(R, "uneven", une, idx)
    srv = synth.serve(20)
    workload_cigars(R, "serve", srv, np.arange(20))
    digest, nbytes, nrec = cli_fasta_digest(mito)
    meta = {
        "mito1000_cli_fasta_sha256": digest,
        "mito1000_cli_fasta_bytes": nbytes,
        "mito1000_cli_records": nrec,
        "center_header": "center synthetic mito center seed0",
        "cli": "halign4 -i queries.fa -o out.fa -c center.fa --keep-length -p 'cp {input} {output}' -t 1 "
               "--kmer-size 15 --kmer-window 10",
        "uneven_with_n_runs": has_n,
    }
    (OUT / "meta.json").write_text(json.dumps(meta, indent=1) + "\n")
    mash_fixtures(R)
    center_fixtures()
    for p in sorted(OUT.glob("*.npz")):
        print(p.name, os.path.getsize(p))


if __name__ == "__main__":
    main()
