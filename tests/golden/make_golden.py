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
    ksw_vectors(R)
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
    for p in sorted(OUT.glob("*.npz")):
        print(p.name, os.path.getsize(p))


if __name__ == "__main__":
    main()
