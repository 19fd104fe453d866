"""Speed of the CPU baseline: the oracle port against the unmodified
reference build (oracle/_ref), both running the align-to-center query loop
on the same mito queries with the same thread count, interleaved in
50-query blocks so machine drift hits both alike.  The port is the CPU
baseline on hosts where the reference cannot build (its KSW2 kernel is
SSE2-only), so it must not understate the reference's speed.  Runs where
the reference builds (x86-64)."""
import numpy as np


def _ratio(pkg, oracle, reference, threads, n=200, blk=50):
    w = pkg.synth.mito(n)
    tp = tr = 0.0
    for a in range(0, w.n, blk):
        b = min(a + blk, w.n)
        offs = w.offsets[a:b + 1] - w.offsets[a]
        seqs = w.seqs[w.offsets[a]:w.offsets[b]]
        tp += oracle.align_batch(w.center, w.center, seqs, offs, nthreads=threads)[0]
        tr += reference.align_batch(w.center, seqs, offs, nthreads=threads)[0]
    return tr / tp


def test_port_keeps_the_reference_speed(pkg, oracle, reference):
    r1 = _ratio(pkg, oracle, reference, 1)
    r4 = _ratio(pkg, oracle, reference, 4)
    print(f"port speed / reference speed: {r1:.3f} (1 thread), {r4:.3f} (4 threads)")
    # measured 0.96-0.98 on this path; the bound leaves room for timing noise
    assert r1 > 0.8 and r4 > 0.8, (r1, r4)
