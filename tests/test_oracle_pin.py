"""Pin the oracle against the unmodified reference sources (oracle/_ref).

Runs only where the reference tree is available and builds (x86-64; the
reference's KSW2 is SSE2-only).  Random inputs with fixed seeds; every
comparison is exact."""
import numpy as np
import pytest

from oracle.oracle import ANCHOR_DTYPE

MAT = np.array([5, -4, -4, -4, 0, -4, 5, -4, -4, 0, -4, -4, 5, -4, 0, -4, -4, -4, 5, 0, 0, 0, 0, 0, 0], np.int8)
M64 = (1 << 64) - 1


def _splitmix(x):
    x = (x + 0x9E3779B97F4A7C15) & M64
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & M64
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & M64
    return x ^ (x >> 31)


def _code(s, k):
    c = 0
    for ch in s[-k:]:
        c = (c << 2) | "ACGT".index(ch)
    return c


def increasing_run(rng, k, run):
    """A sequence holding `run` consecutive strictly increasing k-mer hashes
    (run >= w makes the reference's window deque overflow)."""
    s = "".join("ACGT"[i] for i in rng.integers(0, 4, 200))

    def h_of(x):
        return _splitmix(_code(x, k)) >> 8

    def low_start(x):
        while h_of(x) > (1 << 50):
            x += "ACGT"[rng.integers(0, 4)]
        return x

    s = low_start(s)
    h, got, steps = h_of(s), 0, 0
    while got < run:
        steps += 1
        if steps > 20000:
            return None
        up = [(h_of(s + b), b) for b in "ACGT" if h_of(s + b) > h]
        if not up:
            s = low_start(s + "ACGT"[rng.integers(0, 4)])
            h, got = h_of(s), 0
            continue
        h, b = min(up)
        s += b
        got += 1
    dn = [(h_of(s + b), b) for b in "ACGT" if h_of(s + b) < h]
    s += min(dn)[1] if dn else "A"
    return s + "".join("ACGT"[i] for i in rng.integers(0, 4, 150))


def test_minimizers_fuzz(oracle, reference):
    rng = np.random.default_rng(3)
    alphabet = np.frombuffer(b"ACGTACGTACGTACGTNacgtU-", np.uint8)
    for it in range(150):
        n = int(rng.integers(0, 12000))
        s = np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, n)].copy()
        if it % 3 == 0 and n:
            m = rng.random(n) < 0.02
            s[m] = alphabet[rng.integers(0, len(alphabet), int(m.sum()))]
        k = int(rng.choice([15, 11, 21, 31, 5]))
        w = int(rng.choice([10, 40, 255, 10]))
        for nc in (True, False):
            o = oracle.extract_minimizer(s.tobytes(), k, w, nc)
            assert oracle.last_ring_oob() == 0
            r = reference.extract_minimizer(s.tobytes(), k, w, nc)
            assert np.array_equal(o[0], r[0]) and np.array_equal(o[1], r[1]), (it, n, k, w, nc)


def test_minimizer_deque_overflow(oracle, reference):
    """w+1 strictly increasing hashes overflow RingMinQueue; cases that stay in
    bounds of its vector must match the reference exactly."""
    rng = np.random.default_rng(11)
    tested = 0
    for it in range(120):
        k = int(rng.choice([15, 21]))
        w = int(rng.choice([10, 12, 16]))
        s = increasing_run(rng, k, w + int(rng.integers(0, 3)))
        if s is None:
            continue
        o = oracle.extract_minimizer(s, k, w, True)
        if oracle.last_ring_oob():
            continue  # the reference would write past its buffer (undefined)
        r = reference.extract_minimizer(s, k, w, True)
        assert np.array_equal(o[0], r[0]) and np.array_equal(o[1], r[1]), it
        tested += 1
    assert tested >= 50


def test_extz2_fuzz(oracle, reference):
    rng = np.random.default_rng(1)
    for it in range(3000):
        ql, tl = int(rng.integers(1, 150)), int(rng.integers(1, 150))
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
        a = oracle.ksw_extz2(q, t, 5, MAT, 6, 2, w, zdrop, eb, flag)
        b = reference.ksw_extz2(q, t, 5, MAT, 6, 2, w, zdrop, eb, flag)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]), (it, ql, tl, w, flag)


def test_chain_score_and_anchors_fuzz(oracle, reference):
    rng = np.random.default_rng(7)
    # chain score over the whole linkable range (dd up to bw, dg up to 5000)
    for _ in range(3000):
        aj_r, aj_q = int(rng.integers(0, 10000)), int(rng.integers(0, 10000))
        ai_r, ai_q = aj_r + int(rng.integers(-10, 5200)), aj_q + int(rng.integers(-10, 5200))
        span = int(rng.integers(1, 40))
        ai_r, ai_q = max(ai_r, 0), max(ai_q, 0)
        assert oracle.chain_score(ai_r, ai_q, aj_r, aj_q, span) == reference.chain_score(ai_r, ai_q, aj_r, aj_q, span)
    # anchors + chains on random multi-rid / strand inputs
    for it in range(200):
        nr, nq = int(rng.integers(0, 400)), int(rng.integers(0, 400))
        hs = rng.integers(1, 60, max(nr, nq) + 1)
        rx = (hs[:nr].astype(np.uint64) << np.uint64(8)) | np.uint64(15)
        ry = (rng.integers(0, 3, nr).astype(np.uint64) << np.uint64(32)) | rng.integers(0, 20000, nr).astype(np.uint64)
        ry |= (rng.integers(0, 2, nr).astype(np.uint64) << np.uint64(63))
        qx = (rng.integers(1, 60, nq).astype(np.uint64) << np.uint64(8)) | np.uint64(15)
        qy = rng.integers(0, 20000, nq).astype(np.uint64) | (rng.integers(0, 2, nq).astype(np.uint64) << np.uint64(63))
        filt = None if it % 2 else (2e-4 * rng.integers(0, 200), 1, 30, 0.01 * rng.integers(0, 5), 7)
        a = oracle.collect_anchors(rx, ry, qx, qy, filt)
        b = reference.collect_anchors(rx, ry, qx, qy, filt)
        assert np.array_equal(a, b), it
        if len(a):
            sa, ca = oracle.chain_anchors(a, [5000, 5000, 500, 25, 5000, 1, 10])
            sb, cb = reference.chain_anchors(b, [5000, 5000, 500, 25, 5000, 1, 10])
            assert np.array_equal(ca, cb), it


def test_full_queries(oracle, reference, pkg):
    for name, n in (("mito", 12), ("divergent", 12), ("uneven", 40), ("serve", 6)):
        w = getattr(pkg.synth, name)(n)
        cx, cy = oracle.extract_minimizer(w.center)
        for i in range(w.n):
            a = oracle.align_query(w.center, cx, cy, w.query(i))
            b = reference.align_query_full(w.center, w.query(i))
            assert np.array_equal(a, b), (name, i)


def test_global_ksw2_and_mm2(oracle, reference):
    rng = np.random.default_rng(5)
    for it in range(60):
        r = np.frombuffer(b"ACGTN", np.uint8)[rng.integers(0, 5 if it % 5 == 0 else 4, int(rng.integers(0, 700)))]
        q = r.copy()
        if len(q):
            m = rng.random(len(q)) < 0.05
            q[m] = np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, int(m.sum()))]
        cut = int(rng.integers(0, 300))
        q = np.concatenate([q[: len(q) // 3], q[len(q) // 3 + cut:]])
        for flag in (-1, 0x04):
            assert np.array_equal(oracle.global_align_ksw2(r.tobytes(), q.tobytes(), flag),
                                  reference.global_align_ksw2(r.tobytes(), q.tobytes(), flag)), it
        rx, ry = oracle.extract_minimizer(r.tobytes())
        qx, qy = oracle.extract_minimizer(q.tobytes())
        an = oracle.collect_anchors(rx, ry, qx, qy)
        assert np.array_equal(oracle.global_align_mm2(r.tobytes(), q.tobytes(), an),
                              reference.global_align_mm2(r.tobytes(), q.tobytes(), an)), it
