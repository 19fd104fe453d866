"""GPU parity: the CUDA path (through the C ABI) against the oracle and the
golden vectors the reference produced.  Integer work, so every comparison is
bit-exact (CIGAR words, ez fields, minimizer words, row bytes, counters)."""
import hashlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAT = np.array([5, -4, -4, -4, 0, -4, 5, -4, -4, 0, -4, -4, 5, -4, 0, -4, -4, -4, 5, 0, 0, 0, 0, 0, 0], np.int8)


def _ragged(z, name, i):
    off = z[name + "_off"]
    return z[name][off[i]:off[i + 1]]


def test_ksw_extz2_golden_vectors(gpu, golden):
    z = golden.load("ksw_extz2.npz")
    n = len(z["params"])
    bad = []
    for i in range(n):
        w, zdrop, eb, flag = (int(x) for x in z["params"][i])
        ez, cig = gpu.ksw_extz2(_ragged(z, "q", i), _ragged(z, "t", i), 5, MAT, 6, 2, w, zdrop, eb, flag)
        if not (np.array_equal(ez, z["ez"][i]) and np.array_equal(cig, _ragged(z, "cigar", i))):
            bad.append(i)
    assert not bad, f"{len(bad)} of {n} extz2 cases differ, first {bad[:5]}"


def test_ksw_extz2_large_banded_vs_oracle(gpu, oracle):
    rng = np.random.default_rng(5)
    for it in range(40):
        ql, tl = int(rng.integers(200, 900)), int(rng.integers(200, 900))
        q = rng.integers(0, 4, ql).astype(np.uint8)
        t = np.resize(q, tl).copy()
        m = rng.random(tl) < 0.1
        t[m] = rng.integers(0, 5, int(m.sum()))
        w = int(rng.choice([-1, 7, 33, 150, 400]))
        flag = int(rng.choice([0x04, 0x06, 0x86, 0x0E]))
        zdrop = int(rng.choice([-1, 100]))
        e1, c1 = oracle.ksw_extz2(q, t, 5, MAT, 6, 2, w, zdrop, 0, flag)
        e2, c2 = gpu.ksw_extz2(q, t, 5, MAT, 6, 2, w, zdrop, 0, flag)
        assert np.array_equal(e1, e2) and np.array_equal(c1, c2), (it, ql, tl, w, flag)


@pytest.mark.parametrize("non_canonical", [True, False])
def test_minimizers_vs_oracle(gpu, oracle, non_canonical):
    rng = np.random.default_rng(3)
    alphabet = np.frombuffer(b"ACGTACGTACGTACGTNacgtU-", np.uint8)
    for it in range(60):
        n = int(rng.integers(0, 9000))
        s = np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, n)].copy()
        if it % 3 == 0 and n:
            m = rng.random(n) < 0.02
            s[m] = alphabet[rng.integers(0, len(alphabet), int(m.sum()))]
        if it % 5 == 0 and n > 300:
            a = int(rng.integers(0, n - 200))
            s[a:a + int(rng.integers(1, 200))] = ord("N")
        k = int(rng.choice([15, 15, 11, 21, 31, 5]))
        w = int(rng.choice([10, 10, 1, 5, 40, 255]))
        ox, oy = oracle.extract_minimizer(s.tobytes(), k, w, non_canonical)
        gx, gy = gpu.extract_minimizer(s.tobytes(), k, w, non_canonical)
        assert np.array_equal(ox, gx) and np.array_equal(oy, gy), (it, n, k, w)


def test_minimizers_golden_stage(gpu, golden, pkg):
    z = golden.load("mito_stages.npz")
    w = pkg.synth.mito(3)
    cx, cy = gpu.extract_minimizer(w.center)
    assert np.array_equal(cx, z["center_x"]) and np.array_equal(cy, z["center_y"])
    for j in range(3):
        qx, qy = gpu.extract_minimizer(w.query(j))
        assert np.array_equal(qx, z[f"q{j}_x"]) and np.array_equal(qy, z[f"q{j}_y"])


def _assemble_fasta(w, res, header):
    ins = [i for i in range(w.n) if res.has_ins[i]]
    non = [i for i in range(w.n) if not res.has_ins[i]]
    parts = [b">" + header.encode() + b"\n" + w.center + b"\n"]
    for i in ins + non:
        parts.append(b">" + w.names[i].encode() + b"\n" + res.rows[i].tobytes() + b"\n")
    return b"".join(parts)


@pytest.fixture(scope="module")
def mito1000(gpu, pkg):
    w = pkg.synth.mito(1000)
    ix = gpu.Index(w.center)
    ctx = gpu.Context(ix, max_queries=600, max_bases=600 * 17000)  # two sub-batches
    res = ctx.align(gpu.pack(w.seqs, w.offsets), rows=True)
    return w, ix, ctx, res


def test_batch_mito_fasta_identical_to_reference_cli(mito1000, golden):
    w, ix, ctx, res = mito1000
    assert not res.status.any()
    fa = _assemble_fasta(w, res, golden.meta["center_header"])
    assert len(fa) == golden.meta["mito1000_cli_fasta_bytes"]
    assert hashlib.sha256(fa).hexdigest() == golden.meta["mito1000_cli_fasta_sha256"]


def test_batch_mito_cigars_golden_and_oracle(mito1000, golden, oracle):
    w, ix, ctx, res = mito1000
    z = golden.load("mito_cigars.npz")
    for j, i in enumerate(z["idx"]):
        assert np.array_equal(res.cigar_of(int(i)), _ragged(z, "cigar", j)), int(i)
    _, cigs = oracle.align_batch(w.center, w.center, w.seqs, w.offsets, nthreads=8)
    for i in range(w.n):
        assert np.array_equal(res.cigar_of(i), cigs[i]), i
        assert bool(res.has_ins[i]) == oracle.has_insertion(cigs[i])


def test_counters_match_rows(mito1000, oracle):
    w, ix, ctx, res = mito1000
    cnt, ins = ctx.counters()
    assert np.array_equal(cnt, oracle.count_rows(res.rows))
    ref_ins = np.zeros(ix.L + 1, np.uint32)
    for i in range(w.n):
        oracle.count_insertions(res.cigar_of(i), ix.L, ref_ins)
    assert np.array_equal(ins, ref_ins)
    # pickConsensusChar over the counters restores the center
    cons = bytes(ord(oracle.pick_consensus(cnt[c])) for c in range(ix.L))
    assert cons == w.center


@pytest.mark.parametrize("name,n", [("divergent", 40), ("uneven", 400), ("serve", 20)])
def test_batch_workloads_golden(gpu, pkg, golden, oracle, name, n):
    w = getattr(pkg.synth, name)(n)
    ix = gpu.Index(w.center)
    ctx = gpu.Context(ix, max_queries=n, max_bases=int(w.total_bases) + 1024)
    res = ctx.align(gpu.pack(w.seqs, w.offsets), rows=True)
    z = golden.load(f"{name}_cigars.npz")
    for j, i in enumerate(z["idx"]):
        assert np.array_equal(res.cigar_of(int(i)), _ragged(z, "cigar", j)), (name, int(i))
    for i in range(w.n):
        row = oracle.del_query(w.query(i), res.cigar_of(i))
        assert res.rows[i].tobytes() == row, (name, i)


def test_plain_form_equals_batched(gpu, pkg):
    w = pkg.synth.mito(24)
    ix = gpu.Index(w.center)
    ctx = gpu.Context(ix, max_queries=32, max_bases=32 * 17000)
    b = gpu.pack(w.seqs, w.offsets)
    r1 = ctx.align(b, rows=True)
    r2 = ctx.align(b, rows=True, plain=True)
    assert np.array_equal(r1.cigar_off, r2.cigar_off) and np.array_equal(r1.cigar, r2.cigar)
    assert np.array_equal(r1.rows, r2.rows) and np.array_equal(r1.has_ins, r2.has_ins)


def test_staged_equals_batched(gpu, pkg):
    w = pkg.synth.mito(64)
    ix = gpu.Index(w.center)
    ctx = gpu.Context(ix, max_queries=64, max_bases=64 * 17000)
    b = gpu.pack(w.seqs, w.offsets)
    r1 = ctx.align(b, rows=True)
    ctx.stage(b)
    ctx.run_staged()  # a new sub-batch shape: direct launches
    ctx.run_staged()  # seen before: captured into a graph and launched
    ctx.run_staged()  # replay of the captured graph
    r2 = ctx.fetch_staged(rows=True)
    assert np.array_equal(r1.cigar, r2.cigar) and np.array_equal(r1.rows, r2.rows)


def test_edge_cases_vs_oracle(gpu, oracle, pkg):
    rng = np.random.default_rng(9)
    center = pkg.synth.random_center(3000, 77)
    cmx, cmy = oracle.extract_minimizer(center)
    c = np.frombuffer(center, np.uint8)
    cases = [b"", b"A", b"ACGTACGTACGTAC", b"N" * 500, center, center + b"ACGTTTGA" * 40,
             center[:1000], center[2000:], center[100:140], b"acgt" + center[10:900].lower(),
             center[:500] + b"N" * 120 + center[620:1500], center[:700].replace(b"T", b"U"),
             np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, 800)].tobytes(),
             center[:1200] + center[1700:2600],
             # middle segment 1000 (center) vs 550 (unrelated): the band cannot reach
             # the segment end, so the segment becomes I(q)D(t)
             center[:1000] + np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, 550)].tobytes() + center[2000:],
             # chainless 1600 vs 3000: band-limited global alignment stops early (partial CIGAR)
             np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, 1600)].tobytes()]
    seqs = b"".join(cases)
    offs = np.concatenate([[0], np.cumsum([len(x) for x in cases])]).astype(np.int64)
    ix = gpu.Index(center)
    ctx = gpu.Context(ix, max_queries=64, max_bases=200000)
    res = ctx.align(gpu.pack(seqs, offs), rows=True, check=False)
    for i, q in enumerate(cases):
        want = oracle.align_query(center, cmx, cmy, q)
        assert np.array_equal(res.cigar_of(i), want), (i, oracle.cigar_str(want)[:120],
                                                        oracle.cigar_str(res.cigar_of(i))[:120])
        if not (res.status[i] & (pkg.ST_PARTIAL_CIGAR | pkg.ST_LENGTH_MISMATCH)):
            assert res.rows[i].tobytes() == oracle.del_query(q, want), i
    # the single-query entry point agrees with the batch
    for i in (2, 4, 9, 11):
        assert np.array_equal(ix.align_query(cases[i]), res.cigar_of(i))
    del c


def test_wavefront_tiers_vs_oracle(gpu, oracle, pkg):
    """Segments of the two wavefront tiers: long thin tails (one warp, 1-8
    columns per lane) and wide unbounded-band global alignments (16-warp CTA,
    1-8 columns per lane, several direction blocks), with and without N
    runs, in both orientations and both gap modes."""
    rng = np.random.default_rng(21)
    L = 12000
    center = pkg.synth.random_center(L, 31)
    cmx, cmy = oracle.extract_minimizer(center)
    acgt = np.frombuffer(b"ACGT", np.uint8)

    def rand(n):
        return acgt[rng.integers(0, 4, n)].tobytes()

    cases = []
    for a, n in ((100, 420), (5000, 515), (9000, 540)):   # < 100 minimizers: chainless
        cases.append(center[a:a + n])
    for n in (300, 700, 1100, 2100, 4000):                # unrelated: chainless, unbounded band
        cases.append(rand(n))
    cases.append(center[5000:5600])                       # long tails both sides
    cases.append(rand(40) + center[3000:6000])            # left tail 3000 x ~40
    cases.append(center[200:3000] + rand(90))             # right tail
    cases.append(center[:2000] + rand(300) + center[2000:4000])   # inserted block
    cases.append(center[:2000] + center[2250:5000])       # deleted block
    q = bytearray(center[1000:1510])
    q[100:160] = b"N" * 60
    cases.append(bytes(q))                                # chainless with an N run
    cases.append(center[7000:11000].lower())
    seqs = b"".join(cases)
    offs = np.concatenate([[0], np.cumsum([len(x) for x in cases])]).astype(np.int64)
    ix = gpu.Index(center)
    ctx = gpu.Context(ix, max_queries=64, max_bases=200000)
    res = ctx.align(gpu.pack(seqs, offs), rows=True, check=False)
    for i, qq in enumerate(cases):
        want = oracle.align_query(center, cmx, cmy, qq)
        assert np.array_equal(res.cigar_of(i), want), (i, len(qq), oracle.cigar_str(want)[:120],
                                                        oracle.cigar_str(res.cigar_of(i))[:120])
        if not (res.status[i] & (pkg.ST_PARTIAL_CIGAR | pkg.ST_LENGTH_MISMATCH)):
            assert res.rows[i].tobytes() == oracle.del_query(qq, want), i


def thin_cases(pkg, seed=5, L=12000):
    """Queries whose end segments are thin: a short side of 1..32 bases against
    up to ~12 kb of the other side, in both orientations, both gap modes, with
    plain and N-carrying ends."""
    rng = np.random.default_rng(seed)
    center = pkg.synth.random_center(L, 57)
    acgt = np.frombuffer(b"ACGT", np.uint8)

    def rand(n, alpha=acgt):
        return alpha[rng.integers(0, len(alpha), n)].tobytes()

    cases = []
    for _ in range(40):                                   # substrings with short random ends
        a = int(rng.integers(0, L - 300))
        b = int(min(L, a + rng.integers(200, 7000)))
        cases.append(rand(int(rng.integers(0, 14))) + center[a:b] + rand(int(rng.integers(0, 14))))
    for _ in range(8):                                    # query ends of 17..32 bases
        a = int(rng.integers(0, L - 3000))
        cases.append(rand(int(rng.integers(14, 30))) + center[a:a + 2500] + rand(int(rng.integers(14, 30))))
    for _ in range(10):                                   # N inside the short ends
        a = int(rng.integers(0, L - 3000))
        cases.append(rand(6, np.frombuffer(b"ACGTN", np.uint8)) + center[a:a + 2500] +
                     rand(9, np.frombuffer(b"ACGTN", np.uint8)))
    for s in (0, 2, 5, 8, 10, 12, 14, 16):                # long query ends against a short center end
        cases.append(rand(int(rng.integers(100, 3000))) + center[s:4000])
        cases.append(center[L - 4000:L - s] + rand(int(rng.integers(100, 3000))))
    for d in range(0, 16, 2):                             # inserted blocks: short center gap inside
        a = int(rng.integers(0, L - 3200))
        cases.append(center[a:a + 1500] + rand(int(rng.integers(35, 70))) + center[a + 1500 + d:a + 3000])
    cases.append(center[3000:9000].lower())
    return center, cases


def dp_center(raw: bytes) -> bytes:
    """The center the DP aligns against: the consensus of the single center
    record (pickConsensusChar: A/C/G/T/U of either case upper-cased, any other
    letter becomes A).  Minimizers still come from the raw center."""
    t = bytearray(b"A" * 256)
    for c in b"ACGTU":
        t[c] = t[c + 32] = c
    return raw.translate(bytes(t))


def test_thin_tier_vs_oracle(gpu, oracle, pkg):
    """Thin end segments (grouped wavefronts): every CIGAR and row equals the
    oracle's, on a plain center, one carrying N runs and one carrying U."""
    center, cases = thin_cases(pkg)
    c2 = bytearray(center)
    for a in (700, 4100, 8800):
        c2[a:a + 30] = b"N" * 30
    # U stays U in the DP center, a non-A/C/G/T code there
    c3 = center[:3000].replace(b"T", b"U") + center[3000:9000] + center[9000:].replace(b"T", b"U")
    for raw in (center, bytes(c2), c3):
        cmx, cmy = oracle.extract_minimizer(raw)
        cen = dp_center(raw)
        seqs = b"".join(cases)
        offs = np.concatenate([[0], np.cumsum([len(x) for x in cases])]).astype(np.int64)
        ix = gpu.Index(raw)
        ctx = gpu.Context(ix, max_queries=128, max_bases=len(seqs) + 1024)
        res = ctx.align(gpu.pack(seqs, offs), rows=True, check=False)
        for i, qq in enumerate(cases):
            want = oracle.align_query(cen, cmx, cmy, qq)
            assert np.array_equal(res.cigar_of(i), want), (i, len(qq), oracle.cigar_str(want)[:120],
                                                            oracle.cigar_str(res.cigar_of(i))[:120])
            if not (res.status[i] & (pkg.ST_PARTIAL_CIGAR | pkg.ST_LENGTH_MISMATCH)):
                assert res.rows[i].tobytes() == oracle.del_query(qq, want), i


def test_batch_window_overflow_vs_oracle(gpu, oracle, pkg):
    """Queries holding 10+ consecutive strictly increasing k-mer hashes at the
    default k=15, w=10: the reference's window deque overflows there, the
    tile pass must detect it and the sequential replay must reproduce the
    reference's minimizers (checked through the whole alignment)."""
    from tests.test_oracle_pin import increasing_run
    rng = np.random.default_rng(44)
    center = pkg.synth.random_center(6000, 8)
    cmx, cmy = oracle.extract_minimizer(center)
    cases = []
    for it in range(6):
        run = increasing_run(rng, 15, 10 + it % 3)
        assert run is not None
        a = int(rng.integers(0, 4000))
        cases.append(center[a:a + 800] + run.encode() + center[a + 800:a + 1800])
        if it < 2:  # exception bytes around the run: lowercase, an N run, U
            cases.append((center[a:a + 800] + run.encode() + center[a + 800:a + 1800]).lower())
            cases.append(center[a:a + 700] + b"N" * 40 + center[a + 740:a + 800] + run.encode() +
                         center[a + 800:a + 1800].replace(b"T", b"U"))
    cases.append(center[1000:5000])
    seqs = b"".join(cases)
    offs = np.concatenate([[0], np.cumsum([len(x) for x in cases])]).astype(np.int64)
    ix = gpu.Index(center)
    ctx = gpu.Context(ix, max_queries=16, max_bases=100000)
    res = ctx.align(gpu.pack(seqs, offs), rows=False, check=False)
    for i, q in enumerate(cases):
        assert np.array_equal(res.cigar_of(i), oracle.align_query(center, cmx, cmy, q)), i


def test_minimizer_replay_many_overflows_vs_oracle(gpu, oracle, pkg):
    """Several deque overflows per query, some a few k-mers apart (inside one
    32-base step of the replay, or before the ring is back to the ideal
    deque), with N runs between them: the replay's switches between its
    ideal and exact modes, through the single-call extraction and through
    the batched path's CIGARs."""
    from tests.test_oracle_pin import increasing_run
    rng = np.random.default_rng(52)
    center = pkg.synth.random_center(6000, 21)
    cmx, cmy = oracle.extract_minimizer(center)
    cases = []
    for it, (k, w) in enumerate([(15, 10), (15, 10), (15, 11), (11, 3), (21, 2), (15, 1), (13, 5), (15, 10)]):
        parts = [center[int(rng.integers(0, 3000)):][:int(rng.integers(0, 400))]]
        for r in range(int(rng.integers(2, 6))):
            run = increasing_run(rng, k, w + int(rng.integers(0, 3)))
            assert run is not None
            parts.append(run[-int(rng.integers(w + 20, 80)):].encode())
            if rng.random() < 0.3:
                parts.append(b"N" * int(rng.integers(1, 30)))
            parts.append(np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, int(rng.integers(0, 90)))].tobytes())
        s = b"".join(parts)
        ox, oy = oracle.extract_minimizer(s, k, w, True)
        gx, gy = gpu.extract_minimizer(s, k, w, True)
        assert np.array_equal(ox, gx) and np.array_equal(oy, gy), (it, k, w, len(s))
        if k == 15 and w == 10:
            cases.append(s)
    seqs = b"".join(cases)
    offs = np.concatenate([[0], np.cumsum([len(x) for x in cases])]).astype(np.int64)
    ix = gpu.Index(center)
    ctx = gpu.Context(ix, max_queries=16, max_bases=len(seqs) + 1024)
    res = ctx.align(gpu.pack(seqs, offs), rows=False, check=False)
    for i, q in enumerate(cases):
        assert np.array_equal(res.cigar_of(i), oracle.align_query(center, cmx, cmy, q)), i


def test_global_align_mm2_vs_oracle(gpu, oracle, pkg):
    """The single-call globalAlignMM2 with caller anchors (the anchors
    collect_anchors makes for each query, shuffled: the call sorts them as
    chainAnchors does), against the oracle's globalAlignMM2."""
    rng = np.random.default_rng(17)
    w = pkg.synth.divergent(6)
    ix = gpu.Index(w.center)
    cmx, cmy = oracle.extract_minimizer(w.center)
    center_dp = w.center  # uniform ACGT center: its consensus is itself
    for i in range(w.n):
        q = w.query(i)
        qx, qy = oracle.extract_minimizer(q)
        an = oracle.collect_anchors(cmx, cmy, qx, qy)
        an = an[rng.permutation(len(an))]
        want = oracle.global_align_mm2(center_dp, q, an)
        got = ix.global_align_mm2(q, an["pos_ref"], an["pos_qry"])
        assert np.array_equal(got, want), i
    # chainless: no anchors at all
    q = w.query(0)[:300]
    assert np.array_equal(ix.global_align_mm2(q, [], []), oracle.global_align_mm2(center_dp, q, an[:0]))


def test_global_align_ksw2_vs_oracle(gpu, oracle):
    rng = np.random.default_rng(2)
    for it in range(30):
        r = np.frombuffer(b"ACGTN", np.uint8)[rng.integers(0, 5 if it % 4 == 0 else 4, int(rng.integers(0, 400)))]
        q = r.copy()
        if len(q):
            m = rng.random(len(q)) < 0.05
            q[m] = np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, int(m.sum()))]
        q = np.concatenate([q[: len(q) // 2], np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, it)],
                            q[len(q) // 2 + it // 2:]])
        flag = -1 if it % 2 else 0x04
        assert np.array_equal(gpu.global_align_ksw2(r.tobytes(), q.tobytes(), flag),
                              oracle.global_align_ksw2(r.tobytes(), q.tobytes(), flag)), it


def _same_result(a, b, n):
    for i in range(n):
        assert np.array_equal(a.cigar_of(i), b.cigar_of(i)), i
    assert np.array_equal(a.status, b.status) and np.array_equal(a.has_ins, b.has_ins)
    assert np.array_equal(a.rows, b.rows)


def test_pipelined_sub_batches_equal_one_batch(gpu, pkg):
    """hg_align_batch over several sub-batches (inputs of the next uploaded
    while one computes, CIGARs compacted and copied out behind it) returns
    exactly what one sub-batch returns."""
    w = pkg.synth.uneven(600)
    b = gpu.pack(w.seqs, w.offsets)
    ix = gpu.Index(w.center)
    one = gpu.Context(ix, max_queries=w.n, max_bases=int(w.total_bases) + 1024).align(b, rows=True, check=False)
    lens = np.diff(w.offsets)
    sub = gpu.Context(ix, max_queries=130, max_bases=int(130 * lens.max()) + 1024)
    _same_result(sub.align(b, rows=True, check=False), one, w.n)
    _same_result(sub.align(b, rows=True, check=False), one, w.n)  # reused pipeline buffers and graphs


@pytest.mark.parametrize("cap", [700, 1300, 3000])
def test_host_path_edge_split_equals_staged(gpu, pkg, cap):
    """32 MB or more to move: the host-buffer call re-cuts its first and
    last sub-batches into small edge parts (four sub-batches: the first two
    and the last two; three or fewer: all of them), on two lanes with two
    row buffers each; CIGARs, flags and rows equal the device-resident
    run's."""
    w = pkg.synth.mito(2600)
    b = gpu.pack(w.seqs, w.offsets)
    ix = gpu.Index(w.center)
    ctx = gpu.Context(ix, max_queries=cap, max_bases=cap * 16700)
    got = ctx.align(b, rows=True, check=False)
    again = ctx.align(b, rows=True, check=False)  # reused buffers and graphs
    one = gpu.Context(ix, max_queries=w.n, max_bases=w.n * 16700)  # the whole batch as one sub-batch
    one.stage(b)
    one.run_staged()
    want = one.fetch_staged(rows=True)
    _same_result(got, want, w.n)
    _same_result(again, want, w.n)
    _same_result(ctx.align_ascii(w.seqs, w.offsets, rows=True, check=False), want, w.n)
    # one lane (two input slots, two row buffers), and no edge cut
    knobs = ctx.get_launch()
    for lanes, share in ((1, 10), (2, 0), (1, 0)):
        ctx.set_launch(knobs[:9] + [lanes, share])
        _same_result(ctx.align(b, rows=True, check=False), want, w.n)
        _same_result(ctx.align_ascii(w.seqs, w.offsets, rows=True, check=False), want, w.n)


def _ascii_cases(pkg, rng, center, n):
    """Queries with exception bytes of every kind: N runs, lower case, U,
    IUPAC codes, runs of alternating bytes, an exception at either end."""
    cases = []
    for i in range(n):
        a = int(rng.integers(0, len(center) - 3000))
        q = bytearray(center[a:a + int(rng.integers(1500, 3000))])
        kind = i % 6
        if kind == 1:
            p, r = int(rng.integers(0, len(q) - 60)), int(rng.integers(1, 60))
            q[p:p + r] = b"N" * r
        if kind == 2:
            q = bytearray(bytes(q).lower()) if i % 12 == 2 else bytearray(bytes(q[:700]).lower() + bytes(q[700:]))
        if kind == 3:
            for p in rng.integers(0, len(q), 12):
                q[int(p)] = b"RYKMSWBDHVNU"[int(rng.integers(0, 12))]
        if kind == 4:
            p = int(rng.integers(0, len(q) - 40))
            q[p:p + 40] = b"NANRNNRRNU" * 4
        if kind == 5:
            q[0:1] = b"n"
            q[-3:] = b"NNN"
        cases.append(bytes(q))
    return cases


@pytest.mark.parametrize("cap", [37, 1000])
def test_align_ascii_equals_packed_path(gpu, pkg, cap):
    """hg_align_ascii (bytes uploaded per sub-batch, packed and their
    exception runs listed on the device) returns exactly what hg_pack +
    hg_align_batch return: CIGARs, flags, status and rows (which carry the
    exception bytes back)."""
    rng = np.random.default_rng(61)
    center = pkg.synth.random_center(8000, 23)
    cases = _ascii_cases(pkg, rng, center, 180)
    seqs = b"".join(cases)
    offs = np.concatenate([[0], np.cumsum([len(x) for x in cases])]).astype(np.int64)
    ix = gpu.Index(center)
    ctx = gpu.Context(ix, max_queries=cap, max_bases=cap * 3000 + 1024)
    want = ctx.align(gpu.pack(seqs, offs), rows=True, check=False)
    for _ in range(2):
        _same_result(ctx.align_ascii(seqs, offs, rows=True, check=False), want, len(cases))
    got = ctx.align_ascii(seqs, offs, rows=False, check=False)
    for i in range(len(cases)):
        assert np.array_equal(got.cigar_of(i), want.cigar_of(i)), i


def test_align_ascii_empty_and_single(gpu, pkg, oracle):
    """hg_align_ascii with no query, one empty query among others, and a
    single query: the same results as the packed path."""
    center = pkg.synth.random_center(4000, 25)
    ix = gpu.Index(center)
    ctx = gpu.Context(ix, max_queries=8, max_bases=8 * 4100)
    res = ctx.align_ascii(b"", np.zeros(1, np.int64), rows=True)
    assert len(res.cigar_off) == 1 and res.cigar_off[0] == 0
    for cases in ([center[100:3900]], [b"", center[:2000], b"", center[1000:4000]]):
        seqs = b"".join(cases)
        offs = np.concatenate([[0], np.cumsum([len(x) for x in cases])]).astype(np.int64)
        _same_result(ctx.align_ascii(seqs, offs, rows=True, check=False),
                     ctx.align(gpu.pack(seqs, offs), rows=True, check=False), len(cases))


def test_align_ascii_exception_capacity(gpu, pkg):
    """More exception runs in a sub-batch than max_bases / 16 + 4096: a
    capacity error (no query reads past the run buffer), and the context
    aligns the next batch correctly."""
    rng = np.random.default_rng(62)
    center = pkg.synth.random_center(6000, 24)
    ix = gpu.Index(center)
    ctx = gpu.Context(ix, max_queries=40, max_bases=40 * 6000)
    bad = [b"NA" * 2500 + center[:1000] for _ in range(10)]  # 2,500 runs each, 25,000 > 19,096
    seqs = b"".join(bad)
    offs = np.concatenate([[0], np.cumsum([len(x) for x in bad])]).astype(np.int64)
    with pytest.raises(RuntimeError, match="exception runs"):
        ctx.align_ascii(seqs, offs, rows=True)
    cases = _ascii_cases(pkg, rng, center, 30)
    seqs = b"".join(cases)
    offs = np.concatenate([[0], np.cumsum([len(x) for x in cases])]).astype(np.int64)
    _same_result(ctx.align_ascii(seqs, offs, rows=True, check=False),
                 ctx.align(gpu.pack(seqs, offs), rows=True, check=False), len(cases))


def test_pipelined_cigar_overflow_copies_in_pieces(gpu, pkg, oracle):
    """Sub-batches whose CIGARs outgrow the compaction buffer (short unrelated
    queries against a long center: global alignments with many ops) are
    copied in pieces and still equal the oracle."""
    rng = np.random.default_rng(12)
    center = pkg.synth.random_center(3000, 5)
    cmx, cmy = oracle.extract_minimizer(center)
    acgt = np.frombuffer(b"ACGT", np.uint8)
    cases = [acgt[rng.integers(0, 4, 64)].tobytes() for _ in range(300)]
    seqs = b"".join(cases)
    offs = np.concatenate([[0], np.cumsum([len(x) for x in cases])]).astype(np.int64)
    ix = gpu.Index(center)
    ctx = gpu.Context(ix, max_queries=100, max_bases=100 * 64 + 64)
    res = ctx.align(gpu.pack(seqs, offs), rows=True, check=False)
    words = int(res.cigar_off[100])  # CIGAR words of the first sub-batch
    assert words > (100 * 64 + 64) // 4 + 1024  # more than the compaction buffer holds
    for i, q in enumerate(cases):
        assert np.array_equal(res.cigar_of(i), oracle.align_query(center, cmx, cmy, q)), i


def test_low_complexity_vs_oracle(gpu, oracle, pkg):
    """Repeats inside the minimizer window (equal hashes: the reference's
    latest-equal-wins ties, equal hash prefixes in the increase test) in the
    batched fast path: poly-A, short tandem repeats, and repeats spliced into
    center substrings."""
    rng = np.random.default_rng(31)
    center = pkg.synth.random_center(8000, 13)
    cmx, cmy = oracle.extract_minimizer(center)
    cases = [b"A" * 3000, b"AC" * 1500, b"ACG" * 1000, b"ACGTTTGA" * 400, b"AACCGGTTA" * 300]
    for period in (2, 3, 5, 7, 11, 13):
        unit = np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, period)].tobytes()
        a = int(rng.integers(0, 5000))
        cases.append(center[a:a + 1500] + unit * (600 // period) + center[a + 1500:a + 3000])
    seqs = b"".join(cases)
    offs = np.concatenate([[0], np.cumsum([len(x) for x in cases])]).astype(np.int64)
    ix = gpu.Index(center)
    ctx = gpu.Context(ix, max_queries=32, max_bases=len(seqs) + 1024)
    res = ctx.align(gpu.pack(seqs, offs), rows=False, check=False)
    for i, q in enumerate(cases):
        assert np.array_equal(res.cigar_of(i), oracle.align_query(center, cmx, cmy, q)), i


@pytest.mark.parametrize("chunk", [1000, 237])
def test_streamed_fasta_identical_to_reference_cli(gpu, pkg, golden, tmp_path, chunk):
    """FASTA files in, aligned FASTA out, streamed in chunks (the reader, the
    GPU and the writer overlapped): byte-identical to the reference CLI's
    output on the 1,000 mito queries, whatever the chunk size."""
    w = pkg.synth.mito(1000)
    pkg.synth.write_fasta(str(tmp_path), "center", w.center, w, "synthetic mito center seed0")
    out = tmp_path / "out.fa"
    n = gpu.align_fasta(tmp_path / "center.fa", tmp_path / "queries.fa", out, 15, 10, chunk)
    assert n == 1000
    data = out.read_bytes()
    assert len(data) == golden.meta["mito1000_cli_fasta_bytes"]
    assert hashlib.sha256(data).hexdigest() == golden.meta["mito1000_cli_fasta_sha256"]
