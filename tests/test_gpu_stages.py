"""Stage-level GPU parity of anchors and chains (collect_anchors and
chainAnchors), the single-call general forms behind the C++ drop-in, row
projection and SiteCount counting of caller rows.

Two kinds of checks:
* the batch kernels' own stage outputs (hg_fetch_chain after a staged run):
  the anchors the chain stage saw, the chain DP arrays f and p, and the best
  chain, against the reference's stage dumps (tests/golden/mito_stages.npz)
  and against the oracle on the mito, divergent and uneven samples, also with
  non-default seeding and chaining parameters;
* the general single calls (hg_collect_anchors, hg_chain_anchors) on hit and
  anchor lists with several sequence ids, both strands and mixed spans.
Everything is integer work: bit-exact comparisons."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _anchors_from_golden(z, name):
    a = z[name]
    out = np.zeros(len(a), dtype=[("hash", "<u8"), ("rid_ref", "<u4"), ("pos_ref", "<u4"), ("rid_qry", "<u4"),
                                  ("pos_qry", "<u4"), ("span", "<u4"), ("is_rev", "<u4")])
    for f in out.dtype.names:
        out[f] = a[f]
    return out


def test_collect_and_chain_match_reference_stage_dumps(gpu, golden):
    z = golden.load("mito_stages.npz")
    hits = gpu.Hits(z["center_x"], z["center_y"])
    for j in range(3):
        got = hits.collect(z[f"q{j}_x"], z[f"q{j}_y"])
        want = _anchors_from_golden(z, f"q{j}_anchors")
        assert len(got) == len(want)
        for f in want.dtype.names:
            assert np.array_equal(got[f], want[f]), (j, f)
        srt, chain, f_, p_ = gpu.chain_anchors(got)
        want_sorted = _anchors_from_golden(z, f"q{j}_sorted")
        want_chain = _anchors_from_golden(z, f"q{j}_chain")
        for f in want.dtype.names:
            assert np.array_equal(srt[f], want_sorted[f]), (j, f)
            assert np.array_equal(srt[chain][f], want_chain[f]), (j, f)


def _sorted_oracle_stage(oracle, center, qry, prm=None):
    """The oracle's collect_anchors + chainAnchors for one query against the
    center, with the same filter / chain parameters."""
    cx, cy = oracle.extract_minimizer(center)
    qx, qy = oracle.extract_minimizer(qry)
    fp = None if prm is None else (prm.f_top_frac, prm.u_floor, prm.u_ceil, prm.q_occ_frac, prm.sample_every_bp)
    anchors = oracle.collect_anchors(cx, cy, qx, qy, fp)
    ip = fpp = None
    if prm is not None:
        ip = [prm.max_dist_x, prm.max_dist_y, prm.bw, prm.max_skip, prm.max_iter, prm.min_cnt, prm.min_score]
        fpp = [prm.gap_penalty, prm.skip_penalty]
    srt, chain, f, p = oracle.chain_anchors_fp(anchors, ip, fpp)
    return anchors, srt, chain, f, p


CHAIN_PARAMS = [
    None,
    dict(gap_penalty=0.05, skip_penalty=0.02, bw=120, max_skip=3, max_iter=40, min_score=60, min_cnt=5),
    dict(max_dist_x=900, max_dist_y=700, bw=35, max_skip=0, max_iter=7, gap_penalty=0.3, skip_penalty=0.11),
    dict(q_occ_frac=0.001, sample_every_bp=7, f_top_frac=0.05, u_floor=1, u_ceil=2, max_skip=60, max_iter=200),
]


@pytest.mark.parametrize("name,n", [("mito", 24), ("divergent", 24), ("uneven", 40)])
@pytest.mark.parametrize("pi", range(len(CHAIN_PARAMS)))
def test_batch_anchor_and_chain_stage_vs_oracle(gpu, pkg, oracle, name, n, pi):
    """The batch kernels' anchors, f, p and best chain for every query of a
    staged sample, with default and non-default hg_params_t."""
    w = getattr(pkg.synth, name)(n)
    prm = None if CHAIN_PARAMS[pi] is None else gpu.params(**CHAIN_PARAMS[pi])
    ix = gpu.Index(w.center, prm=prm)
    ctx = gpu.Context(ix, max_queries=n, max_bases=int(w.total_bases) + 1024)
    ctx.stage(gpu.pack(w.seqs, w.offsets))
    ctx.run_staged()
    for i in range(w.n):
        got = ctx.fetch_chain(i)
        _, srt, chain, f, p = _sorted_oracle_stage(oracle, w.center, w.query(i), prm)
        assert np.array_equal(got["pos_ref"], srt["pos_ref"]), (i, "pos_ref")
        assert np.array_equal(got["pos_qry"], srt["pos_qry"]), (i, "pos_qry")
        assert np.array_equal(got["f"], f), (i, "f")
        assert np.array_equal(got["p"], p), (i, "p")
        # (pos_ref, pos_qry) is unique on one forward-strand center
        where = {(int(r), int(q)): k for k, (r, q) in enumerate(zip(srt["pos_ref"], srt["pos_qry"]))}
        idx = [where[(int(c["pos_ref"]), int(c["pos_qry"]))] for c in chain]
        assert got["n_chain"] == len(chain), i
        assert list(got["chain"]) == idx, i


def _random_hits(rng, n, n_rid, span_choices):
    x = np.zeros(n, np.uint64)
    y = np.zeros(n, np.uint64)
    h = rng.integers(0, max(4, n // 3), n).astype(np.uint64)  # shared hashes: multi-occurrence entries
    span = rng.choice(span_choices, n).astype(np.uint64)
    x[:] = (h << np.uint64(8)) | span
    rid = rng.integers(0, n_rid, n).astype(np.uint64)
    strand = rng.integers(0, 2, n).astype(np.uint64)
    pos = rng.integers(0, 20000, n).astype(np.uint64)
    y[:] = (strand << np.uint64(63)) | (rid << np.uint64(32)) | pos
    return x, y


@pytest.mark.parametrize("seed", range(6))
def test_general_collect_and_chain_vs_oracle(gpu, oracle, seed):
    """Several sequence ids, both strands, mixed spans and shared hashes:
    collect_anchors with its filters, then chainAnchors."""
    rng = np.random.default_rng(100 + seed)
    rx, ry = _random_hits(rng, int(rng.integers(50, 3000)), 3, [11, 15, 21])
    qx, qy = _random_hits(rng, int(rng.integers(30, 1500)), 2, [13, 15])
    # half of the query hashes come from the reference so anchors exist
    take = rng.random(len(qx)) < 0.5
    src = rng.integers(0, len(rx), len(qx))
    qx[take] = (rx[src[take]] & ~np.uint64(0xff)) | (qx[take] & np.uint64(0xff))
    prm = gpu.params(q_occ_frac=float(rng.choice([0.0, 0.01, 0.05])), sample_every_bp=int(rng.choice([0, 3, 500])),
                     f_top_frac=float(rng.choice([2e-4, 0.02])), u_floor=int(rng.choice([1, 2, 10])),
                     u_ceil=int(rng.choice([3, 1000000])))
    hits = gpu.Hits(rx, ry, prm)
    got = hits.collect(qx, qy, prm)
    want = oracle.collect_anchors(rx, ry, qx, qy, (prm.f_top_frac, prm.u_floor, prm.u_ceil, prm.q_occ_frac,
                                                   prm.sample_every_bp))
    assert len(got) == len(want)
    for f in want.dtype.names:
        assert np.array_equal(got[f], want[f]), f
    if len(want) == 0:
        return
    # chain with relaxed scores so multi-anchor chains form on random data
    cp = gpu.params(max_dist_x=8000, max_dist_y=8000, bw=int(rng.choice([500, 5000])), min_cnt=1, min_score=1,
                    max_skip=int(rng.choice([0, 2, 25])), max_iter=int(rng.choice([3, 50, 5000])))
    srt, chain, f, p = gpu.chain_anchors(want, cp)
    osrt, ochain, of, op = oracle.chain_anchors_fp(
        want, [cp.max_dist_x, cp.max_dist_y, cp.bw, cp.max_skip, cp.max_iter, cp.min_cnt, cp.min_score],
        [cp.gap_penalty, cp.skip_penalty])
    for fld in want.dtype.names:
        assert np.array_equal(srt[fld], osrt[fld]), fld
    assert np.array_equal(f, of) and np.array_equal(p, op)
    for fld in want.dtype.names:
        assert np.array_equal(srt[chain][fld], ochain[fld]), fld


def test_chain_reference_known_answers(gpu):
    """Known answers of the reference's chainAnchors tests (test/test_anchor.cpp):
    empty input, a single anchor, linkable and unlinkable pairs, best chain
    across sequence ids and strands, bandwidth and distance cut-offs."""
    def A(rows):
        a = np.zeros(len(rows), gpu.ANCHOR_DTYPE)
        for i, (rid, pr, pq, span, rev) in enumerate(rows):
            a[i]["rid_ref"], a[i]["pos_ref"], a[i]["pos_qry"], a[i]["span"], a[i]["is_rev"] = rid, pr, pq, span, rev
        return a

    loose = gpu.params(min_cnt=1, min_score=0)
    _, ch, _, _ = gpu.chain_anchors(A([]), loose)
    assert len(ch) == 0
    s, ch, _, _ = gpu.chain_anchors(A([(0, 100, 50, 20, 0)]), loose)
    assert len(ch) == 1 and s[ch][0]["span"] == 20
    s, ch, _, _ = gpu.chain_anchors(A([(0, 200, 150, 20, 0), (0, 100, 50, 20, 0)]), loose)
    assert list(s[ch]["pos_ref"]) == [100, 200] and list(s[ch]["pos_qry"]) == [50, 150]
    # best chain is on sequence 0 (three anchors) rather than sequence 1 (one)
    s, ch, _, _ = gpu.chain_anchors(A([(1, 100, 50, 20, 0), (0, 100, 50, 20, 0), (0, 200, 150, 20, 0),
                                       (0, 300, 250, 20, 0)]), loose)
    assert all(s[ch]["rid_ref"] == 0) and len(ch) >= 2
    s, ch, _, _ = gpu.chain_anchors(A([(0, 100, 50, 20, 1), (0, 100, 50, 20, 0), (0, 200, 150, 20, 0),
                                       (0, 300, 250, 20, 0)]), loose)
    assert all(s[ch]["is_rev"] == 0) and len(ch) >= 2
    # further apart than max_dist: no link
    s, ch, _, _ = gpu.chain_anchors(A([(0, 100, 50, 20, 0), (0, 10000, 9950, 20, 0)]), loose)
    assert len(ch) == 1
    # diagonal offset beyond bw: no link
    s, ch, _, _ = gpu.chain_anchors(A([(0, 100, 100, 20, 0), (0, 1000, 200, 20, 0)]), loose)
    assert len(ch) == 1
    # min_cnt and min_score reject short chains
    two = A([(0, 100, 50, 20, 0), (0, 200, 150, 20, 0)])
    assert len(gpu.chain_anchors(two, gpu.params(min_cnt=3, min_score=0))[1]) == 0
    assert len(gpu.chain_anchors(two, gpu.params(min_cnt=1, min_score=1000))[1]) == 0


def test_project_row_vs_oracle(gpu, oracle, pkg):
    w = pkg.synth.mito(6)
    cx, cy = oracle.extract_minimizer(w.center)
    for i in range(w.n):
        q = w.query(i)
        cig = oracle.align_query(w.center, cx, cy, q)
        assert gpu.project_row(q, cig) == oracle.del_query(q, cig)
        # padQueryToRefByCigar: every op but D/N/H/P copies query bases
        want = bytearray()
        r = 0
        for c in cig:
            op, ln = int(c) & 0xf, int(c) >> 4
            if op in (2, 3):
                want += b"-" * ln
            elif op in (5, 6):
                continue
            else:
                want += q[r:r + ln]
                r += ln
        assert gpu.project_row(q, cig, pad=True) == bytes(want)
    # an empty CIGAR leaves the query as it is; a CIGAR that does not consume
    # the query exactly is refused
    assert gpu.project_row(b"ACGT", np.zeros(0, np.uint32)) == b"ACGT"
    with pytest.raises(gpu.HalignError):
        gpu.project_row(b"ACGT", np.array([3 << 4], np.uint32))


def test_count_rows_vs_oracle(gpu, oracle):
    rng = np.random.default_rng(9)
    alphabet = np.frombuffer(b"ACGTacgtUuNn-.XR*", np.uint8)
    rows = alphabet[rng.integers(0, len(alphabet), (777, 1003))]
    want = oracle.count_rows(rows)
    assert np.array_equal(gpu.count_rows(rows), want)
    assert np.array_equal(gpu.count_rows(rows[:100], gpu.count_rows(rows[100:])), want)


MAT = np.array([5, -4, -4, -4, 0, -4, 5, -4, -4, 0, -4, -4, 5, -4, 0, -4, -4, -4, 5, 0, 0, 0, 0, 0, 0], np.int8)


def test_extz2_match_mismatch_golden_vectors(gpu, golden):
    """ksw_extz2 without KSW_EZ_GENERIC_SC (extendAlignKSW2's scoring)
    against the reference's outputs, including the score lanes past the band
    end that the reference fills from its padding."""
    z = golden.load("ksw_extz2_ng.npz")
    bad = []
    for i in range(len(z["params"])):
        w, zdrop, eb, flag = (int(x) for x in z["params"][i])
        q = z["q"][z["q_off"][i]:z["q_off"][i + 1]]
        t = z["t"][z["t_off"][i]:z["t_off"][i + 1]]
        ez, cig = gpu.ksw_extz2(q, t, 5, MAT, 6, 2, w, zdrop, eb, flag)
        if not (np.array_equal(ez, z["ez"][i]) and
                np.array_equal(cig, z["cigar"][z["cigar_off"][i]:z["cigar_off"][i + 1]])):
            bad.append(i)
    assert not bad, f"{len(bad)} of {len(z['params'])} differ, first {bad[:5]}"


def test_extend_align_vs_oracle(gpu, oracle, pkg):
    """extendAlignKSW2 (z-drop, end bonus 50, match/mismatch scoring) on
    longer pairs than the golden vectors, against the oracle."""
    import ctypes as C
    L = gpu.lib()
    L.hg_extend_align_ksw2.argtypes = [C.c_char_p, C.c_int64, C.c_char_p, C.c_int64, C.c_int, C.c_void_p,
                                       C.c_int64]
    L.hg_extend_align_ksw2.restype = C.c_int64
    rng = np.random.default_rng(31)
    dna5 = np.full(256, 4, np.uint8)
    for i, ch in enumerate(b"ACGT"):
        dna5[ch] = i
        dna5[ch + 32] = i
    for it in range(30):
        ref = np.frombuffer(b"ACGTN", np.uint8)[rng.integers(0, 5 if it % 4 == 0 else 4, int(rng.integers(50, 900)))]
        qry = ref[int(rng.integers(0, 40)):].copy()
        m = rng.random(len(qry)) < 0.08
        qry[m] = np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, int(m.sum()))]
        if it % 3 == 0:  # a divergent tail makes z-drop end the extension
            qry[len(qry) // 2:] = np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, len(qry) - len(qry) // 2)]
        zd = int(rng.choice([200, 30]))
        out = np.zeros(len(ref) + len(qry) + 4, np.uint32)
        n = L.hg_extend_align_ksw2(ref.tobytes(), len(ref), qry.tobytes(), len(qry), zd, gpu._p(out), len(out))
        assert n >= 0
        w = oracle.auto_band(len(ref), len(qry))
        _, want = oracle.ksw_extz2(dna5[qry], dna5[ref], 5, MAT, 6, 2, w, zd, 50, 0x40 | 0x02 | 0x10)
        assert np.array_equal(out[:n], want), it


def test_packed_dp_cell_equals_int32_cell(gpu):
    """The small tier's int16x2 cell (two segments per instruction) against
    the int32 cell over every input a band-free cell can see, both gap
    modes, with different inputs in the two halves."""
    import ctypes as C
    L = gpu.lib()
    L.hg_dp_lane_selftest.argtypes = [C.c_void_p]
    bad = C.c_uint32(123)
    gpu._check(L.hg_dp_lane_selftest(C.byref(bad)))
    assert bad.value == 0


@pytest.mark.parametrize("name,n", [("divergent", 60), ("uneven", 120), ("serve", 40), ("mito", 60)])
def test_tier_boundary_knobs_do_not_change_results(gpu, pkg, name, n):
    """The thin and square tiers switched off, or narrowed, move their
    segments to other tiers, and the small tier runs in either form: the
    CIGARs stay identical."""
    w = getattr(pkg.synth, name)(n)
    ix = gpu.Index(w.center)
    ctx = gpu.Context(ix, max_queries=n, max_bases=int(w.total_bases) + 1024)
    b = gpu.pack(w.seqs, w.offsets)
    base = ctx.align(b, rows=True)
    default = ctx.get_launch()
    for thin, sq, pair in ((0, 0, 0), (8, 2000, 1), (32, 0, 0), (0, 12288, 1), (32, 12288, 1)):
        ctx.set_launch(default[:6] + [thin, sq, pair] + default[9:])
        got = ctx.align(b, rows=True)
        assert np.array_equal(got.cigar, base.cigar) and np.array_equal(got.cigar_off, base.cigar_off), (thin, sq,
                                                                                                      pair)
        assert np.array_equal(got.rows, base.rows)
    ctx.set_launch(default)


def test_second_lane_covers_the_same_work(gpu, pkg):
    """A staged run of several sub-batches on one lane and on two: the same
    counters, status, DP cells and work totals (every other sub-batch runs
    on the second lane's own arenas)."""
    w = pkg.synth.mito(120)
    ix = gpu.Index(w.center)
    ctx = gpu.Context(ix, max_queries=32, max_bases=32 * 16700)
    ctx.stage(gpu.pack(w.seqs, w.offsets))
    knobs = ctx.get_launch()
    out = []
    for lanes in (1, 2):
        ctx.set_launch(knobs[:9] + [lanes])
        ctx.counters(reset=True)
        w0 = np.array(list(ctx.work().values()))
        ctx.run_staged()
        ctx.last_timing()
        cnt, ins = ctx.counters(reset=True)
        out.append((cnt, ins, ctx.staged_flags(), ctx.last_cells(), np.array(list(ctx.work().values())) - w0))
    (c1, i1, f1, l1, k1), (c2, i2, f2, l2, k2) = out
    assert np.array_equal(c1, c2) and np.array_equal(i1, i2)
    assert f1 == f2 == 0 and l1 == l2
    assert np.array_equal(k1, k2)
