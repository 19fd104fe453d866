"""Serving loop (continuous batching over several contexts/streams): every
request's result in the mix equals the result of aligning it alone, the
device-memory budget bounds what is in flight, and the resident counters
cover every served request."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def serve_setup(gpu, pkg):
    w = pkg.synth.serve(240, rate=20000.0)
    ix = gpu.Index(w.center)
    return w, ix


def test_results_identical_alone_and_in_the_mix(gpu, pkg, serve_setup):
    w, ix = serve_setup
    srv = pkg.serve.Server(ix, n_slots=3, slot_queries=32, slot_bases=600_000)
    st = srv.run(w.seqs, w.offsets, w.arrivals, keep_results=True)
    assert st.batches > 3  # requests really were split over several micro-batches
    alone_ctx = gpu.Context(ix, max_queries=1, max_bases=40_000)
    for i in range(w.n):
        b = gpu.pack(w.query(i), np.array([0, len(w.query(i))], np.int64))
        alone = alone_ctx.align(b, rows=False).cigar_of(0)
        assert np.array_equal(st.results[i], alone), i
    s = st.summary()
    assert s["requests"] == w.n and s["p99_ms"] >= s["p50_ms"] > 0


def test_memory_budget_bounds_inflight(gpu, pkg, serve_setup):
    w, ix = serve_setup
    lens = np.diff(w.offsets)
    budget = int(lens.max()) * pkg.serve.BYTES_PER_BASE * 3
    srv = pkg.serve.Server(ix, n_slots=4, slot_queries=64, slot_bases=2_000_000, budget_bytes=budget)
    st = srv.run(w.seqs, w.offsets[:61], None)
    assert st.max_inflight_bytes <= budget
    assert st.summary()["requests"] == 60


def test_resident_counters_cover_served_rows(gpu, pkg, serve_setup, oracle):
    w, ix = serve_setup
    srv = pkg.serve.Server(ix, n_slots=2, slot_queries=16, slot_bases=400_000)
    st = srv.run(w.seqs, w.offsets[:41], None, keep_results=True)
    cnt, ins = srv.counters()
    rows = np.stack([np.frombuffer(oracle.del_query(w.query(i), st.results[i]), np.uint8) for i in range(40)])
    assert np.array_equal(cnt, oracle.count_rows(rows))


def test_native_server_results_identical_alone_and_in_the_mix(gpu, pkg, serve_setup):
    """The library's own serving loop (hg_serve_*): every request's CIGAR in
    the mix equals its CIGAR alone, statuses come back, and the resident
    counters cover every served row."""
    w, ix = serve_setup
    srv = pkg.serve.NativeServer(ix, n_slots=3, slot_queries=32, slot_bases=600_000, budget_bytes=40 << 30)
    out = srv.run(w.seqs, w.offsets, w.arrivals, keep_results=True)
    assert out["requests"] == w.n and out["micro_batches"] > 3
    assert out["status_or"] == 0 and out["p99_ms"] >= out["p50_ms"] > 0
    alone_ctx = gpu.Context(ix, max_queries=1, max_bases=40_000)
    for i in range(w.n):
        b = gpu.pack(w.query(i), np.array([0, len(w.query(i))], np.int64))
        assert np.array_equal(out["results"][i], alone_ctx.align(b, rows=False).cigar_of(0)), i
    srv.close()


def test_native_server_counters_and_budget(gpu, pkg, serve_setup, oracle):
    w, ix = serve_setup
    # a budget of one context's arenas creates one context only
    probe = pkg.serve.NativeServer(ix, n_slots=1, slot_queries=16, slot_bases=400_000)
    one = probe.stats()["device_bytes"]
    probe.close()
    srv = pkg.serve.NativeServer(ix, n_slots=4, slot_queries=16, slot_bases=400_000, budget_bytes=int(one * 1.5))
    assert srv.stats()["contexts"] == 1
    out = srv.run(w.seqs, w.offsets[:41], None, keep_results=True)
    cnt, ins = srv.counters()
    rows = np.stack([np.frombuffer(oracle.del_query(w.query(i), out["results"][i]), np.uint8) for i in range(40)])
    assert np.array_equal(cnt, oracle.count_rows(rows))
    srv.close()


def _alone(gpu, ix, seqs, offs):
    ctx = gpu.Context(ix, max_queries=1, max_bases=40_000)
    out = []
    for i in range(len(offs) - 1):
        q = seqs[offs[i]:offs[i + 1]]
        out.append(ctx.align(gpu.pack(q, np.array([0, len(q)], np.int64)), rows=False, check=False).cigar_of(0))
    return out


def test_native_server_burst_larger_than_its_ring(gpu, pkg, serve_setup):
    """A burst of ~3.6 MB into a 1 MB request ring: submission waits for
    space, the ring wraps several times, micro-batches upload from it in one
    or two runs, and every CIGAR equals the request's CIGAR alone."""
    w, ix = serve_setup
    srv = pkg.serve.NativeServer(ix, n_slots=2, slot_queries=8, slot_bases=60_000, budget_bytes=40 << 30)
    assert int(w.offsets[-1]) > 3 << 20
    out = srv.run(w.seqs, w.offsets, None, keep_results=True)
    assert out["requests"] == w.n and out["status_or"] == 0
    alone = _alone(gpu, ix, w.seqs, w.offsets)
    for i in range(w.n):
        assert np.array_equal(out["results"][i], alone[i]), i
    srv.close()


def test_native_server_exception_bytes_and_empty_requests(gpu, pkg, serve_setup):
    """Requests with bytes other than A/C/G/T (N runs, lower case, IUPAC
    codes, exceptions at either end) and empty requests: the device packing
    of the serving loop gives the host packing's CIGARs."""
    w, ix = serve_setup
    rng = np.random.default_rng(17)
    center = w.center
    cases = []
    for i in range(60):
        a = int(rng.integers(0, len(center) - 3000))
        q = bytearray(center[a:a + int(rng.integers(1500, 3000))])
        kind = i % 6
        if kind == 1:
            p, r = int(rng.integers(0, len(q) - 60)), int(rng.integers(1, 60))
            q[p:p + r] = b"N" * r
        if kind == 2:
            q = bytearray(bytes(q[:700]).lower() + bytes(q[700:]))
        if kind == 3:
            for p in rng.integers(0, len(q), 12):
                q[int(p)] = b"RYKMSWBDHVNU"[int(rng.integers(0, 12))]
        if kind == 4:
            p = int(rng.integers(0, len(q) - 40))
            q[p:p + 40] = b"NANRNNRRNU" * 4
        if kind == 5:
            q[0:1] = b"n"
            q[-3:] = b"NNN"
        cases.append(bytes(q) if i % 20 != 7 else b"")
    seqs = b"".join(cases)
    offs = np.concatenate([[0], np.cumsum([len(x) for x in cases])]).astype(np.int64)
    srv = pkg.serve.NativeServer(ix, n_slots=3, slot_queries=16, slot_bases=40_000, budget_bytes=40 << 30)
    out = srv.run(seqs, offs, None, keep_results=True)
    assert out["requests"] == len(cases)
    alone = _alone(gpu, ix, seqs, offs)
    for i in range(len(cases)):
        assert np.array_equal(out["results"][i], alone[i]), i
    srv.close()


def test_native_server_exception_capacity_fails_the_loop(gpu, pkg, serve_setup):
    """More exception runs than a context holds (one per byte of a 20 kb
    request of alternating bytes) fail the loop with HG_ERR_CAPACITY, found
    by the device packing and reported when the micro-batch is collected."""
    w, ix = serve_setup
    bad = b"NR" * 10_000
    srv = pkg.serve.NativeServer(ix, n_slots=1, slot_queries=4, slot_bases=40_000, budget_bytes=40 << 30)
    with pytest.raises(pkg.HalignError) as e:
        srv.run(bad, np.array([0, len(bad)], np.int64), None)
    assert e.value.code == pkg.HG_ERR_CAPACITY and "exception runs" in str(e.value)
    srv.close()


def test_native_server_concurrent_submitters(gpu, pkg, serve_setup):
    """Four threads submit requests one at a time (hg_serve_submit) into a
    small ring while a fifth takes results one at a time (hg_serve_result):
    every id comes back once, with the CIGAR of the request that got it."""
    import ctypes as C
    import threading
    w, ix = serve_setup
    lib = pkg.lib()
    srv = pkg.serve.NativeServer(ix, n_slots=2, slot_queries=8, slot_bases=60_000, budget_bytes=40 << 30)
    n = w.n
    req_of_id = {}
    lock = threading.Lock()

    def submit(part):
        for i in range(part, n, 4):
            q = w.query(i)
            rid = lib.hg_serve_submit(srv.h, q, len(q))
            assert rid >= 0
            with lock:
                req_of_id[rid] = i

    threads = [threading.Thread(target=submit, args=(p,)) for p in range(4)]
    for t in threads:
        t.start()
    got = {}
    cig = np.zeros(1 << 16, np.uint32)
    rid, st, lat, nc = C.c_int64(), C.c_uint32(), C.c_double(), C.c_int64()
    while len(got) < n:
        r = lib.hg_serve_result(srv.h, C.byref(rid), C.byref(st), C.byref(lat), cig.ctypes.data_as(C.c_void_p),
                                len(cig), C.byref(nc), 10_000)
        assert r == 1, r
        assert rid.value not in got and st.value == 0
        got[rid.value] = cig[:nc.value].copy()
    for t in threads:
        t.join()
    alone = _alone(gpu, ix, w.seqs, w.offsets)
    assert sorted(req_of_id) == sorted(got)
    for k, v in got.items():
        assert np.array_equal(v, alone[req_of_id[k]]), k
    srv.close()
