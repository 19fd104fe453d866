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
