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
