"""Host logic of the continuous-batching loop (halign-4_gb300/serve.py) on
CPU: contexts are replaced by fakes that finish a micro-batch after a delay,
so admission, the packing worker, budgets and result routing run without a
GPU.  Packing is the real native host routine."""
import time

import numpy as np
import pytest


class FakeResult:
    def __init__(self, qlens):
        self.qlens = qlens

    def cigar_of(self, j):  # "result" of request j of the micro-batch: its length as one M op
        return np.array([int(self.qlens[j]) << 4], np.uint32)


class FakeContext:
    def __init__(self, delay, log):
        self.delay, self.log, self.t = delay, log, None

    def submit(self, b):
        assert self.t is None, "submitted twice without collect"
        self.b, self.t = b, time.perf_counter()
        self.log.append(b.n)

    def poll(self):
        return time.perf_counter() - self.t >= self.delay

    def collect(self, check=True):
        r = FakeResult(self.b.qlen.copy())
        self.t = None
        return r


def make_server(pkg, n_slots, slot_queries, slot_bases, budget, delay):
    from concurrent.futures import ThreadPoolExecutor
    srv = object.__new__(pkg.serve.Server)
    srv.index, srv.budget, srv.slot_bases, srv.slot_queries = None, budget, slot_bases, slot_queries
    srv.log = []
    srv.slots = [FakeContext(delay, srv.log) for _ in range(n_slots)]
    srv.packer = ThreadPoolExecutor(max_workers=1)
    return srv


def requests(n, seed=0):
    rng = np.random.default_rng(seed)
    lens = rng.integers(1, 400, n)
    seqs = b"".join(rng.choice(list(b"ACGT"), int(k)).astype(np.uint8).tobytes() for k in lens)
    return seqs, np.concatenate([[0], np.cumsum(lens)]).astype(np.int64), lens


def test_every_request_gets_its_own_result(pkg, native):
    seqs, offs, lens = requests(300)
    srv = make_server(pkg, n_slots=3, slot_queries=16, slot_bases=2000, budget=1 << 30, delay=0.001)
    st = srv.run(seqs, offs, None, keep_results=True)
    assert len(st.results) == 300
    for i in range(300):
        assert int(st.results[i][0]) >> 4 == lens[i]
    assert (st.latencies_ms >= 0).all()
    assert max(srv.log) <= 16
    assert st.batches == len(srv.log)


def test_budget_bounds_inflight_bytes(pkg, native):
    seqs, offs, lens = requests(200, seed=1)
    budget = int(lens.max()) * pkg.serve.BYTES_PER_BASE * 3
    srv = make_server(pkg, n_slots=8, slot_queries=64, slot_bases=100_000, budget=budget, delay=0.0005)
    st = srv.run(seqs, offs, None)
    assert st.max_inflight_bytes <= budget
    assert len(st.latencies_ms) == 200


def test_arrivals_wait_for_their_time(pkg, native):
    seqs, offs, lens = requests(40, seed=2)
    arrivals = np.linspace(0.0, 0.04, 40)
    srv = make_server(pkg, n_slots=2, slot_queries=8, slot_bases=10_000, budget=1 << 30, delay=0.0005)
    t0 = time.perf_counter()
    st = srv.run(seqs, offs, arrivals)
    assert time.perf_counter() - t0 >= 0.04
    assert (st.latencies_ms >= 0).all()


def test_oversized_request_is_refused_not_left_waiting(pkg, native):
    seqs, offs, lens = requests(10, seed=3)
    srv = make_server(pkg, n_slots=2, slot_queries=8, slot_bases=int(lens.max()) - 1, budget=1 << 30, delay=0.0)
    with pytest.raises(ValueError):
        srv.run(seqs, offs, None)
    srv = make_server(pkg, n_slots=2, slot_queries=8, slot_bases=100_000, budget=8, delay=0.0)
    with pytest.raises(ValueError):
        srv.run(seqs, offs, None)
