"""Continuous-batching serving loop for align-to-center requests.

The center index and the per-column consensus counters stay resident on the
GPU.  Requests (one query each) arrive over time; the loop keeps a FIFO of
arrived requests and a pool of contexts, each with its own CUDA stream and
arenas.  Whenever a context is free it admits the oldest waiting requests as
one micro-batch - as many as fit its capacity and the device-memory budget
of everything in flight - and enqueues it asynchronously (hg_submit); the
loop polls the busy contexts and collects finished micro-batches.  Packing a
micro-batch (ASCII to the 2-bit input format, a native call that releases
the interpreter lock) runs on a worker thread, so the loop keeps submitting
and collecting while the next micro-batch is packed.  Requests
that arrive while others are on the GPU therefore join as soon as a slot and
memory free up, and micro-batches of different contexts overlap on the
device.  Each request's CIGAR is identical to aligning it alone: requests are
independent and the batch kernels are order-insensitive per query.
"""
from __future__ import annotations

import time
from collections import deque
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field

import numpy as np

from . import Context, Index, pack

# device bytes a request of L bases holds while in flight (arenas scale with
# bases: hits, anchors, segments, CIGAR scratch, rows)
BYTES_PER_BASE = 64


@dataclass
class ServeStats:
    latencies_ms: np.ndarray
    bases: int
    wall_s: float
    batches: int
    max_inflight_bytes: int
    results: dict = field(default_factory=dict)

    def summary(self) -> dict:
        lat = self.latencies_ms
        return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "mean_ms": float(lat.mean()), "max_ms": float(lat.max()), "requests": int(len(lat)),
                "mbp_per_s": self.bases / self.wall_s / 1e6, "micro_batches": self.batches,
                "max_inflight_bytes": self.max_inflight_bytes}


class Server:
    def __init__(self, index: Index, n_slots: int = 4, slot_queries: int = 512, slot_bases: int = 8_000_000,
                 budget_bytes: int = 40 << 30):
        self.index = index
        self.budget = budget_bytes
        self.slot_bases = slot_bases
        self.slots = [Context(index, max_queries=slot_queries, max_bases=slot_bases) for _ in range(n_slots)]
        self.slot_queries = slot_queries
        self.packer = ThreadPoolExecutor(max_workers=1)

    @staticmethod
    def _pack(seqs, offsets, lens, take):
        a, z = take[0], take[-1]
        if z - a + 1 == len(take):  # consecutive requests: pack straight from the source buffer
            blob = memoryview(seqs)[offsets[a]:offsets[z + 1]]
            offs = (offsets[a:z + 2] - offsets[a]).astype(np.int64)
        else:
            blob = b"".join(seqs[offsets[i]:offsets[i + 1]] for i in take)
            offs = np.concatenate([[0], np.cumsum(lens[take])]).astype(np.int64)
        return pack(blob, offs)

    def run(self, seqs: bytes, offsets: np.ndarray, arrivals: np.ndarray | None = None,
            keep_results: bool = False) -> ServeStats:
        """Serve requests i = 0..n-1 arriving at arrivals[i] seconds (None: all
        at once).  Returns latency statistics (arrival to collected result)."""
        n = len(offsets) - 1
        if arrivals is None:
            arrivals = np.zeros(n)
        lens = np.diff(offsets).astype(np.int64)
        # a request that no context or budget can ever hold would wait forever
        if n and int(lens.max()) > self.slot_bases:
            raise ValueError(f"request of {int(lens.max())} bases exceeds the context capacity ({self.slot_bases})")
        if n and int(lens.max()) * BYTES_PER_BASE > self.budget:
            raise ValueError("request exceeds the device-memory budget")
        pending: deque[int] = deque()
        busy: dict[int, tuple[list[int], int]] = {}
        packing: dict = {}  # slot -> (pack future, requests, bases)
        free = list(range(len(self.slots)))
        done_t = np.zeros(n)
        results = {}
        inflight = 0
        max_inflight = 0
        batches = 0
        nxt = 0
        finished = 0
        t0 = time.perf_counter()
        while finished < n:
            now = time.perf_counter() - t0
            while nxt < n and arrivals[nxt] <= now:
                pending.append(nxt)
                nxt += 1
            # admit: fill free contexts with the oldest waiting requests
            while free and pending:
                take, tb = [], 0
                while pending and len(take) < self.slot_queries:
                    i = pending[0]
                    need = int(lens[i]) * BYTES_PER_BASE
                    if tb + lens[i] > self.slot_bases or inflight + need > self.budget:
                        break
                    take.append(pending.popleft())
                    tb += int(lens[i])
                    inflight += need
                if not take:
                    break
                s = free.pop()  # reserved; submitted once its micro-batch is packed
                packing[s] = (self.packer.submit(self._pack, seqs, offsets, lens, take), take, tb)
                batches += 1
                max_inflight = max(max_inflight, inflight)
            progressed = False
            for s in list(packing):
                fut, take, tb = packing[s]
                if fut.done():
                    del packing[s]
                    self.slots[s].submit(fut.result())
                    busy[s] = (take, tb)
                    progressed = True
            # collect finished micro-batches
            for s in list(busy):
                if self.slots[s].poll():
                    take, tb = busy.pop(s)
                    res = self.slots[s].collect(check=False)
                    t = time.perf_counter() - t0
                    for j, i in enumerate(take):
                        done_t[i] = t
                        if keep_results:
                            results[i] = res.cigar_of(j).copy()
                    inflight -= tb * BYTES_PER_BASE
                    finished += len(take)
                    free.append(s)
                    progressed = True
            if not progressed and not (free and pending):
                if nxt < n and not busy and not pending and not packing:
                    time.sleep(max(0.0, arrivals[nxt] - (time.perf_counter() - t0)))
                else:
                    time.sleep(20e-6)
        wall = time.perf_counter() - t0
        lat = (done_t - arrivals) * 1e3
        return ServeStats(lat, int(lens.sum()), wall, batches, max_inflight, results)

    def counters(self, reset: bool = False):
        tot_c = tot_i = None
        for c in self.slots:
            cnt, ins = c.counters(reset)
            tot_c = cnt if tot_c is None else tot_c + cnt
            tot_i = ins if tot_i is None else tot_i + ins
        return tot_c, tot_i


class NativeServer:
    """The same continuous-batching loop run by the library's threads
    (hg_serve_*): Python only feeds requests at their arrival times and drains
    results on a second thread, so the host path is native end to end.  The
    device-memory budget caps the contexts created (their arenas are
    allocated up front); every result carries its HG_ST_* status."""

    STAT_KEYS = ("p50_ms", "p99_ms", "mean_ms", "max_ms", "requests", "bases", "micro_batches", "wall_s",
                 "contexts", "device_bytes")

    def __init__(self, index: Index, n_slots: int = 8, slot_queries: int = 1024, slot_bases: int = 16_000_000,
                 budget_bytes: int = 40 << 30):
        import ctypes as C
        from . import _check, lib
        self._C, self._lib, self._check = C, lib(), _check
        self.index = index
        h = C.c_void_p()
        _check(self._lib.hg_serve_create(index.h, n_slots, slot_queries, slot_bases, budget_bytes, C.byref(h)))
        self.h = h

    def stats(self, reset: bool = False) -> dict:
        v = np.zeros(len(self.STAT_KEYS), np.float64)
        self._check(self._lib.hg_serve_stats(self.h, v.ctypes.data_as(self._C.c_void_p), len(v), int(reset)))
        return dict(zip(self.STAT_KEYS, (float(x) for x in v)))

    def run(self, seqs: bytes, offsets: np.ndarray, arrivals: np.ndarray | None = None,
            keep_results: bool = False) -> dict:
        """Serve requests i = 0..n-1, submitted at arrivals[i] seconds (None:
        all at once).  Returns the loop's statistics for these requests plus
        per-request status (and CIGARs with keep_results)."""
        import threading
        C = self._C
        n = len(offsets) - 1
        self.stats(reset=True)
        status = np.zeros(n, np.uint32)
        results = {}
        ids = np.full(n, -1, np.int64)
        errors = []

        def drain():
            max_n, cap = 4096, 1 << 22
            buf = np.zeros(cap, np.uint32)
            rid = np.zeros(max_n, np.int64)
            st = np.zeros(max_n, np.uint32)
            coff = np.zeros(max_n + 1, np.int64)
            vp = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
            got = 0
            while got < n:
                m = self._lib.hg_serve_results(self.h, max_n, vp(rid), vp(st), None, vp(buf), cap, vp(coff), 1000)
                if m < 0:  # the message is this thread's: carry it to the caller
                    errors.append((-m, self._lib.hg_last_error().decode(errors="replace")))
                    return
                status[rid[:m] - base] = st[:m]
                if keep_results:
                    for j in range(m):
                        results[int(rid[j] - base)] = buf[coff[j]: coff[j + 1]].copy()
                got += m

        # requests whose arrival time has passed are queued together (one
        # hg_serve_submit_many per loop turn), the rest when they are due
        raw = np.frombuffer(seqs, np.uint8) if len(seqs) else np.zeros(1, np.uint8)
        offsets = np.ascontiguousarray(offsets, np.int64)
        t0 = time.perf_counter()
        base, th, i = None, None, 0
        while i < n:
            if arrivals is None:
                j = n
            else:
                now = time.perf_counter() - t0
                j = int(np.searchsorted(arrivals, now, side="right"))
                if j <= i:
                    time.sleep(max(0.0, min(arrivals[i] - now, 0.001)))
                    continue
            rel = offsets[i:j + 1] - offsets[i]
            first = self._lib.hg_serve_submit_many(self.h, C.c_void_p(raw.ctypes.data + int(offsets[i])),
                                                   rel.ctypes.data_as(C.c_void_p), j - i)
            if first < 0:
                self._check(-first)
            if base is None:
                base = first - i
                th = threading.Thread(target=drain, daemon=True)
                th.start()
            ids[i:j] = np.arange(first, first + (j - i))
            i = j
        if th is not None:
            th.join()
        if errors:
            from . import HalignError
            raise HalignError(*errors[0])
        out = self.stats()
        out["status_or"] = int(np.bitwise_or.reduce(status)) if n else 0
        out["mbp_per_s"] = out["bases"] / out["wall_s"] / 1e6 if out["wall_s"] > 0 else 0.0
        out["status"] = status
        out["results"] = results
        return out

    def counters(self, reset: bool = False):
        L = self.index.L
        cnt = np.zeros((L, 7), np.uint32)
        ins = np.zeros(L + 1, np.uint32)
        C = self._C
        self._check(self._lib.hg_serve_counters(self.h, cnt.ctypes.data_as(C.c_void_p), ins.ctypes.data_as(C.c_void_p),
                                                int(reset)))
        return cnt, ins

    def close(self):
        if getattr(self, "h", None):
            self._lib.hg_serve_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
