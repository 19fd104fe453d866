"""Benchmark of the GB300 align-to-center path.

Workload (the configuration the headline metric is quoted on): 100,000
full-length mutated copies of a 16,569 bp uniform ACGT center (seed 0; 1%
substitutions, 0.1% + 0.1% indels of geometric length mean 3), k=15, w=10,
stored 2-bit packed.  Synthetic, seeded; no dataset is read.

One step = one pass of the hot path (minimizers -> anchors -> chain ->
gap-fill DP -> CIGAR -> aligned rows -> per-column counters) over the whole
batch, run as two 50,000-query sub-batches (`--sub-batch`; each stage is
one launch per sub-batch).  Inputs (1.66 Gbp, 415 MB packed) and all
intermediates exceed the 129 MB L2, so no flush is needed between steps.

  value   aligned Mbp/s with the packed batch resident in HBM (hg_run_staged),
          CUDA events on the context stream
  e2e     the same metric through the C ABI call a user makes
          (hg_align_batch with pinned host buffers): packed input H2D,
          CIGARs + insertion flags + aligned rows D2H inside the timed region
  cpu_baseline / --impl reference: the CPU path (the oracle's restatement of
          the reference loop, OpenMP over every host core) on a bounded sample

Multi-GPU (torchrun): queries are independent, so ranks take contiguous
shards of a fixed per-rank batch (weak scaling, no data-path collective);
timing is max over ranks.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "aligned Mbp/s (align-to-center, bit-exact)"
UNIT = "Mbp/s"
N_QUERIES = 100_000
CENTER_LEN = 16_569
MEASURED = ROOT / "MEASURED_PEAKS.json"
FALLBACK_HBM = 6800.0


# Speed of the oracle port relative to the unmodified reference build on the
# same queries and threads (x86-64, where the reference's SSE2 KSW2 builds;
# interleaved 50-query blocks of the mito workload, tests/test_port_speed.py).
PORT_VS_REF_X86 = {"threads_1": 0.98, "threads_8": 0.96}

# Warp instructions per query base of the stage kernels, from their ncu
# captures on the mito workload (profiles/kernels_mito4k.md).
MITO_INST_PER_BASE = {"seed": 273.3e6 / 66.3e6, "anchor": 71.0e6 / 66.3e6, "chain": 319.6e6 / 66.3e6,
                      "rows": 32.6e6 / 66.3e6}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    def __init__(self, world, local, use_gpu):
        self.world = world
        self.pg = None
        if world > 1:
            import torch.distributed as dist
            backend = "nccl" if use_gpu else "gloo"
            if use_gpu:
                import torch
                torch.cuda.set_device(local)
            dist.init_process_group(backend)
            self.dist = dist

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64, device="cuda" if self.dist.get_backend() == "nccl" else "cpu")
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.dist.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.samples.append([x.strip() for x in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *exc):
        self._stop.set()
        if self._t:
            self._t.join(timeout=6)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 5 + i and s[5 + i].strip().lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def load_peaks():
    if MEASURED.exists():
        d = json.loads(MEASURED.read_text())
        return float(d.get("hbm_gbs", FALLBACK_HBM)), "measured"
    return FALLBACK_HBM, "fallback"


WORKLOADS = {
    "mito": "mito: {n} queries x ~16,569 bp vs a 16,569 bp center, 1% sub, 0.1%+0.1% indels (geometric mean 3), "
            "k=15, w=10, 2-bit packed",
    "uneven": "uneven: {n} substrings (lognormal length, median 8 kb, sigma 0.5, 300..29,903 bp, 1% with "
              "10-200 bp N-runs) of a 29,903 bp center, 0.1% sub, 0.025%+0.025% indels, k=15, w=10",
    "divergent": "divergent: {n} queries x ~5,000 bp vs a 5,000 bp center, 10% sub, 1%+1% indels (mean 8), "
                 "k=15, w=10",
    "serve": "serve: {n} substrings (uniform 500..29,903 bp) of a 29,903 bp center, 0.5% divergence, k=15, w=10",
}


def make_workload(pkg, n, name="mito", rank=0):
    """Rank r's shard of the seeded workload: queries [r*n, (r+1)*n) (mito:
    1000-query generator blocks; the others: generator chunk r)."""
    t = time.time()
    if name == "mito":
        w = pkg.synth.mito(n, block0=rank * (-(-n // pkg.synth.MITO_CHUNK)))
    else:
        w = getattr(pkg.synth, name)(n, chunk=rank)
    log(f"[bench] generated {w.n} queries / {w.total_bases} bases in {time.time() - t:.1f}s")
    t = time.time()
    b = pkg.pack(w.seqs, w.offsets)
    log(f"[bench] packed {b.packed.nbytes} bytes in {time.time() - t:.1f}s")
    return w, b


def cpu_sample(oracle, w, budget_s: float, threads: int):
    """Time the CPU path on consecutive 1000-query blocks until budget_s."""
    done_q = done_b = 0
    tot = 0.0
    i = 0
    while tot < budget_s and i < w.n:
        j = min(i + 1000, w.n)
        offs = w.offsets[i:j + 1] - w.offsets[i]
        seqs = w.seqs[w.offsets[i]: w.offsets[j]]
        t, _ = oracle.align_batch(w.center, w.center, seqs, offs, nthreads=threads)
        tot += t
        done_q += j - i
        done_b += int(offs[-1])
        i = j
    return done_b / tot / 1e6, done_q, done_b, tot


# the kernel behind each event-timed stage (dp_small: the small, medium and
# thin tiers on the main stream; dp_large: the wait for the two side streams)
STAGE_KERNEL = {"seed": "seed_fast_kernel", "anchor": "anchor_kernel", "chain": "chain_kernel",
                "dp_small": "dp_small_kernel + dp_medium_kernel + dp_thin_kernel",
                "dp_large": "dp_wave_kernel + dp_large_kernel + dp_wave_cta_kernel",
                "stitch": "stitch_kernel", "rows": "row_kernel", "count": "count_kernel"}


def algorithmic_bytes(b, n_cigar_words: int, L: int):
    """HBM bytes the path must move: packed input + per-query arrays in, rows +
    CIGARs + flags out."""
    inp = b.packed.nbytes + b.exc.nbytes + 8 * b.n * 3
    out = b.n * L + 4 * n_cigar_words + b.n
    return inp + out


def integer_roofline(pkg, args, stages, top, top_ms, bases, local, clocks):
    """The dominant kernel's warp-instruction rate against the issue ceiling
    and the measured integer-pipe ceiling (hg_int_peaks)."""
    peaks = pkg.int_peaks()
    sms = 152
    try:
        import torch
        sms = torch.cuda.get_device_properties(local).multi_processor_count
    except Exception:
        pass
    sm_mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0
    issue_peak = 4.0 * sms * sm_mhz * 1e6
    roof = {"bound": "int-issue", "kernel": STAGE_KERNEL.get(top, top), "unit": "warp-inst/s",
            "peak": round(issue_peak, 1), "peak_source": f"4 warp-inst/clk/SM x {sms} SMs x {sm_mhz:.0f} MHz (sampled)",
            "int_pipe_peak_warp_inst": round(peaks["int_pipe_warp_inst"], 1),
            "measured_int_peaks_per_s": {k: round(v, 1) for k, v in peaks.items()}}
    if args.workload == "mito" and top in MITO_INST_PER_BASE and top_ms > 0:
        ach = MITO_INST_PER_BASE[top] * bases / (top_ms / 1e3)
        roof.update({"achieved": round(ach, 1), "frac": round(ach / issue_peak, 4),
                     "frac_of_int_pipe_peak": round(ach / peaks["int_pipe_warp_inst"], 4),
                     "inst_per_base": round(MITO_INST_PER_BASE[top], 3)})
    if args.workload == "mito":
        roof["stage_issue_frac"] = {k: round(v * bases / (stages[k] / 1e3) / issue_peak, 4)
                                    for k, v in MITO_INST_PER_BASE.items() if stages.get(k, 0) > 0}
    return roof


def measure_link(nbytes: int = 1 << 30, reps: int = 3) -> dict:
    """Pinned-memory copy rates of this host's link to the GPU: one 1 GiB
    copy each way, and both directions at once on two streams (median of
    reps, CUDA events).  The host-buffer call overlaps its copies with
    compute, so its step cannot be shorter than the copies' time at these
    rates."""
    import torch
    dev = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    dev2 = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    host = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    host2 = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    st, st2 = torch.cuda.Stream(), torch.cuda.Stream()
    rates = {}

    def median(ms):
        ms = sorted(ms[1:])
        return ms[len(ms) // 2]

    for name, dst, src in (("h2d", dev, host), ("d2h", host, dev)):
        ms = []
        for _ in range(reps + 1):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(st):
                e0.record(st)
                dst.copy_(src, non_blocking=True)
                e1.record(st)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        rates[name] = nbytes / (median(ms) / 1e3) / 1e9
    ms = []
    for _ in range(reps + 1):
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(st)
        st2.wait_event(e0)
        with torch.cuda.stream(st):
            dev.copy_(host, non_blocking=True)
            e1.record(st)
        with torch.cuda.stream(st2):
            host2.copy_(dev2, non_blocking=True)
            e2.record(st2)
        e1.synchronize()
        e2.synchronize()
        ms.append(max(e0.elapsed_time(e1), e0.elapsed_time(e2)))
    rates["both"] = 2 * nbytes / (median(ms) / 1e3) / 1e9
    del dev, dev2, host, host2
    return rates


def measure_plain(pkg, ctx, w, n_plain: int):
    """The plain form (one launch sequence per query, hg_align_plain) on the
    first n_plain queries, and the batched form on the same queries."""
    offs = w.offsets[: n_plain + 1]
    b = pkg.pack(w.seqs[: offs[-1]], offs)
    ctx.align(b, rows=True, plain=True)  # warm-up
    t0 = time.perf_counter()
    ctx.align(b, rows=True, plain=True)
    t_plain = time.perf_counter() - t0
    ctx.align(b, rows=True)
    t0 = time.perf_counter()
    ctx.align(b, rows=True)
    t_batch = time.perf_counter() - t0
    return {"queries": n_plain, "plain_mbp_per_s": round(b.bases / t_plain / 1e6, 3),
            "batched_same_queries_mbp_per_s": round(b.bases / t_batch / 1e6, 3),
            "note": "host-timed hg_align_plain vs hg_align_batch (both with H2D/D2H) on the same queries"}


def measure_serving(pkg, n_req: int, rate: float, n_sat: int = 240000):
    """The serving loop (hg_serve_*, scheduler in the library) on the serve
    workload (Poisson arrivals, 500..29,903 bp substrings of a 29,903 bp
    center, 0.5% divergence): p50/p99 at `rate` req/s; saturation (n_sat
    requests all waiting at t=0) against the same n_sat requests aligned as
    one device-resident batch; and an offered load of 70% of that batched
    rate (Poisson arrivals) for latency at load."""
    w = pkg.synth.serve(n_req, rate=rate)
    ix = pkg.Index(w.center)
    srv = pkg.serve.NativeServer(ix, n_slots=12, slot_queries=4096, slot_bases=64_000_000, budget_bytes=120 << 30)
    srv.run(w.seqs, w.offsets[: min(w.n, 400) + 1], None)  # warm-up
    st = srv.run(w.seqs, w.offsets, w.arrivals)
    ws = pkg.synth.serve(n_sat, rate=rate, chunk=1)
    sat = srv.run(ws.seqs, ws.offsets, None)
    # the same requests as one batch, device-resident and through the host-buffer call
    sub = 20000  # the batched denominator in 20,000-request sub-batches (two compute lanes)
    lens = np.diff(ws.offsets)
    ctx = pkg.Context(ix, max_queries=sub, max_bases=max(int(lens[i:i + sub].sum()) for i in range(0, ws.n, sub)) + 1024)
    b = pkg.pack(ws.seqs, ws.offsets)
    ctx.stage(b)
    for _ in range(2):
        ctx.run_staged()
    ctx.last_timing()
    ctx.run_staged()
    ms = ctx.last_timing()[0]
    batched = b.bases / (ms / 1e3) / 1e6
    ctx.align(b, rows=False, check=False)
    t0 = time.perf_counter()
    ctx.align(pkg.pack(ws.seqs, ws.offsets), rows=False, check=False)
    batched_e2e = b.bases / (time.perf_counter() - t0) / 1e6
    ctx.close()
    # offered load at 70% of the batched device rate
    rate_hi = 0.7 * batched * 1e6 / (b.bases / ws.n)
    wh = pkg.synth.serve(n_sat, rate=rate_hi, chunk=2)
    hi = srv.run(wh.seqs, wh.offsets, wh.arrivals)
    keep = ("p50_ms", "p99_ms", "mean_ms", "max_ms", "requests", "micro_batches", "mbp_per_s", "status_or")
    out = {k: st[k] for k in keep}
    out.update({"rate_req_per_s": rate, "center_bp": len(w.center), "loop": "native (hg_serve_*)",
                "contexts": int(st["contexts"]), "device_bytes": int(st["device_bytes"]), "budget_bytes": 120 << 30,
                "saturation": {k: sat[k] for k in keep},
                "batched_same_requests_mbp_per_s": batched, "batched_same_requests_e2e_mbp_per_s": batched_e2e,
                "saturation_frac_of_batched": sat["mbp_per_s"] / batched,
                "saturation_frac_of_batched_e2e": sat["mbp_per_s"] / batched_e2e,
                "high_load": {"offered_frac_of_batched": 0.7, "rate_req_per_s": rate_hi,
                              **{k: hi[k] for k in keep}}})
    srv.close()
    return _round(out)


def _round(d):
    if isinstance(d, dict):
        return {k: _round(v) for k, v in d.items()}
    return round(d, 3) if isinstance(d, float) else d


def run_serve_million(args, pkg):
    """The serving loop over args.serve_requests requests generated in
    chunks (the stated 10^6), all waiting: the resident counters of the
    served rows must equal those of the batch path over the same requests,
    and a sample of the served CIGARs must equal the oracle's."""
    import multiprocessing as mp
    pool = mp.get_context("spawn").Pool(max(1, (os.cpu_count() or 2) - 2))
    chunk = 50000
    n_chunks = -(-args.serve_requests // chunk)
    w0 = pkg.synth.serve(min(chunk, args.serve_requests), chunk=0)
    ix = pkg.Index(w0.center)
    srv = pkg.serve.NativeServer(ix, n_slots=4, slot_queries=8192, slot_bases=128_000_000, budget_bytes=100 << 30)
    ctx = pkg.Context(ix, max_queries=chunk, max_bases=chunk * 20000)  # requests average 15.2 kb
    pending, served, bases, t_serve, p99s, st_or = [], 0, 0, 0.0, [], 0
    for c in range(n_chunks):
        m = min(chunk, args.serve_requests - c * chunk)
        w = w0 if c == 0 else pkg.synth.serve(m, chunk=c)
        out = srv.run(w.seqs, w.offsets, None, keep_results=True)
        t_serve += out["wall_s"]
        p99s.append(out["p99_ms"])
        st_or |= out["status_or"]
        ctx.align(pkg.pack(w.seqs, w.offsets), rows=False, check=False)  # batch path: its own counters
        served += w.n
        bases += int(w.total_bases)
        idx = list(range(0, w.n, max(1, w.n // max(1, args.check_sample // n_chunks))))
        for a in range(0, len(idx), 100):
            part = idx[a:a + 100]
            pending.append(pool.apply_async(_oracle_check_cigars, ((w.center, [w.query(i) for i in part],
                                                                    [out["results"][i] for i in part]),)))
        log(f"[serve] chunk {c + 1}/{n_chunks}: {w.n} requests served")
    cs, ins_s = srv.counters()
    cb, ins_b = ctx.counters()
    bad = sum(r.get() for r in pending)
    pool.close()
    line = {"metric": "serving loop over a stated-size request stream", "mode": "serve", "requests": served,
            "bases": bases, "mbp_per_s_saturated": round(bases / t_serve / 1e6, 3),
            "p99_ms_worst_chunk": round(max(p99s), 3), "status_or": st_or,
            "counters_equal_batch_path": bool(np.array_equal(cs, cb) and np.array_equal(ins_s, ins_b)),
            "counters_total": int(cs.astype(np.uint64).sum()),
            "cigar_sample_checked": args.check_sample, "cigar_sample_mismatches": int(bad),
            "note": "chunks of 50,000 requests, all waiting; counters of the serving contexts vs a batch context "
                    "over the same requests; CIGAR sample vs the oracle"}
    srv.close()
    print(json.dumps(line), flush=True)
    return 0


def _oracle_check_cigars(args_tuple):
    center, queries, cigs = args_tuple
    from oracle.oracle import Oracle
    o = Oracle()
    cx, cy = o.extract_minimizer(center)
    return sum(0 if np.array_equal(c, o.align_query(center, cx, cy, q)) else 1 for q, c in zip(queries, cigs))


def _oracle_check(args_tuple):
    """CIGARs and rows (as sha256 digests) of sampled queries against the
    oracle (pool worker)."""
    center, queries, cigs, rows = args_tuple
    from oracle.oracle import Oracle
    o = Oracle()
    cx, cy = o.extract_minimizer(center)
    bad_c = bad_r = 0
    for j, q in enumerate(queries):
        want = o.align_query(center, cx, cy, q)
        if not np.array_equal(cigs[j], want):
            bad_c += 1
        row = o.del_query(q, want)
        if rows[j] != hashlib.sha256(row).digest():
            bad_r += 1
    return bad_c, bad_r, len(queries)


def run_stream(args, pkg):
    """A workload at its stated size, streamed: chunk c of the seeded
    workload (all chunks generated first) is copied into a pinned buffer
    (the caller's input) and aligned through hg_align_ascii (uploaded and
    packed on the device; CIGARs, insertion flags and rows come back into
    pinned buffers); a fixed
    sample of every chunk - every query with an N-run plus a stride - is
    kept and checked against the oracle (CIGARs and rows) on the host cores
    (a spawned pool) after the last chunk, so the checks do not take the
    host cores from the timed calls.  The value is aligned Mbp/s over
    all chunks (transfers, packing and alignment; generation excluded)."""
    import multiprocessing as mp
    name, n_total, chunk = args.workload, args.queries, args.stream_chunk
    n_chunks = -(-n_total // chunk)
    if name == "mito":
        def gen(c, m):
            return pkg.synth.mito(m, block0=c * (-(-chunk // pkg.synth.MITO_CHUNK)))
    else:
        def gen(c, m):
            return getattr(pkg.synth, name)(m, chunk=c)
    pool = mp.get_context("spawn").Pool(max(1, (os.cpu_count() or 2) - 2))
    w0 = gen(0, min(chunk, n_total))
    ix = pkg.Index(w0.center)
    longest = 29903 if name in ("uneven", "serve") else len(w0.center) + 64
    sub = min(chunk, 50000)
    ctx = pkg.Context(ix, max_queries=sub, max_bases=min(sub * longest, 900_000_000))
    import torch
    pin = lambda a: torch.from_numpy(a).pin_memory().numpy()  # noqa: E731
    L, P = pkg.lib(), pkg._p
    stride = (ix.L + 15) // 16 * 16
    seq_pin = pin(np.zeros(chunk * longest + 64, np.uint8))
    rows_pin = pin(np.zeros((chunk, stride), np.uint8))
    cig_pin = pin(np.zeros(chunk * longest // 8 + 64 * chunk + 1024, np.uint32))
    off_out, ins_out, st_out = np.zeros(chunk + 1, np.int64), np.zeros(chunk, np.uint8), np.zeros(chunk, np.uint32)
    pending = []
    t_align = 0.0
    bases = queries = 0
    per_chunk = max(1, args.check_sample // n_chunks)
    # every chunk is generated before the timed loop: generating (and freeing
    # gigabytes of) numpy temporaries right before a call measured slowing
    # the next call by up to 3x (the host's memory churn, not the library)
    chunks = [w0] + [gen(c, min(chunk, n_total - c * chunk)) for c in range(1, n_chunks)]
    for c in range(-1, n_chunks):  # chunk 0 once untimed first: the context's lanes and buffers are set up
        m = min(chunk, n_total - max(c, 0) * chunk)
        w = chunks[max(c, 0)]
        offs = np.ascontiguousarray(w.offsets, np.int64)
        seq_pin[:len(w.seqs)] = np.frombuffer(w.seqs, np.uint8)  # the caller's pinned input buffer
        if c < 0:
            pkg._check(L.hg_align_ascii(ctx.h, P(seq_pin), P(offs), m, P(cig_pin), len(cig_pin), P(off_out),
                                        P(ins_out), P(rows_pin), stride, P(st_out)))
            continue
        t0 = time.perf_counter()
        code = L.hg_align_ascii(ctx.h, P(seq_pin), P(offs), m, P(cig_pin), len(cig_pin), P(off_out), P(ins_out),
                                P(rows_pin), stride, P(st_out))
        dt = time.perf_counter() - t0
        t_align += dt
        pkg._check(code)
        if st_out[:m].any():
            raise SystemExit(f"stream: chunk {c} reported status flags")
        bases += int(offs[-1] - offs[0])
        queries += m
        # sample: every query with an N-run, plus a stride over the rest
        has_n = [i for i in range(m) if b"N" in w.query(i)]
        stride_i = list(range(0, m, max(1, m // per_chunk)))[:per_chunk]
        idx = sorted(set(has_n) | set(stride_i))
        for a in range(0, len(idx), 200):  # tasks of 200 queries spread over the pool
            part = idx[a:a + 200]
            pending.append((w.center, [w.query(i) for i in part], [cig_pin[off_out[i]:off_out[i + 1]].copy() for i in part],
                            [hashlib.sha256(rows_pin[i, :ix.L]).digest() for i in part]))
        log(f"[stream] chunk {c + 1}/{n_chunks}: {m} queries, {(offs[-1] - offs[0]) / 1e6:.1f} Mbp in {1e3 * dt:.1f} ms, "
            f"{len(idx)} sampled")
    bad_c = bad_r = n_chk = 0
    for bc, br, nn in pool.imap_unordered(_oracle_check, pending):
        bad_c, bad_r, n_chk = bad_c + bc, bad_r + br, n_chk + nn
    pool.close()
    line = {"metric": METRIC, "value": round(bases / t_align / 1e6, 3), "unit": UNIT, "n_gpus": 1,
            "mode": "stream", "higher_is_better": True, "dtype": "u8/int32", "data": "synthetic",
            "config": {"workload": WORKLOADS[name].format(n=n_total), "queries": queries, "bases": bases,
                       "chunk_queries": chunk, "chunks": n_chunks,
                       "timed": "per chunk: hg_align_ascii from the chunk's ASCII bytes in pinned memory "
                                "(rows back into pinned memory); generation and the fill of the pinned input "
                                "buffer excluded"},
            "parity_full_size": {"checked_queries": n_chk, "cigar_mismatches": bad_c, "row_mismatches": bad_r,
                                 "against": "oracle CIGARs and rows; every N-run query plus a stride sample"}}
    print(json.dumps(line), flush=True)
    return 0


def _oracle_check_multiref(args_tuple):
    refs, queries, bests, cigs = args_tuple
    from oracle.oracle import Oracle
    o = Oracle()
    sks = [o.sketch(r) for r in refs]
    mz = [o.extract_minimizer(r) for r in refs]
    bad_b = bad_c = 0
    for q, b, c in zip(queries, bests, cigs):
        ob, _ = o.best_reference(o.sketch(q), sks)
        bad_b += int(ob != b)
        bad_c += int(not np.array_equal(o.align_query(refs[ob], mz[ob][0], mz[ob][1], q), c))
    return bad_b, bad_c, len(queries)


def run_multiref(args, pkg):
    """Multi-reference mode (several references of one length, each query
    aligned to its best reference by MinHash jaccard): the device selection
    alone (sketch + jaccard over the resident reference sketches, one
    launch, CUDA events) and end to end through hg_refset_align with host
    buffers (H2D, selection, per-reference batches, rows back), with an
    oracle check of a sample (best reference and CIGAR)."""
    import multiprocessing as mp
    pool = mp.get_context("spawn").Pool(max(1, (os.cpu_count() or 2) - 2))
    n, n_refs = args.queries, args.refs
    w = pkg.synth.multiref(n, n_refs=n_refs, ref_len=16569)
    sub = min(n, 12_500)  # per-reference contexts: sub-batches of 12,500 queries
    rs = pkg.RefSet(w.refs, max_queries=sub, max_bases=sub * 16700)
    b = pkg.pack(w.seqs, w.offsets)
    k = 15
    kmers = int(np.maximum(b.qlen.astype(np.int64) - k + 1, 0).sum())
    for _ in range(args.warmup):
        rs.select(b)
    sel_ms = []
    for _ in range(args.steps):
        best, jac = rs.select(b)
        sel_ms.append(rs.last_select_ms())
    t0 = time.perf_counter()
    res = rs.align(b, keep_length=True, rows=True)
    t_keep = time.perf_counter() - t0
    t0 = time.perf_counter()
    res_c = rs.align(b, keep_length=False, rows=True)
    t_cons = time.perf_counter() - t0
    idx = list(range(0, n, max(1, n // max(1, args.check_sample))))[: args.check_sample]
    pending = [pool.apply_async(_oracle_check_multiref, ((w.refs, [w.query(i) for i in idx[a:a + 50]],
                                                          [int(res.best[i]) for i in idx[a:a + 50]],
                                                          [res.cigar_of(i).copy() for i in idx[a:a + 50]]),))
               for a in range(0, len(idx), 50)]
    bad_b = bad_c = n_chk = 0
    for r in pending:
        x, y, z = r.get()
        bad_b, bad_c, n_chk = bad_b + x, bad_c + y, n_chk + z
    pool.close()
    ms = float(np.median(sel_ms))
    # the oracle's sketch + selection on one host core, over a sample
    from oracle.oracle import Oracle
    o = Oracle()
    sks = [o.sketch(r) for r in w.refs]
    t0, cb = time.perf_counter(), 0
    for i in range(0, min(n, 300)):
        o.best_reference(o.sketch(w.query(i)), sks)
        cb += len(w.query(i))
    cpu_sel = cb / (time.perf_counter() - t0) / 1e6
    line = {"metric": "multi-reference selection and alignment", "mode": "multiref", "unit": "Mbp/s",
            "config": {"workload": f"multiref: {n} queries x ~16,569 bp, {n_refs} references of 16,569 bp "
                                   "(3% substitution variants of one center), queries 1% sub, 0.1%+0.1% indels; "
                                   "k=15, w=10, sketch size 2000, seed 42",
                       "queries": n, "bases": b.bases, "kmers": kmers},
            "select_kernel": {"ms": round(ms, 3), "mbp_per_s": round(b.bases / ms / 1e3, 3),
                              "kmer_hashes_per_s": round(kmers / ms * 1e3, 1),
                              "input_gb_per_s": round(b.packed.nbytes / ms / 1e6, 3),
                              "timing": "CUDA events around the one sketch + selection launch, median of steps"},
            "cpu_baseline_select": {"value": round(cpu_sel, 3), "unit": "Mbp/s", "cores": 1, "kind": "port",
                                    "sample": "sketch + best reference of the first 300 queries"},
            "e2e_keep_length": {"mbp_per_s": round(b.bases / t_keep / 1e6, 3), "s": round(t_keep, 3),
                                "timed": "hg_refset_align with host buffers: upload, selection, one batch per "
                                         "reference, rows back"},
            "e2e_consensus_recheck": {"mbp_per_s": round(b.bases / t_cons / 1e6, 3), "s": round(t_cons, 3)},
            "chosen_reference_counts": np.bincount(res.best, minlength=n_refs).tolist(),
            "parity_sample": {"checked_queries": n_chk, "best_ref_mismatches": bad_b, "cigar_mismatches": bad_c,
                              "status_or": int(np.bitwise_or.reduce(res.status)) | int(np.bitwise_or.reduce(
                                  res_c.status)), "against": "oracle sketch/jaccard selection and CIGAR"}}
    rs.close()
    print(json.dumps(line), flush=True)
    return 0


def run_impl_reference(args, rank, world):
    """The reference's CPU path (the oracle restatement) on the host cores."""
    if rank != 0:
        return 0
    from oracle.oracle import Oracle
    from tests.pkgload import load_package
    pkg = load_package()
    o = Oracle()
    threads = os.cpu_count() or 1
    w = pkg.synth.mito(4000)
    for _ in range(args.warmup):
        cpu_sample(o, w, 0.5, threads)
    vals = []
    for _ in range(args.steps):
        v, nq, nb, t = cpu_sample(o, w, 5.0, threads)
        vals.append((v, nq, nb, t))
    value = float(np.median([v[0] for v in vals]))
    tot_t = sum(v[3] for v in vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1000 * tot_t / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8/int32",
        "data": "synthetic (seeded mutated copies of a uniform ACGT center)",
        "config": {"workload": "mito 16,569 bp center x mutated full-length queries; bounded sample per step",
                   "k": 15, "w": 10, "sample_queries_per_step": int(np.median([v[1] for v in vals]))},
        "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "consecutive 1000-query blocks of the mito workload, ~5 s per step",
                         "port_vs_reference_x86": PORT_VS_REF_X86},
        "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--queries", type=int, default=N_QUERIES, help="queries per GPU")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--sub-batch", type=int, default=50_000,
                    help="queries per device sub-batch (sizes the arenas; fewer, larger sub-batches shorten the per-kernel tails, two still overlap copies with compute)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=4000)
    ap.add_argument("--plain-queries", type=int, default=128)
    ap.add_argument("--stage-timing", action="store_true", help="per-stage event timing pass (extra run)")
    ap.add_argument("--no-tune", action="store_true", help="skip the launch-shape autotuner")
    ap.add_argument("--workload", default="mito", choices=sorted(WORKLOADS),
                    help="synthetic workload (the headline metric is quoted on mito)")
    ap.add_argument("--stream-chunk", type=int, default=0,
                    help="stream the workload in generated chunks of this many queries and check a full-size "
                         "sample against the oracle (the stated-size checks)")
    ap.add_argument("--multiref", action="store_true",
                    help="multi-reference mode: device selection and per-reference alignment (--queries, --refs)")
    ap.add_argument("--refs", type=int, default=4)
    ap.add_argument("--serve-million", action="store_true",
                    help="serve --serve-requests requests (10^6 stated) and check the resident counters")
    ap.add_argument("--check-sample", type=int, default=10000,
                    help="queries checked against the oracle in stream mode (plus every N-run query)")
    args = ap.parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        return run_impl_reference(args, rank, world)

    from tests.pkgload import load_package
    pkg = load_package()
    pkg.lib()
    if pkg.device_count() == 0:
        raise SystemExit("bench: no CUDA device")
    if args.multiref:
        return run_multiref(args, pkg)
    if args.stream_chunk > 0:
        return run_stream(args, pkg)
    if args.serve_million:
        return run_serve_million(args, pkg)
    dist = Dist(world, local, use_gpu=True)
    if world > 1:
        pkg.set_device(local)  # the library's current device for this process: its index and contexts live there
    w, b = make_workload(pkg, args.queries, args.workload, rank)
    ix = pkg.Index(w.center)
    gpu_ordinal, gpu_bus = ix.device()
    if world > 1:
        from halign_gb300 import shard
        shard.check_distinct_devices(gpu_bus, dist.dist)  # two ranks on one GPU would overstate throughput
    sub = min(args.sub_batch, args.queries)
    lens = np.diff(w.offsets)
    # capacity: the largest base count of `sub` consecutive queries (the sub-batches the batch splits into)
    chunk_bases = max(int(lens[i:i + sub].sum()) for i in range(0, len(lens), sub))
    ctx = pkg.Context(ix, max_queries=sub, max_bases=chunk_bases + 1024)
    ctx.stage(b)
    tuning = None
    if not args.no_tune:
        # launch-shape autotuner (coordinate descent on CTAs per SM, staged runs)
        t0 = time.perf_counter()
        default = ctx.get_launch()[:pkg.DEVICE_KNOBS]
        best, best_ms, tried = pkg.autotune.tune(pkg.autotune.staged_measure(ctx, reps=1), default, rounds=1)
        ctx.set_launch(best)
        tuning = {"knobs": dict(zip(pkg.LAUNCH_KNOBS, best)), "default_knobs": dict(zip(pkg.LAUNCH_KNOBS, default)),
                  "default_ms": round(tried[0][1], 3), "tuned_ms": round(best_ms, 3), "candidates": len(tried),
                  "seconds": round(time.perf_counter() - t0, 1)}
        log(f"[bench] tuned launch {best} ({tried[0][1]:.1f} -> {best_ms:.1f} ms, {len(tried)} candidates)")
    # warm-up (also builds and caches the CUDA graphs of every sub-batch)
    for _ in range(args.warmup):
        ctx.run_staged()
    ctx.last_timing()
    dist.barrier()
    import ctypes as C
    L = pkg.lib()
    # device-resident timing: CUDA events on the context stream bracket every
    # staged run; the per-step sync sits between the events of two steps
    dev_ms = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            ctx.run_staged()
            ms, _, launches = ctx.last_timing()  # synchronizes the context stream
            dev_ms.append(ms)
    dist.barrier()
    flags = ctx.staged_flags()
    if flags:
        raise SystemExit(f"bench: staged run reported status flags 0x{flags:x} (incomplete alignments)")
    step_s = dist.max(float(np.sum(dev_ms)) / 1e3 / args.steps)
    cells, match_cells = ctx.last_cells()  # cells of the last step, and those of match segments
    value = world * b.bases / step_s / 1e6
    # per-stage breakdown (event-timed pass; excluded from the headline number)
    # and the pass's unit counts (anchors, segment records, DP segments)
    work0 = ctx.work()
    ctx.set_timing(True)
    ctx.run_staged()
    stage_tot, stages, _ = ctx.last_timing()
    ctx.set_timing(False)
    work1 = ctx.work()
    work = {k: work1[k] - work0[k] for k in work0}
    n_cig_words = None
    # e2e: the C ABI call with pinned host buffers
    e2e = None
    parity = None
    if not args.no_e2e:
        import torch
        pin = lambda a: torch.from_numpy(a).pin_memory().numpy()  # noqa: E731
        pb = pkg.Packed(pin(b.packed), pin(b.poff), pin(b.qlen), pin(b.exc), pin(b.exc_off))
        rows_out = pin(np.zeros((b.n, (ix.L + 15) // 16 * 16), np.uint8))
        cig_out = pin(np.zeros(b.bases // 8 + 64 * b.n + 1024, np.uint32))
        off_out = np.zeros(b.n + 1, np.int64)
        ins_out = np.zeros(b.n, np.uint8)
        st_out = np.zeros(b.n, np.uint32)
        P = pkg._p

        def call():
            code = L.hg_align_batch(ctx.h, P(pb.packed), P(pb.poff), P(pb.qlen), P(pb.exc), P(pb.exc_off), pb.n,
                                    P(cig_out), len(cig_out), P(off_out), P(ins_out), P(rows_out),
                                    rows_out.shape[1], P(st_out))
            pkg._check(code)

        # warm-up: the pinned buffers were just allocated (a large allocation
        # measured slowing the calls right after it)
        for _ in range(max(2, args.warmup)):
            call()
        dist.barrier()
        e2e_steps = args.steps
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            call()
        e_wall = dist.max((time.perf_counter() - t0) / e2e_steps)
        # from ASCII: hg_align_ascii on the queries' bytes in pinned memory
        # (uploaded per sub-batch and packed on the device), every step
        asc_steps = max(1, args.steps)
        seqs_u8 = pin(np.frombuffer(w.seqs, np.uint8))
        offs64 = np.ascontiguousarray(w.offsets, np.int64)

        def call_ascii():
            pkg._check(L.hg_align_ascii(ctx.h, P(seqs_u8), P(offs64), b.n, P(cig_out), len(cig_out), P(off_out),
                                        P(ins_out), P(rows_out), rows_out.shape[1], P(st_out)))

        # warm-up: the pinned input was just allocated (a large allocation
        # measured slowing the calls right after it), and the first call sets
        # up the ASCII buffers
        for _ in range(max(2, args.warmup)):
            call_ascii()
        t0 = time.perf_counter()
        for _ in range(asc_steps):
            call_ascii()
        a_wall = dist.max((time.perf_counter() - t0) / asc_steps)
        call()  # the outputs checked below come from the packed-input call
        n_cig_words = int(off_out[-1])
        # spot check of the timed output against the CPU path (bit-exact)
        from oracle.oracle import Oracle
        rng = np.random.default_rng(rank)
        pick = np.sort(rng.choice(b.n, size=min(200, b.n), replace=False))
        o = Oracle()
        mism = 0
        for i in pick:
            want = o.align_query(w.center, *o.extract_minimizer(w.center), w.query(int(i)))
            if not np.array_equal(cig_out[off_out[i]:off_out[i + 1]], want):
                mism += 1
        parity = {"checked_queries": int(len(pick)), "mismatches": int(mism), "against": "oracle CIGARs"}
        h2d = b.nbytes
        d2h = 4 * n_cig_words + 8 * (b.n + 1) + b.n + 4 * b.n + b.n * ix.L
        link = measure_link()
        e2e = {"value": round(world * b.bases / e_wall / 1e6, 3), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "ms_per_step": round(1000 * e_wall, 3), "steps": e2e_steps,
               "link": {"h2d_gb_per_s": round(link["h2d"], 1), "d2h_gb_per_s": round(link["d2h"], 1),
                        "both_ways_gb_per_s": round(link["both"], 1),
                        "copy_ms_per_step": round(1000 * (h2d / link["h2d"] + d2h / link["d2h"]) / 1e9, 3),
                        "note": "pinned 1 GiB copies on this host; the call overlaps copies with compute, so its "
                                "step is bounded below by the device step and by these copies"},
               "input": "2-bit packed host buffers (the C ABI's input format)",
               "from_ascii": {"value": round(world * b.bases / a_wall / 1e6, 3), "unit": UNIT,
                              "ms_per_step": round(1000 * a_wall, 3), "steps": asc_steps,
                              "input": "ASCII query bytes in pinned host memory (hg_align_ascii: uploaded per "
                                       "sub-batch, packed on the device)"}}
    if n_cig_words is None:
        n_cig_words = 64 * b.n
    plain = measure_plain(pkg, ctx, w, args.plain_queries) if args.plain_queries > 0 else None
    ctx.close()  # (and its second lane) before the serving measurement allocates its own contexts
    serving = None if args.no_serve or rank != 0 else measure_serving(pkg, args.serve_requests, 2000.0)
    peak, peak_kind = load_peaks()
    # dominant stage (one kernel launch per sub-batch) and its algorithmic
    # bytes from the pass's unit counts: A anchors, R segment records, B bases
    top = max(stages, key=lambda k: stages[k])
    alg = algorithmic_bytes(b, n_cig_words, ix.L)
    A, R, B = work["anchors"], work["records"], b.bases
    stage_bytes = {"seed": b.packed.nbytes + 8 * A,           # packed in; (pos, entry) hits out
                   "anchor": 8 * A + 8 * A,                    # hits in; (pos_ref, pos_qry) out
                   "chain": 16 * A + 32 * R + b.packed.nbytes,  # positions in, f/p out; records out; 2-bit windows
                   "dp_small": b.packed.nbytes + 4 * n_cig_words, "dp_large": b.packed.nbytes + 4 * n_cig_words,
                   "stitch": 32 * R + 8 * n_cig_words,
                   "rows": b.n * ix.L + b.packed.nbytes + 4 * n_cig_words, "count": b.n * ix.L}
    top_ms = stages[top]
    n_sub = max(1, -(-b.n // sub))
    achieved = (alg / (stage_tot / 1e3) / 1e9) if stage_tot > 0 else None
    top_achieved = (stage_bytes.get(top, 0) / (top_ms / 1e3) / 1e9) if top_ms > 0 else None
    # DRAM bytes (read + written) per query base of each dominant-stage kernel
    # from its ncu capture on the mito workload (4,000 queries, 66.3 Mbp),
    # scaled to one launch (one sub-batch) of this run
    mito_dram_per_base = {"seed": (17.17e6 + 24.66e6) / 66.3e6, "anchor": (81.10e6 + 38.27e6) / 66.3e6,
                          "chain": (296.61e6 + 62.36e6) / 66.3e6, "rows": (18.44e6 + 7.78e6) / 66.3e6}
    traffic = None
    if args.workload == "mito" and top in mito_dram_per_base:
        traffic = int(round(mito_dram_per_base[top] * B / n_sub))
    clocks = clk.summary()
    # integer roofline: the path is bound by integer instruction issue.  Warp
    # instructions per query base of each stage's kernel from its ncu capture
    # on the mito workload (4,000 queries, 66.3 Mbp; profiles/), times the
    # bases of this run, over the stage's event time, against the issue
    # ceiling (4 warp instructions per clock per SM at the sampled SM clock)
    # and the measured integer-pipe ceiling (hg_int_peaks: 2 per clock per
    # SM; kernels that also use the FMA, load/store and uniform pipes can
    # exceed it).
    int_roof = integer_roofline(pkg, args, stages, top, top_ms, B, local, clocks)
    cpu = None
    if rank == 0 and args.cpu_seconds > 0:
        from oracle.oracle import Oracle
        v, nq, nb, t = cpu_sample(Oracle(), w, args.cpu_seconds, os.cpu_count() or 1)
        cpu = {"value": round(v, 3), "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
               "sample": f"first {nq} queries ({nb} bases) of the workload, {t:.1f} s of CPU time",
               "port_vs_reference_x86": PORT_VS_REF_X86}
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1000 * step_s, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8/int32",
        "data": "synthetic (seeded mutated copies of a uniform ACGT center)",
        "config": {"workload": WORKLOADS[args.workload].format(n=args.queries),
                   "queries_per_gpu": args.queries, "bases_per_gpu": b.bases,
                   "l2": "inputs and intermediates exceed L2 (no flush needed)",
                   "parallelism": f"dp{world}: rank r aligns queries [r*n, (r+1)*n) of the seeded workload, "
                                  "center index replicated, no data-path collective",
                   "device": {"ordinal": gpu_ordinal, "pci_bus_id": gpu_bus},
                   "launch_tuning": tuning},
        "gcups": round(world * cells / step_s / 1e9, 3) if cells else None,
        "dp_cells": {"work_unit": cells, "in_match_segments": match_cells, "computed": cells - match_cells,
                     "computed_gcups": round(world * (cells - match_cells) / step_s / 1e9, 3) if cells else None,
                     "note": "match segments (exact k-mer spans, d M) are counted in the work unit but need no DP"},
        "gpu_launches": int(launches),
        "stage_ms": {k: round(v, 3) for k, v in stages.items()},
        "int_roofline": int_roof,
        "roofline": {"bound": "hbm", "kernel": STAGE_KERNEL.get(top, top),
                     "achieved": round(top_achieved, 2) if top_achieved else None, "peak": peak, "unit": "GB/s",
                     "frac": round(top_achieved / peak, 5) if top_achieved else None, "traffic": traffic,
                     "algorithmic_bytes_per_launch": int(stage_bytes.get(top, 0) / n_sub),
                     "launch_ms": round(top_ms / n_sub, 3), "launches": n_sub,
                     "units": {"anchors": A, "segment_records": R, "dp_segments": work["dp_segments"], "bases": B},
                     "peak_source": peak_kind,
                     "whole_path_achieved_gbs": round(achieved, 2) if achieved else None,
                     "note": "latency-bound integer path; the HBM fraction is low by construction"},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "parity_sample": parity,
        "plain_form": plain,
        "serve": serving,
        "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    dist.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
