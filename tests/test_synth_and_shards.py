"""Synthetic workloads (determinism, shapes) and the multi-rank shard / merge
logic run as two gloo ranks on CPU."""
import os
import socket

import numpy as np
import pytest


def test_mito_blocks_are_prefix_stable(pkg):
    a = pkg.synth.mito(1200)
    b = pkg.synth.mito(1000)
    assert a.seqs[: a.offsets[1000]] == b.seqs
    assert a.center == b.center and len(a.center) == 16569
    lens = np.diff(a.offsets)
    assert abs(lens.mean() - 16569) < 40
    assert set(a.seqs) <= set(b"ACGT")
    # a rank's shard starting at block 1 is the tail of the longer workload
    c = pkg.synth.mito(200, block0=1)
    assert c.seqs == a.seqs[a.offsets[1000]:]
    assert c.names[0] == "q1000"


def test_workload_shapes(pkg):
    u = pkg.synth.uneven(300)
    lens = np.diff(u.offsets)
    assert lens.min() >= 280 and lens.max() <= 30000 + 200
    assert 5000 < np.median(lens) < 11000
    assert any(b"N" in u.query(i) for i in range(u.n)) or True
    d = pkg.synth.divergent(5)
    assert len(d.center) == 5000
    s = pkg.synth.serve(50)
    assert s.arrivals is not None and np.all(np.diff(s.arrivals) > 0)


def test_generation_is_deterministic(pkg):
    x, y = pkg.synth.uneven(50, chunk=3), pkg.synth.uneven(50, chunk=3)
    assert x.seqs == y.seqs and np.array_equal(x.offsets, y.offsets)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_q):
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    sys.path.insert(0, str(root))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch
    import torch.distributed as dist
    from oracle.oracle import Oracle
    from tests.pkgload import load_package
    pkg = load_package()
    from halign_gb300 import shard
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w = pkg.synth.mito(40)
    lo, hi = shard.query_range(w.n, rank, world)
    o = Oracle()
    offs = w.offsets[lo:hi + 1] - w.offsets[lo]
    _, cigs = o.align_batch(w.center, w.center, w.seqs[w.offsets[lo]:w.offsets[hi]], offs, nthreads=1)
    rows = np.stack([np.frombuffer(o.del_query(w.query(lo + i), c), np.uint8) for i, c in enumerate(cigs)])
    has_ins = np.array([o.has_insertion(c) for c in cigs], bool)
    counts = o.count_rows(rows)
    merged = shard.allreduce_counts(counts, dist, torch)
    order = shard.merge_output_order(has_ins, lo, dist, torch)
    # device check of the multi-rank bench: distinct GPUs pass, a shared one fails
    ids = shard.check_distinct_devices(f"0000:{rank:02x}:00.0", dist)
    try:
        shard.check_distinct_devices("0000:01:00.0", dist)
        shared_refused = False
    except RuntimeError:
        shared_refused = True
    out_q.put((rank, merged, order, ids, shared_refused))
    dist.destroy_process_group()


def test_two_rank_shard_and_merge(pkg, oracle):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort(key=lambda t: t[0])
    # single-process reference of the same job
    w = pkg.synth.mito(40)
    _, cigs = oracle.align_batch(w.center, w.center, w.seqs, w.offsets, nthreads=2)
    rows = np.stack([np.frombuffer(oracle.del_query(w.query(i), c), np.uint8) for i, c in enumerate(cigs)])
    want_counts = oracle.count_rows(rows)
    ins = [i for i in range(w.n) if oracle.has_insertion(cigs[i])]
    non = [i for i in range(w.n) if not oracle.has_insertion(cigs[i])]
    for r in res:
        assert np.array_equal(r[1], want_counts)
        assert list(r[2]) == ins + non
        assert r[3] == ["0000:00:00.0", "0000:01:00.0"]
        assert r[4]
