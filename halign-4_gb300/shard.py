"""Multi-rank sharding of the align-to-center path.

Queries are independent, so ranks take contiguous query ranges and align
them with a replicated center index.  Two exchanges remain, both small and
both host-side:

* the per-column SiteCount counters (L x 7 uint32) are summed over ranks;
* the aligned FASTA keeps the reference's order (every insertion-bearing row,
  then every other row, each group in input order - mergeAlignedResults,
  src/align/ref_aligner.cpp:676-740), which needs each rank's insertion flags.

``dist`` is ``torch.distributed`` (gloo or NCCL) and ``torch`` the torch
module; nothing here runs on the alignment data path.  Under an NCCL process
group the exchanged tensors live on the rank's current CUDA device (NCCL
takes no CPU tensors); under gloo they stay on the CPU.
"""
from __future__ import annotations

import numpy as np


def _dev(dist, torch):
    return torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")


def check_distinct_devices(bus_id: str, dist) -> list[str]:
    """Gather every rank's GPU (its PCI bus id) and fail if two ranks share
    one: replicas that landed on the same GPU would overstate throughput."""
    ids = [None] * dist.get_world_size()
    dist.all_gather_object(ids, bus_id)
    if len(set(ids)) != len(ids):
        raise RuntimeError(f"ranks share a GPU: {ids}")
    return ids


def query_range(n: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous [lo, hi) share of n queries for this rank."""
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def allreduce_counts(counts: np.ndarray, dist, torch) -> np.ndarray:
    """Sum the L x 7 counters over ranks (uint32 arithmetic, as SiteCount)."""
    t = torch.from_numpy(counts.astype(np.int64)).to(_dev(dist, torch))
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return (t.cpu().numpy() & 0xFFFFFFFF).astype(np.uint32)


def merge_output_order(has_ins: np.ndarray, lo: int, dist, torch) -> np.ndarray:
    """Global query indices in output order: insertion rows first, then the
    rest, each in input order."""
    world = dist.get_world_size()
    dev = _dev(dist, torch)
    n_local = torch.tensor([len(has_ins)], dtype=torch.int64, device=dev)
    sizes = [torch.zeros(1, dtype=torch.int64, device=dev) for _ in range(world)]
    dist.all_gather(sizes, n_local)
    m = int(max(int(s.item()) for s in sizes))
    pad = torch.zeros(m, dtype=torch.int64, device=dev)
    pad[: len(has_ins)] = torch.from_numpy(has_ins.astype(np.int64)).to(dev)
    parts = [torch.zeros(m, dtype=torch.int64, device=dev) for _ in range(world)]
    dist.all_gather(parts, pad)
    flags = np.concatenate([p.cpu().numpy()[: int(s.item())] for p, s in zip(parts, sizes)]).astype(bool)
    idx = np.arange(len(flags))
    return np.concatenate([idx[flags], idx[~flags]])
