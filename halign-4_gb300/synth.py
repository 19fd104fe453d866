"""Seeded synthetic workloads for the align-to-center path.

No public dataset is used.  Each workload is a uniform i.i.d. ACGT center and
queries mutated from it, matching the shapes and value distributions of the
five benchmark configurations:

* ``mito``       16,569 bp center (seed 0), full-length copies, 1% substitutions,
                 0.1% insertions + 0.1% deletions, geometric lengths (mean 3).
                 ``n=1000`` is the CPU-runnable case, ``n=100000`` the batched one.
* ``uneven``     29,903 bp center, random substrings with lognormal lengths
                 (median 8 kb, sigma 0.5) clipped to 300..29,903, 0.1%
                 substitutions, 0.025% + 0.025% indels (mean 3), and 1% of the
                 queries carrying N-runs of 10..200 bp.
* ``divergent``  5,000 bp center, 10% substitutions, 1% + 1% indels of
                 geometric length (mean 8).
* ``serve``      29,903 bp center, substrings of uniform length 500..29,903,
                 0.5% divergence (0.4% substitutions, 0.05% + 0.05% indels,
                 mean 3), Poisson arrivals.
* ``multiref``   several references of one length (substitution variants of
                 one center) and full-length queries mutated from a random one.

All generation is vectorised (numpy PCG64), so the same seed gives the same
bytes on x86-64 and aarch64.  Queries come back as one concatenated ``bytes``
object plus an int64 offset array (``offsets[i]:offsets[i+1]``).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

ACGT = np.frombuffer(b"ACGT", np.uint8)


@dataclass
class Workload:
    name: str
    center: bytes
    seqs: bytes
    offsets: np.ndarray  # int64, len n+1
    names: list[str]
    arrivals: np.ndarray | None = None  # seconds, serving workloads only
    refs: list[bytes] | None = None     # multi-reference workloads: the references
    src_ref: np.ndarray | None = None   # multi-reference workloads: the reference each query came from

    @property
    def n(self) -> int:
        return len(self.offsets) - 1

    def query(self, i: int) -> bytes:
        return self.seqs[self.offsets[i]: self.offsets[i + 1]]

    @property
    def total_bases(self) -> int:
        return int(self.offsets[-1])


def random_center(length: int, seed: int) -> bytes:
    rng = np.random.Generator(np.random.PCG64(seed))
    return ACGT[rng.integers(0, 4, length)].tobytes()


def _geometric(rng, mean: float, size: int) -> np.ndarray:
    # support {1, 2, ...} with the given mean
    return rng.geometric(1.0 / mean, size).astype(np.int64)


def mutate_batch(src: np.ndarray, starts: np.ndarray, lens: np.ndarray, rng, p_sub: float, p_ins: float,
                 p_del: float, mean_indel: float):
    """Mutate ``len(starts)`` substrings ``src[starts[i]:starts[i]+lens[i]]``.

    Returns (bytes_concat, offsets).  Substitutions change a base to one of
    the three others; a deletion removes a geometric run starting at a base; an
    insertion adds a geometric run of random bases after a base.  Events are
    drawn per base independently.
    """
    n = len(starts)
    lens = lens.astype(np.int64)
    tot = int(lens.sum())
    seq_off = np.zeros(n + 1, np.int64)
    np.cumsum(lens, out=seq_off[1:])
    # gather the source substrings into one flat array
    if n and np.all(starts == 0) and np.all(lens == len(src)):
        flat = np.tile(src, n)
    else:
        idx = np.repeat(starts.astype(np.int64) - seq_off[:-1], lens) + np.arange(tot, dtype=np.int64)
        flat = src[idx]
        del idx
    # substitutions
    n_sub = rng.binomial(tot, p_sub)
    pos = rng.integers(0, tot, n_sub)
    code = (np.searchsorted(ACGT, flat[pos]) + rng.integers(1, 4, n_sub)) % 4
    flat[pos] = ACGT[code]
    # deletions: mark removed bases, never crossing a query boundary
    keep = np.ones(tot, bool)
    n_del = rng.binomial(tot, p_del)
    dpos = rng.integers(0, tot, n_del)
    dlen = _geometric(rng, mean_indel, n_del)
    owner = np.searchsorted(seq_off, dpos, side="right") - 1
    dlen = np.minimum(dlen, seq_off[owner + 1] - dpos)
    if n_del:
        ranges = np.repeat(dpos - np.concatenate(([0], np.cumsum(dlen)[:-1])), dlen) + np.arange(dlen.sum())
        keep[ranges] = False
    # insertions after a base
    n_ins = rng.binomial(tot, p_ins)
    ipos = np.sort(rng.integers(0, tot, n_ins))
    ilen = _geometric(rng, mean_indel, n_ins)
    ivals = ACGT[rng.integers(0, 4, int(ilen.sum()))]
    at = np.repeat(ipos + 1, ilen)
    flat = np.insert(flat, at, ivals)
    keep = np.insert(keep, at, True)
    # new per-query lengths
    ins_owner = np.searchsorted(seq_off, ipos, side="right") - 1
    ins_per_q = np.bincount(ins_owner, weights=ilen, minlength=n).astype(np.int64)
    gone = np.nonzero(~keep)[0]
    # positions in the post-insertion array: map back through the inserted runs
    del_per_q = np.bincount(np.searchsorted(seq_off + np.concatenate(([0], np.cumsum(ins_per_q))), gone,
                                            side="right") - 1, minlength=n).astype(np.int64)
    new_lens = lens + ins_per_q - del_per_q
    out = flat[keep]
    offsets = np.zeros(n + 1, np.int64)
    np.cumsum(new_lens, out=offsets[1:])
    assert offsets[-1] == len(out)
    return out, offsets


def _names(prefix: str, i0: int, n: int) -> list[str]:
    return [f"{prefix}{i}" for i in range(i0, i0 + n)]


MITO_CHUNK = 1000


def mito(n: int = 1000, seed: int = 0, center_len: int = 16569, block0: int = 0) -> Workload:
    """Full-length mutated copies of a 16,569 bp center (configs 1 and 2).

    Queries are drawn in blocks of 1000 with one generator per block, so the
    first 1000 queries of the 100,000-query workload are the 1000-query one.
    ``block0`` starts at block ``block0`` (query 1000 * block0) of the same
    sequence: a rank's shard of a larger workload."""
    center = random_center(center_len, seed)
    src = np.frombuffer(center, np.uint8)
    parts, offs = [], [np.zeros(1, np.int64)]
    for c in range((n + MITO_CHUNK - 1) // MITO_CHUNK):
        m = min(MITO_CHUNK, n - c * MITO_CHUNK)
        rng = np.random.Generator(np.random.PCG64([seed, 1, block0 + c]))
        out, o = mutate_batch(src, np.zeros(MITO_CHUNK, np.int64), np.full(MITO_CHUNK, center_len, np.int64), rng,
                              0.01, 0.001, 0.001, 3.0)
        parts.append(out[: o[m]])
        offs.append(o[1: m + 1] + offs[-1][-1])
    return Workload("mito", center, np.concatenate(parts).tobytes(), np.concatenate(offs),
                    _names("q", block0 * MITO_CHUNK, n))


def divergent(n: int = 50000, seed: int = 4, center_len: int = 5000, chunk: int = 0) -> Workload:
    """High-divergence gap-fill stress (config 4)."""
    center = random_center(center_len, seed)
    src = np.frombuffer(center, np.uint8)
    rng = np.random.Generator(np.random.PCG64([seed, 1, chunk]))
    out, offs = mutate_batch(src, np.zeros(n, np.int64), np.full(n, center_len, np.int64), rng, 0.10, 0.01, 0.01,
                             8.0)
    return Workload("divergent", center, out.tobytes(), offs, _names("d", 0, n))


def _substring_queries(center: bytes, lens: np.ndarray, rng, p_sub, p_ins, p_del, mean, n_run_frac=0.0):
    L = len(center)
    src = np.frombuffer(center, np.uint8)
    starts = rng.integers(0, L - lens + 1)
    out, offs = mutate_batch(src, starts, lens, rng, p_sub, p_ins, p_del, mean)
    if n_run_frac > 0:
        n = len(lens)
        which = np.nonzero(rng.random(n) < n_run_frac)[0]
        for i in which:
            ql = int(offs[i + 1] - offs[i])
            rl = int(min(rng.integers(10, 201), ql))
            s = int(rng.integers(0, ql - rl + 1))
            out[offs[i] + s: offs[i] + s + rl] = ord("N")
    return out, offs


def uneven(n: int = 1000, seed: int = 3, center_len: int = 29903, chunk: int = 0) -> Workload:
    """Uneven-length substrings with N-runs (config 3); generated per chunk."""
    center = random_center(center_len, seed)
    rng = np.random.Generator(np.random.PCG64([seed, 1, chunk]))
    lens = np.clip(np.round(rng.lognormal(np.log(8000.0), 0.5, n)), 300, center_len).astype(np.int64)
    out, offs = _substring_queries(center, lens, rng, 0.001, 0.00025, 0.00025, 3.0, n_run_frac=0.01)
    return Workload("uneven", center, out.tobytes(), offs, _names("u", chunk * n, n))


def serve(n: int = 2000, seed: int = 5, center_len: int = 29903, rate: float = 2000.0, chunk: int = 0) -> Workload:
    """Poisson-arrival align requests of uniform length (config 5)."""
    center = random_center(center_len, seed)
    rng = np.random.Generator(np.random.PCG64([seed, 1, chunk]))
    lens = rng.integers(500, center_len + 1, n).astype(np.int64)
    out, offs = _substring_queries(center, lens, rng, 0.004, 0.0005, 0.0005, 3.0)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n))
    return Workload("serve", center, out.tobytes(), offs, _names("r", chunk * n, n), arrivals)


def multiref(n: int = 200, n_refs: int = 4, seed: int = 6, ref_len: int = 5000, ref_div: float = 0.03,
             chunk: int = 0) -> Workload:
    """Multi-reference mode: ``n_refs`` references of one length (a uniform
    center with ``ref_div`` substitutions each, so that they stay aligned
    column by column) and full-length queries mutated from a random one of
    them (1% substitutions, 0.1% + 0.1% indels, mean 3)."""
    base = np.frombuffer(random_center(ref_len, seed), np.uint8)
    rng_r = np.random.Generator(np.random.PCG64([seed, 2]))
    ref_arr, _ = mutate_batch(base, np.zeros(n_refs, np.int64), np.full(n_refs, ref_len, np.int64), rng_r, ref_div,
                              0.0, 0.0, 3.0)
    refs = [ref_arr[r * ref_len:(r + 1) * ref_len].tobytes() for r in range(n_refs)]
    rng = np.random.Generator(np.random.PCG64([seed, 1, chunk]))
    src_ref = rng.integers(0, n_refs, n)
    out, offs = mutate_batch(ref_arr, src_ref * ref_len, np.full(n, ref_len, np.int64), rng, 0.01, 0.001, 0.001, 3.0)
    return Workload("multiref", refs[0], out.tobytes(), offs, _names("m", chunk * n, n), refs=refs,
                    src_ref=src_ref)


def center_build(n_full: int = 40, n_part: int = 160, seed: int = 21, center_len: int = 5000) -> Workload:
    """Queries for a run that builds its own center (no center file):
    ``n_full`` full-length substitution variants of a uniform center (2%
    substitutions, so that they keep its length and are the longest
    records) shuffled among ``n_part`` shorter substrings (1,500..4,899 bp,
    1% substitutions, 0.1% + 0.1% indels)."""
    base = np.frombuffer(random_center(center_len, seed), np.uint8)
    rng = np.random.Generator(np.random.PCG64([seed, 1]))
    full, fo = mutate_batch(base, np.zeros(n_full, np.int64), np.full(n_full, center_len, np.int64), rng, 0.02, 0.0,
                            0.0, 3.0)
    lens = rng.integers(1500, center_len - 100, n_part)
    starts = rng.integers(0, center_len - lens + 1)
    part, po = mutate_batch(base, starts, lens, rng, 0.01, 0.001, 0.001, 3.0)
    recs = [full[fo[i]:fo[i + 1]].tobytes() for i in range(n_full)] + [part[po[i]:po[i + 1]].tobytes()
                                                                      for i in range(n_part)]
    order = rng.permutation(len(recs))
    seqs = [recs[i] for i in order]
    offs = np.zeros(len(seqs) + 1, np.int64)
    np.cumsum([len(x) for x in seqs], out=offs[1:])
    return Workload("center_build", base.tobytes(), b"".join(seqs), offs, _names("c", 0, len(seqs)))


def write_refs_fasta(path: str, refs: list[bytes]) -> None:
    """The reference FASTA of a multi-reference run: records ref<i> with a
    description, 80 columns per line."""
    with open(path, "wb") as f:
        for r, s in enumerate(refs):
            f.write(b">ref%d reference %d\n" % (r, r))
            for i in range(0, len(s), 80):
                f.write(s[i:i + 80] + b"\n")


def pack_2bit(seqs: bytes, offsets: np.ndarray, align: int = 16):
    """2-bit pack a batch: A=0 C=1 G=2 T=3, base i of a query at bits 2*(i%4) of
    byte i//4; each query starts on an ``align``-byte boundary.  Every other
    byte value (N, lowercase, U, ...) is kept losslessly in an exception list of
    runs (query-relative start, length, byte) and packs as 0.
    Returns (packed uint8, packed_off int64[n], exc int32[m,3] with columns
    start/len/byte, exc_off int64[n+1])."""
    raw = np.frombuffer(seqs, np.uint8)
    n = len(offsets) - 1
    lens = np.diff(offsets)
    nbytes = (lens + 3) // 4
    padded = (nbytes + align - 1) // align * align
    poff = np.zeros(n + 1, np.int64)
    np.cumsum(padded, out=poff[1:])
    lut = np.full(256, 255, np.uint8)
    lut[ord("A")], lut[ord("C")], lut[ord("G")], lut[ord("T")] = 0, 1, 2, 3
    codes = lut[raw]
    is_exc = codes == 255
    codes = np.where(is_exc, 0, codes).astype(np.uint8)
    # per-base destination byte/shift
    q_of = np.repeat(np.arange(n), lens)
    local = np.arange(len(raw), dtype=np.int64) - np.repeat(offsets[:-1], lens)
    dst = poff[q_of] + local // 4
    packed = np.zeros(int(poff[-1]), np.uint8)
    # the four 2-bit sub-positions of a byte never collide: OR them in by shift
    for sh in range(4):
        m = (local % 4) == sh
        packed[dst[m]] |= (codes[m] << (2 * sh)).astype(np.uint8)
    # exception runs
    exc_list = []
    exc_off = np.zeros(n + 1, np.int64)
    if is_exc.any():
        e_idx = np.nonzero(is_exc)[0]
        vals = raw[e_idx]
        # run breaks: new query, non-consecutive position, or different byte
        q_e = q_of[e_idx]
        brk = np.ones(len(e_idx), bool)
        brk[1:] = (np.diff(e_idx) != 1) | (np.diff(q_e) != 0) | (vals[1:] != vals[:-1])
        starts = np.nonzero(brk)[0]
        ends = np.append(starts[1:], len(e_idx))
        runs = np.stack([local[e_idx[starts]], ends - starts, vals[starts]], 1).astype(np.int32)
        exc_list = runs
        cnt = np.bincount(q_e[starts], minlength=n)
        np.cumsum(cnt, out=exc_off[1:])
    exc = np.asarray(exc_list, np.int32).reshape(-1, 3)
    return packed, poff[:-1].copy(), exc, exc_off


def write_fasta(path, center_name: str, center: bytes, w: Workload, center_desc: str = "") -> None:
    """Write the center FASTA and the query FASTA the reference CLI reads."""
    import os
    with open(os.path.join(path, "center.fa"), "wb") as f:
        f.write(b">" + center_name.encode() + ((b" " + center_desc.encode()) if center_desc else b"") + b"\n")
        for i in range(0, len(center), 80):
            f.write(center[i:i + 80] + b"\n")
    with open(os.path.join(path, "queries.fa"), "wb") as f:
        for i in range(w.n):
            f.write(b">" + w.names[i].encode() + b"\n")
            q = w.query(i)
            for j in range(0, len(q), 80):
                f.write(q[j:j + 80] + b"\n")
