"""halign_gb300 - GB300-native align-to-center path of HAlign-4.

Python host binding over the C ABI of ``include/halign_gb300.h`` (the
library ``_build/libhalign_gb300.so`` built from ``csrc/`` by ``build.py``).
Every call here runs the CUDA kernels; there is no CPU fallback: without the
built library or a CUDA device the calls raise ``HalignError``.

Typical use (mirrors RefAligner: one center, many queries):

    ix = Index(center_bytes, k=15, w=10)
    ctx = Context(ix, max_queries=16384, max_bases=300_000_000)
    batch = pack(seqs_bytes, offsets)
    res = ctx.align(batch, rows=True)      # CIGARs, insertion flags, rows
    counts, ins = ctx.counters()           # per-column SiteCount totals
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from pathlib import Path

import numpy as np

# Each context drives five streams (three DP streams, the input and the copy
# stream) and a serving pool runs several contexts at once: with the default
# eight hardware work queues their kernels alias onto shared queues and
# serialise.  Read when the process creates its CUDA context, so it is set
# before the library makes its first call (a value already set is kept).
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libhalign_gb300.so"

HG_OK = 0
HG_ERR_LENGTH_MISMATCH = 5
HG_ERR_CAPACITY = 4
ST_ARENA_OVERFLOW, ST_PARTIAL_CIGAR, ST_CIGAR_OVERFLOW, ST_LENGTH_MISMATCH = 0x01, 0x02, 0x08, 0x10
# hg_ctx_set_launch order: CTAs per SM of six stages, then two DP tier boundaries
LAUNCH_KNOBS = ("seed", "anchor", "chain", "dp_small", "stitch", "rows", "thin_max_inner", "square_max_cells",
                "small_pair", "lanes", "tail_share")
LAUNCH_BOUNDS = ((1, 32), (1, 6), (1, 64), (1, 32), (1, 32), (1, 32), (0, 32), (0, 12288), (0, 1), (1, 2), (0, 24))
DEVICE_KNOBS = 10  # the leading knobs a staged (device-resident) run depends on; tail_share is the host path's
STAGES = ("seed", "anchor", "chain", "dp_small", "dp_large", "stitch", "rows", "count")


# anchor::Anchor as the C ABI's hg_anchor_t (32 bytes)
ANCHOR_DTYPE = np.dtype([("hash", "<u8"), ("rid_ref", "<u4"), ("pos_ref", "<u4"), ("rid_qry", "<u4"),
                         ("pos_qry", "<u4"), ("span", "<u4"), ("is_rev", "<u4")])


class Params(C.Structure):
    """hg_params_t: anchor::SeedFilterParams + anchor::ChainParams."""
    _fields_ = [("f_top_frac", C.c_double), ("u_floor", C.c_uint64), ("u_ceil", C.c_uint64),
                ("q_occ_frac", C.c_double), ("sample_every_bp", C.c_uint64), ("max_dist_x", C.c_int32),
                ("max_dist_y", C.c_int32), ("bw", C.c_int32), ("max_skip", C.c_int32), ("max_iter", C.c_int32),
                ("min_cnt", C.c_int32), ("min_score", C.c_int32), ("gap_penalty", C.c_float),
                ("skip_penalty", C.c_float)]


def params(**overrides) -> Params:
    """The reference's default seeding and chaining parameters with overrides."""
    p = Params()
    lib().hg_default_params(C.byref(p))
    for k, v in overrides.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


class HalignError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


_lib = None


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def lib() -> C.CDLL:
    """Load the native library (build it first with build.py / build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise HalignError(-1, f"native library missing: {LIB_PATH} (run halign-4_gb300/build.py)")
    L = C.CDLL(str(LIB_PATH))
    vp, i64, i32 = C.c_void_p, C.c_int64, C.c_int
    L.hg_last_error.restype = C.c_char_p
    L.hg_device_count.restype = i32
    L.hg_set_device.argtypes = [i32]
    L.hg_index_device.argtypes = [vp, vp, C.c_char_p, i32]
    L.hg_default_params.argtypes = [vp]
    L.hg_index_create.argtypes = [C.c_char_p, i64, i32, i32, vp, C.POINTER(vp)]
    L.hg_index_destroy.argtypes = [vp]
    L.hg_index_info.argtypes = [vp, vp, vp, vp]
    L.hg_ctx_create.argtypes = [vp, i64, i64, C.POINTER(vp)]
    L.hg_ctx_destroy.argtypes = [vp]
    L.hg_pack.argtypes = [vp, vp, i64, vp, i64, vp, vp, i64, vp, vp, vp]
    batch_args = [vp, vp, vp, vp, vp, vp, i64, vp, i64, vp, vp, vp, i64, vp]
    L.hg_align_batch.argtypes = batch_args
    L.hg_align_plain.argtypes = batch_args
    L.hg_align_ascii.argtypes = [vp, vp, vp, i64, vp, i64, vp, vp, vp, i64, vp]
    L.hg_stage.argtypes = [vp, vp, vp, vp, vp, vp, i64]
    L.hg_run_staged.argtypes = [vp]
    L.hg_fetch_staged.argtypes = [vp, vp, i64, vp, vp, vp, i64, vp]
    L.hg_last_timing.argtypes = [vp, vp, vp, vp, vp]
    L.hg_ctx_work.argtypes = [vp, vp, C.c_int]
    L.hg_set_timing.argtypes = [vp, i32]
    L.hg_staged_flags.argtypes = [vp, vp]
    L.hg_submit.argtypes = [vp, vp, vp, vp, vp, vp, i64]
    L.hg_poll.argtypes = [vp]
    L.hg_collect.argtypes = [vp, vp, i64, vp, vp, vp]
    L.hg_counters.argtypes = [vp, vp, vp, i32]
    L.hg_extract_minimizer.argtypes = [C.c_char_p, i64, i32, i32, i32, vp, vp, i64, vp]
    L.hg_extract_minimizer.restype = i64
    L.hg_ksw_extz2.argtypes = [i32, vp, i32, vp, C.c_int8, vp, C.c_int8, C.c_int8, i32, i32, i32, i32, vp, vp, i64]
    L.hg_ksw_extz2.restype = i64
    L.hg_global_align_ksw2.argtypes = [C.c_char_p, i64, C.c_char_p, i64, i32, vp, i64]
    L.hg_global_align_ksw2.restype = i64
    L.hg_align_query.argtypes = [vp, C.c_char_p, i64, vp, i64, vp]
    L.hg_align_query.restype = i64
    L.hg_global_align_mm2.argtypes = [vp, C.c_char_p, i64, vp, vp, i64, vp, i64, vp]
    L.hg_global_align_mm2.restype = i64
    L.hg_ctx_set_launch.argtypes = [vp, vp, i32]
    L.hg_ctx_get_launch.argtypes = [vp, vp, i32]
    L.hg_fetch_chain.argtypes = [vp, i64, vp, vp, vp, vp, i64, vp, vp, vp]
    L.hg_hits_create.argtypes = [vp, vp, i64, vp, C.POINTER(vp)]
    L.hg_hits_destroy.argtypes = [vp]
    L.hg_collect_anchors.argtypes = [vp, vp, vp, i64, vp, vp, i64, vp]
    L.hg_collect_anchors.restype = i64
    L.hg_chain_anchors.argtypes = [vp, i64, vp, vp, i64, vp, vp]
    L.hg_chain_anchors.restype = i64
    L.hg_project_row.argtypes = [C.c_char_p, i64, vp, i64, i32, vp, i64]
    L.hg_project_row.restype = i64
    L.hg_count_rows.argtypes = [vp, i64, i64, i64, vp, i32]
    L.hg_int_peaks.argtypes = [vp, i32]
    L.hg_submit_ascii.argtypes = [vp, vp, vp, i64]
    L.hg_align_fasta.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, i32, i32, i64, vp]
    L.hg_serve_create.argtypes = [vp, i32, i64, i64, i64, C.POINTER(vp)]
    L.hg_serve_destroy.argtypes = [vp]
    L.hg_serve_submit.argtypes = [vp, C.c_char_p, i64]
    L.hg_serve_submit.restype = i64
    L.hg_serve_result.argtypes = [vp, vp, vp, vp, vp, i64, vp, i32]
    L.hg_serve_submit_many.argtypes = [vp, vp, vp, i64]
    L.hg_serve_submit_many.restype = i64
    L.hg_serve_results.argtypes = [vp, i64, vp, vp, vp, vp, i64, vp, i32]
    L.hg_serve_results.restype = i64
    L.hg_serve_stats.argtypes = [vp, vp, i32, i32]
    L.hg_serve_counters.argtypes = [vp, vp, vp, i32]
    L.hg_extend_align_ksw2.argtypes = [C.c_char_p, i64, C.c_char_p, i64, i32, vp, i64]
    L.hg_extend_align_ksw2.restype = i64
    L.hg_last_cells.argtypes = [vp, vp, vp]
    L.hg_build_center.argtypes = [C.c_char_p, i64, vp, i64, vp]
    L.hg_align_fasta_consensus.argtypes = [C.c_char_p, C.c_char_p, i32, i32, i64, i64, vp]
    L.hg_sketch_batch.argtypes = [vp, vp, vp, vp, vp, i64, i32, i32, i32, i32, vp, i64, vp]
    L.hg_refset_create.argtypes = [vp, vp, i32, i32, i32, i32, i32, vp, i64, i64, C.POINTER(vp)]
    L.hg_refset_destroy.argtypes = [vp]
    L.hg_refset_destroy.restype = None
    L.hg_refset_info.argtypes = [vp, vp, vp, vp]
    L.hg_refset_sketch.argtypes = [vp, i32, vp, i64, vp]
    L.hg_refset_consensus.argtypes = [vp, vp, i64, vp]
    L.hg_refset_set_consensus.argtypes = [vp, C.c_char_p, i64]
    L.hg_refset_select.argtypes = [vp, vp, vp, vp, vp, vp, i64, vp, vp]
    L.hg_refset_align.argtypes = [vp, vp, vp, vp, vp, vp, i64, i32, vp, vp, vp, i64, vp, vp, vp, i64, vp]
    L.hg_refset_last_ms.argtypes = [vp, vp]
    _lib = L
    return L


def _check(code: int):
    if code != HG_OK:
        raise HalignError(code, lib().hg_last_error().decode(errors="replace"))


def device_count() -> int:
    return int(lib().hg_device_count())


def set_device(ordinal: int) -> None:
    """Make CUDA device `ordinal` current for this thread (hg_set_device):
    indexes created afterwards, and their contexts, live on it."""
    _check(lib().hg_set_device(int(ordinal)))


def _bytes(s) -> bytes:
    if isinstance(s, str):
        return s.encode("latin-1")
    if isinstance(s, np.ndarray):
        return s.tobytes()
    return bytes(s)


@dataclass
class Packed:
    """A packed batch in the device input format (see hg_pack)."""
    packed: np.ndarray      # uint8
    poff: np.ndarray        # int64[n]
    qlen: np.ndarray        # int32[n]
    exc: np.ndarray         # int32[m*3]
    exc_off: np.ndarray     # int64[n+1]

    @property
    def n(self) -> int:
        return len(self.qlen)

    @property
    def bases(self) -> int:
        return int(self.qlen.sum())

    @property
    def nbytes(self) -> int:
        return self.packed.nbytes + self.poff.nbytes + self.qlen.nbytes + self.exc.nbytes + self.exc_off.nbytes


def pack(seqs: bytes, offsets) -> Packed:
    """Pack concatenated ASCII queries (``offsets``: int64[n+1])."""
    L = lib()
    if not isinstance(seqs, (bytes, bytearray, memoryview)):
        seqs = _bytes(seqs)
    offsets = np.ascontiguousarray(offsets, np.int64)
    n = len(offsets) - 1
    ne = C.c_int64(0)
    buf = np.frombuffer(seqs, np.uint8) if len(seqs) else np.zeros(1, np.uint8)  # no copy
    lens = np.diff(offsets)
    pbytes = int((((lens + 3) // 4 + 15) // 16 * 16).sum()) if n else 0
    packed = np.empty(max(pbytes, 16), np.uint8)  # every byte is written (padding zeroed)
    poff = np.zeros(max(n, 1), np.int64)
    exc = np.zeros(3, np.int32)
    exc_off = np.zeros(n + 1, np.int64)
    # one packing pass; a batch with exception runs packs again into a sized list
    code = L.hg_pack(_p(buf), _p(offsets), n, _p(packed), len(packed), _p(poff), None, 0, _p(exc_off), None,
                     C.byref(ne))
    if code == HG_ERR_CAPACITY and ne.value > 0:
        exc = np.zeros(ne.value * 3, np.int32)
        code = L.hg_pack(_p(buf), _p(offsets), n, _p(packed), len(packed), _p(poff), _p(exc), ne.value,
                         _p(exc_off), None, None)
    _check(code)
    return Packed(packed, poff[:n], lens.astype(np.int32), exc, exc_off)


@dataclass
class AlignResult:
    cigar: np.ndarray       # uint32 ops, concatenated
    cigar_off: np.ndarray   # int64[n+1]
    has_ins: np.ndarray     # uint8[n]
    status: np.ndarray      # uint32[n]
    rows: np.ndarray | None  # uint8[n, L] or None

    def cigar_of(self, i: int) -> np.ndarray:
        return self.cigar[self.cigar_off[i]: self.cigar_off[i + 1]]


class Index:
    """Resident center index (RefAligner's per-center set-up, kept in HBM)."""

    def __init__(self, center, k: int = 15, w: int = 10, prm: Params | None = None):
        L = lib()
        self.center = _bytes(center)
        self.k, self.w = k, w
        h = C.c_void_p()
        _check(L.hg_index_create(self.center, len(self.center), k, w, C.byref(prm) if prm is not None else None,
                                 C.byref(h)))
        self.h = h
        self.L = len(self.center)

    def info(self):
        a, b, c = C.c_int64(), C.c_int64(), C.c_uint64()
        _check(lib().hg_index_info(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def device(self) -> tuple[int, str]:
        """(ordinal, PCI bus id) of the GPU this index lives on."""
        o = C.c_int()
        bus = C.create_string_buffer(32)
        _check(lib().hg_index_device(self.h, C.byref(o), bus, 32))
        return o.value, bus.value.decode()

    def align_query(self, qry) -> np.ndarray:
        q = _bytes(qry)
        cap = len(q) + self.L + 8
        out = np.zeros(cap, np.uint32)
        st = C.c_uint32()
        n = lib().hg_align_query(self.h, q, len(q), _p(out), cap, C.byref(st))
        if n < 0:
            _check(-n)
        return out[:n].copy()

    def global_align_mm2(self, qry, anchor_ref, anchor_qry) -> np.ndarray:
        """align::globalAlignMM2 against the center with the caller's anchors
        (one center, forward strand, span k); returns the CIGAR words."""
        q = _bytes(qry)
        ar = np.ascontiguousarray(anchor_ref, np.uint32)
        aq = np.ascontiguousarray(anchor_qry, np.uint32)
        cap = len(q) + self.L + 8
        out = np.zeros(cap, np.uint32)
        st = C.c_uint32()
        n = lib().hg_global_align_mm2(self.h, q, len(q), _p(ar), _p(aq), len(ar), _p(out), cap, C.byref(st))
        if n < 0:
            _check(-n)
        return out[:n].copy()

    def close(self):
        if getattr(self, "h", None):
            lib().hg_index_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Context:
    """A stream plus device arenas for batches of up to max_queries / max_bases."""

    def __init__(self, index: Index, max_queries: int = 16384, max_bases: int = 1 << 28):
        h = C.c_void_p()
        _check(lib().hg_ctx_create(index.h, max_queries, max_bases, C.byref(h)))
        self.h, self.index = h, index

    def _outputs(self, n: int, bases: int, rows: bool, worst: bool = False):
        # realistic CIGARs are a few ops per kilobase; the worst case is one op
        # per base of query + center
        cap = (bases + n * (self.index.L + 4)) if worst else (bases // 8 + 64 * n + 1024)
        cig = np.zeros(max(cap, 1), np.uint32)
        off = np.zeros(n + 1, np.int64)
        has_ins = np.zeros(max(n, 1), np.uint8)
        status = np.zeros(max(n, 1), np.uint32)
        stride = (self.index.L + 15) // 16 * 16
        rbuf = np.zeros((n, stride), np.uint8) if rows else None
        return cig, off, has_ins, status, rbuf, stride

    def _result(self, cig, off, has_ins, status, rbuf, n):
        rows = rbuf[:, : self.index.L] if rbuf is not None else None
        return AlignResult(cig[: off[-1]] if n else cig[:0], off, has_ins[:n], status[:n], rows)

    def align(self, b: Packed, rows: bool = True, plain: bool = False, check: bool = True) -> AlignResult:
        fn = lib().hg_align_plain if plain else lib().hg_align_batch
        for worst in (False, True):
            cig, off, has_ins, status, rbuf, stride = self._outputs(b.n, b.bases, rows, worst)
            code = fn(self.h, _p(b.packed), _p(b.poff), _p(b.qlen), _p(b.exc), _p(b.exc_off), b.n, _p(cig),
                      len(cig), _p(off), _p(has_ins), _p(rbuf), stride if rows else 0, _p(status))
            if code != 4:  # HG_ERR_CAPACITY: retry once with the worst-case buffer
                break
        if check or code not in (HG_OK, HG_ERR_LENGTH_MISMATCH):
            _check(code)
        return self._result(cig, off, has_ins, status, rbuf, b.n)

    def align_ascii(self, seqs, offsets, rows: bool = True, check: bool = True) -> AlignResult:
        """hg_align_ascii: ASCII queries (query i = seqs[offsets[i]:offsets[i+1]])
        uploaded per sub-batch and packed on the device."""
        s = np.frombuffer(seqs, np.uint8) if isinstance(seqs, (bytes, bytearray)) else np.ascontiguousarray(seqs, np.uint8)
        offs = np.ascontiguousarray(offsets, np.int64)
        n = len(offs) - 1
        bases = int(offs[-1] - offs[0]) if n > 0 else 0
        for worst in (False, True):
            cig, off, has_ins, status, rbuf, stride = self._outputs(n, bases, rows, worst)
            code = lib().hg_align_ascii(self.h, _p(s), _p(offs), n, _p(cig), len(cig), _p(off), _p(has_ins),
                                        _p(rbuf), stride if rows else 0, _p(status))
            if code != 4:  # HG_ERR_CAPACITY: retry once with the worst-case buffer
                break
        if check or code not in (HG_OK, HG_ERR_LENGTH_MISMATCH):
            _check(code)
        return self._result(cig, off, has_ins, status, rbuf, n)

    # device-resident form
    def stage(self, b: Packed):
        _check(lib().hg_stage(self.h, _p(b.packed), _p(b.poff), _p(b.qlen), _p(b.exc), _p(b.exc_off), b.n))
        self._staged = b

    def run_staged(self):
        _check(lib().hg_run_staged(self.h))

    def staged_flags(self) -> int:
        """OR of the per-query status bits of the last staged run (0 = all complete)."""
        f = C.c_uint32()
        _check(lib().hg_staged_flags(self.h, C.byref(f)))
        return f.value

    def fetch_staged(self, rows: bool = True) -> AlignResult:
        b = self._staged
        cig, off, has_ins, status, rbuf, stride = self._outputs(b.n, b.bases, rows, worst=True)
        _check(lib().hg_fetch_staged(self.h, _p(cig), len(cig), _p(off), _p(has_ins), _p(rbuf), stride, _p(status)))
        return self._result(cig, off, has_ins, status, rbuf, b.n)

    # asynchronous form (continuous batching)
    def submit(self, b: Packed):
        _check(lib().hg_submit(self.h, _p(b.packed), _p(b.poff), _p(b.qlen), _p(b.exc), _p(b.exc_off), b.n))
        self._sub = b

    def poll(self) -> bool:
        r = lib().hg_poll(self.h)
        if r < 0:
            _check(-r)
        return r == 1

    def collect(self, check: bool = True) -> AlignResult:
        b = self._sub
        cig, off, has_ins, status, _, _ = self._outputs(b.n, b.bases, False, worst=True)
        code = lib().hg_collect(self.h, _p(cig), len(cig), _p(off), _p(has_ins), _p(status))
        if check or code not in (HG_OK, HG_ERR_LENGTH_MISMATCH):
            _check(code)
        return self._result(cig, off, has_ins, status, None, b.n)

    def set_launch(self, knobs) -> None:
        """CTAs per SM of the seed, anchor, chain, dp_small, stitch and rows stages."""
        k = np.ascontiguousarray([int(x) for x in knobs], np.int32)
        _check(lib().hg_ctx_set_launch(self.h, _p(k), len(k)))

    def get_launch(self) -> list[int]:
        k = np.zeros(len(LAUNCH_KNOBS), np.int32)
        _check(lib().hg_ctx_get_launch(self.h, _p(k), len(k)))
        return [int(x) for x in k]

    def set_timing(self, on: bool):
        _check(lib().hg_set_timing(self.h, int(on)))

    def last_timing(self):
        tot = C.c_float()
        st = np.zeros(8, np.float32)
        la, ce = C.c_int64(), C.c_int64()
        _check(lib().hg_last_timing(self.h, C.byref(tot), _p(st), C.byref(la), C.byref(ce)))
        return tot.value, dict(zip(STAGES, st.tolist())), la.value

    def last_cells(self) -> tuple[int, int]:
        """(cells, match_cells) of the last staged run: the GCUPS work unit and
        its part in match segments (emitted without a DP)."""
        a, m = C.c_int64(), C.c_int64()
        _check(lib().hg_last_cells(self.h, C.byref(a), C.byref(m)))
        return a.value, m.value

    def work(self):
        """Work totals since the context was created: anchors, segment
        records, DP segments (hg_ctx_work)."""
        v = np.zeros(3, np.int64)
        _check(lib().hg_ctx_work(self.h, _p(v), 3))
        return {"anchors": int(v[0]), "records": int(v[1]), "dp_segments": int(v[2])}

    def fetch_chain(self, q: int):
        """Anchors (sorted as chainAnchors sorts them), the chain DP arrays and
        the best chain of staged query q (hg_fetch_chain)."""
        na, end, nc = C.c_int64(), C.c_int64(), C.c_int64()
        _check(lib().hg_fetch_chain(self.h, q, None, None, None, None, 0, C.byref(na), C.byref(end), C.byref(nc)))
        A = na.value
        r, qq = np.zeros(A, np.uint32), np.zeros(A, np.uint32)
        f, pp = np.zeros(A, np.int32), np.zeros(A, np.int32)
        _check(lib().hg_fetch_chain(self.h, q, _p(r), _p(qq), _p(f), _p(pp), A, C.byref(na), C.byref(end),
                                    C.byref(nc)))
        chain = []
        if nc.value > 0:
            c = end.value
            while c >= 0:
                chain.append(c)
                c = int(pp[c])
            chain.reverse()
        return {"pos_ref": r, "pos_qry": qq, "f": f, "p": pp, "chain_end": end.value, "n_chain": nc.value,
                "chain": np.asarray(chain, np.int64)}

    def counters(self, reset: bool = False):
        L = self.index.L
        cnt = np.zeros((L, 7), np.uint32)
        ins = np.zeros(L + 1, np.uint32)
        _check(lib().hg_counters(self.h, _p(cnt), _p(ins), int(reset)))
        return cnt, ins

    def close(self):
        if getattr(self, "h", None):
            lib().hg_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def extract_minimizer(seq, k: int = 15, w: int = 10, non_canonical: bool = True):
    s = _bytes(seq)
    cap = len(s) + 1
    xs = np.zeros(cap, np.uint64)
    ys = np.zeros(cap, np.uint64)
    need = C.c_int64()
    n = lib().hg_extract_minimizer(s, len(s), k, w, int(non_canonical), _p(xs), _p(ys), cap, C.byref(need))
    if n < 0:
        _check(-n)
    return xs[:n].copy(), ys[:n].copy()


def ksw_extz2(query_codes, target_codes, m, mat, q, e, w, zdrop, end_bonus, flag):
    qc = np.ascontiguousarray(query_codes, np.uint8)
    tc = np.ascontiguousarray(target_codes, np.uint8)
    mt = np.ascontiguousarray(mat, np.int8)
    ez = np.zeros(10, np.int32)
    cap = len(qc) + len(tc) + 4
    cig = np.zeros(cap, np.uint32)
    n = lib().hg_ksw_extz2(len(qc), _p(qc), len(tc), _p(tc), m, _p(mt), q, e, w, zdrop, end_bonus, flag, _p(ez),
                           _p(cig), cap)
    if n < 0:
        _check(-n)
    return ez, cig[:n].copy()


def global_align_ksw2(ref, qry, flag: int = -1) -> np.ndarray:
    r, q = _bytes(ref), _bytes(qry)
    cap = len(r) + len(q) + 4
    c = np.zeros(cap, np.uint32)
    n = lib().hg_global_align_ksw2(r, len(r), q, len(q), flag, _p(c), cap)
    if n < 0:
        _check(-n)
    return c[:n].copy()


class Hits:
    """Reference-side minimizer hits of collect_anchors, resident on the GPU
    (hg_hits_create); collect() runs collect_anchors for a query hit list."""

    def __init__(self, ref_x, ref_y, prm: Params | None = None):
        rx = np.ascontiguousarray(ref_x, np.uint64)
        ry = np.ascontiguousarray(ref_y, np.uint64)
        h = C.c_void_p()
        _check(lib().hg_hits_create(_p(rx), _p(ry), len(rx), C.byref(prm) if prm is not None else None,
                                    C.byref(h)))
        self.h = h

    def collect(self, qry_x, qry_y, prm: Params | None = None) -> np.ndarray:
        qx = np.ascontiguousarray(qry_x, np.uint64)
        qy = np.ascontiguousarray(qry_y, np.uint64)
        cap = max(16, 2 * len(qx))
        for _ in range(2):
            out = np.zeros(cap, ANCHOR_DTYPE)
            need = C.c_int64()
            n = lib().hg_collect_anchors(self.h, _p(qx), _p(qy), len(qx), C.byref(prm) if prm is not None else None,
                                         _p(out), cap, C.byref(need))
            if n >= 0:
                return out[:n].copy()
            if n != -HG_ERR_CAPACITY:
                _check(-n)
            cap = need.value
        _check(-n)

    def close(self):
        if getattr(self, "h", None):
            lib().hg_hits_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def chain_anchors(anchors, prm: Params | None = None):
    """anchor::chainAnchors on the GPU: (anchors sorted in place, chain
    indices into them, f, p)."""
    a = np.ascontiguousarray(anchors, ANCHOR_DTYPE).copy()
    n = len(a)
    chain = np.zeros(max(n, 1), np.int64)
    f = np.zeros(max(n, 1), np.int32)
    pp = np.zeros(max(n, 1), np.int64)
    m = lib().hg_chain_anchors(_p(a), n, C.byref(prm) if prm is not None else None, _p(chain), len(chain), _p(f),
                               _p(pp))
    if m < 0:
        _check(-m)
    return a, chain[:m].copy(), f[:n].copy(), pp[:n].copy()


def project_row(qry, cigar, pad: bool = False) -> bytes:
    """delQueryToRefByCigar (pad=False) / padQueryToRefByCigar (pad=True) on the GPU."""
    q = _bytes(qry)
    c = np.ascontiguousarray(cigar, np.uint32)
    cap = len(q) + int(sum(int(x) >> 4 for x in c)) + 16
    out = np.zeros(max(cap, 1), np.uint8)
    n = lib().hg_project_row(q, len(q), _p(c), len(c), int(pad), _p(out), cap)
    if n < 0:
        _check(-n)
    return out[:n].tobytes()


INT_PEAK_KEYS = ("int32_add_max_ops", "dpx_s32_ops", "dpx_s16x2_ops", "dpx_max3_s16x2_ops", "mul64_ops",
                 "int_pipe_warp_inst", "vsub2_ops", "vcmpgts2_ops")


def int_peaks() -> dict:
    """Measured integer / DPX throughput ceilings of the current GPU (per second)."""
    v = np.zeros(len(INT_PEAK_KEYS), np.float64)
    _check(lib().hg_int_peaks(_p(v), len(v)))
    return dict(zip(INT_PEAK_KEYS, (float(x) for x in v)))


def extend_align_ksw2(ref, qry, zdrop: int = 200) -> np.ndarray:
    """align::extendAlignKSW2 on the GPU."""
    r, q = _bytes(ref), _bytes(qry)
    cap = len(r) + len(q) + 4
    c = np.zeros(cap, np.uint32)
    n = lib().hg_extend_align_ksw2(r, len(r), q, len(q), zdrop, _p(c), cap)
    if n < 0:
        _check(-n)
    return c[:n].copy()


def align_fasta(center_fasta, queries_fasta, out_fasta, k: int = 15, w: int = 10,
                chunk_queries: int = 50000) -> int:
    """Aligned FASTA of a query FASTA against the first record of a center
    FASTA, in the reference CLI's --keep-length output order (hg_align_fasta).
    Returns the number of queries aligned."""
    n = C.c_int64()
    _check(lib().hg_align_fasta(str(center_fasta).encode(), str(queries_fasta).encode(), str(out_fasta).encode(),
                                k, w, chunk_queries, C.byref(n)))
    return n.value


SKETCH_MAX = 8192  # HG_SKETCH_MAX


def sketch_batch(b: Packed, k: int = 15, sketch_size: int = 2000, noncanonical: bool = True,
                 seed: int = 42) -> list[np.ndarray]:
    """mash::sketchFromSequence of every query of a packed batch on the
    device (hg_sketch_batch): per query the sorted distinct bottom-sketch_size
    hashes."""
    s = max(int(sketch_size), 0)
    out = np.zeros((max(b.n, 1), max(s, 1)), np.uint64)
    cnt = np.zeros(max(b.n, 1), np.int32)
    _check(lib().hg_sketch_batch(_p(b.packed), _p(b.poff), _p(b.qlen), _p(b.exc), _p(b.exc_off), b.n, k, s,
                                 int(noncanonical), seed, _p(out), out.shape[1], _p(cnt)))
    return [out[i, : cnt[i]].copy() for i in range(b.n)]


@dataclass
class RefAlignResult(AlignResult):
    best: np.ndarray | None = None     # int32[n]: chosen reference
    jaccard: np.ndarray | None = None  # float64[n]


class RefSet:
    """Multi-reference mode (hg_refset_*): resident indexes and sketches of
    several references, best-reference selection and alignment."""

    def __init__(self, refs, k: int = 15, w: int = 10, sketch_size: int = 2000, seed: int = 42,
                 prm: Params | None = None, max_queries: int = 16384, max_bases: int = 1 << 28):
        self.refs = [_bytes(r) for r in refs]
        arr = (C.c_char_p * len(self.refs))(*self.refs)
        lens = np.array([len(r) for r in self.refs], np.int64)
        h = C.c_void_p()
        _check(lib().hg_refset_create(C.cast(arr, C.c_void_p), _p(lens), len(self.refs), k, w, sketch_size, seed,
                                      C.byref(prm) if prm is not None else None, max_queries, max_bases, C.byref(h)))
        self.h = h
        self.max_len = int(lens.max())

    def sketch(self, r: int) -> np.ndarray:
        n = C.c_int64()
        out = np.zeros(SKETCH_MAX, np.uint64)
        _check(lib().hg_refset_sketch(self.h, r, _p(out), len(out), C.byref(n)))
        return out[: n.value].copy()

    def consensus(self) -> bytes:
        n, clen = C.c_int64(), C.c_int64()
        _check(lib().hg_refset_info(self.h, None, None, C.byref(clen)))
        buf = C.create_string_buffer(max(clen.value, 1))
        _check(lib().hg_refset_consensus(self.h, buf, len(buf), C.byref(n)))
        return buf.raw[: n.value]

    def set_consensus(self, seq) -> None:
        b = _bytes(seq)
        _check(lib().hg_refset_set_consensus(self.h, b, len(b)))

    def select(self, b: Packed) -> tuple[np.ndarray, np.ndarray]:
        best = np.zeros(max(b.n, 1), np.int32)
        jac = np.zeros(max(b.n, 1), np.float64)
        _check(lib().hg_refset_select(self.h, _p(b.packed), _p(b.poff), _p(b.qlen), _p(b.exc), _p(b.exc_off), b.n,
                                      _p(best), _p(jac)))
        return best[: b.n], jac[: b.n]

    def last_select_ms(self) -> float:
        """Device time of the last select's sketch + selection launch."""
        ms = C.c_float()
        _check(lib().hg_refset_last_ms(self.h, C.byref(ms)))
        return float(ms.value)

    def align(self, b: Packed, keep_length: bool = True, rows: bool = True, check: bool = True) -> RefAlignResult:
        n = b.n
        clen = C.c_int64()
        _check(lib().hg_refset_info(self.h, None, None, C.byref(clen)))
        L = max(self.max_len, clen.value)
        stride = (L + 15) // 16 * 16
        best = np.zeros(max(n, 1), np.int32)
        jac = np.zeros(max(n, 1), np.float64)
        for worst in (False, True):
            cap = (b.bases + n * (L + 4)) if worst else (b.bases // 8 + 64 * n + 1024)
            cig = np.zeros(max(cap, 1), np.uint32)
            off = np.zeros(n + 1, np.int64)
            has_ins = np.zeros(max(n, 1), np.uint8)
            status = np.zeros(max(n, 1), np.uint32)
            rbuf = np.zeros((n, stride), np.uint8) if rows else None
            code = lib().hg_refset_align(self.h, _p(b.packed), _p(b.poff), _p(b.qlen), _p(b.exc), _p(b.exc_off), n,
                                         int(keep_length), _p(best), _p(jac), _p(cig), len(cig), _p(off),
                                         _p(has_ins), _p(rbuf), stride if rows else 0, _p(status))
            if code != HG_ERR_CAPACITY:
                break
        if check or code not in (HG_OK, HG_ERR_LENGTH_MISMATCH):
            _check(code)
        return RefAlignResult(cig[: off[-1]] if n else cig[:0], off, has_ins[:n], status[:n],
                              rbuf if rows else None, best[:n], jac[:n])

    def close(self):
        if getattr(self, "h", None):
            lib().hg_refset_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def build_center(queries_fasta, cons_n: int = 1000) -> bytes:
    """The center the CLI builds without -c (hg_build_center): consensus of
    the cons_n longest records (which must share one length)."""
    n = C.c_int64()
    code = lib().hg_build_center(str(queries_fasta).encode(), cons_n, None, 0, C.byref(n))
    if code not in (HG_OK, HG_ERR_CAPACITY):
        _check(code)
    buf = C.create_string_buffer(max(n.value, 1))
    _check(lib().hg_build_center(str(queries_fasta).encode(), cons_n, buf, len(buf), C.byref(n)))
    return buf.raw[: n.value]


def align_fasta_consensus(queries_fasta, out_fasta, k: int = 15, w: int = 10, cons_n: int = 1000,
                          chunk_queries: int = 50000) -> int:
    """The CLI's run without a center file (hg_align_fasta_consensus)."""
    n = C.c_int64()
    _check(lib().hg_align_fasta_consensus(str(queries_fasta).encode(), str(out_fasta).encode(), k, w, cons_n,
                                          chunk_queries, C.byref(n)))
    return n.value


def count_rows(rows: np.ndarray, counts: np.ndarray | None = None) -> np.ndarray:
    """SiteCount totals (L x 7: A C G T U N -) of the rows of a 2-D uint8
    array, added to `counts` when given."""
    r = np.ascontiguousarray(rows, np.uint8)
    n, L = r.shape
    out = np.zeros((L, 7), np.uint32) if counts is None else np.ascontiguousarray(counts, np.uint32).copy()
    _check(lib().hg_count_rows(_p(r), n, L, L, _p(out), int(counts is not None)))
    return out


def build_library(force: bool = False) -> Path:
    """Compile csrc/ into _build/libhalign_gb300.so (sm_103a)."""
    import importlib
    return importlib.import_module(__name__ + ".build").build(force=force)
