"""ctypes bindings for the test oracle (and, where built, the reference harness).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
bench.py's CPU-baseline leg, always as the checker or the timed CPU baseline,
never as part of the product path.

``Oracle`` wraps oracle/_build/libhalign_oracle.so (the C restatement).
``Reference`` wraps oracle/_ref/libhalign_ref.so (the unmodified HAlign-4
sources) and exists only where the reference tree was available at build time.
Both expose the same method names so a test can run one case through each.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

HERE = Path(__file__).resolve().parent

ANCHOR_DTYPE = np.dtype([("hash", "<u8"), ("rid_ref", "<u4"), ("pos_ref", "<u4"), ("rid_qry", "<u4"),
                         ("pos_qry", "<u4"), ("span", "<u4"), ("is_rev", "<u4")])

_p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731


def _bytes(s) -> bytes:
    if isinstance(s, str):
        return s.encode("latin-1")
    if isinstance(s, np.ndarray):
        return s.tobytes()
    return bytes(s)


class _Common:
    lib: C.CDLL

    # ---- CIGAR helpers shared by both libraries (pure python) ----
    @staticmethod
    def cigar_str(c) -> str:
        return "".join(f"{int(x) >> 4}{'MIDNSHP=X'[int(x) & 0xf]}" for x in c)


class Oracle(_Common):
    def __init__(self, path: Path | None = None):
        path = path or _build.build_oracle()
        L = self.lib = C.CDLL(str(path))
        vp, i64, i32 = C.c_void_p, C.c_int64, C.c_int
        L.ho_extract_minimizer.argtypes = [C.c_char_p, i64, i32, i32, i32, vp, vp, i64]
        L.ho_extract_minimizer.restype = i64
        L.ho_collect_anchors.argtypes = [vp, vp, i64, vp, vp, i64, vp, vp, i64]
        L.ho_collect_anchors.restype = i64
        L.ho_chain_anchors.argtypes = [vp, i64, vp, vp, i64]
        L.ho_chain_anchors.restype = i64
        L.ho_chain_anchors_fp.argtypes = [vp, i64, vp, vp, i64, vp, vp]
        L.ho_chain_anchors_fp.restype = i64
        L.ho_chain_score.argtypes = [vp, vp, vp]
        L.ho_chain_score.restype = C.c_int32
        L.ho_ksw_extz2.argtypes = [i32, vp, i32, vp, C.c_int8, vp, C.c_int8, C.c_int8, i32, i32, i32, i32, vp,
                                   vp, i64]
        L.ho_ksw_extz2.restype = i64
        L.ho_global_align_ksw2.argtypes = [C.c_char_p, i64, C.c_char_p, i64, i32, vp, i64]
        L.ho_global_align_ksw2.restype = i64
        L.ho_global_align_mm2.argtypes = [C.c_char_p, i64, C.c_char_p, i64, vp, i64, vp, i64]
        L.ho_global_align_mm2.restype = i64
        L.ho_align_query.argtypes = [C.c_char_p, i64, vp, vp, i64, C.c_char_p, i64, i32, i32, vp, i64]
        L.ho_align_query.restype = i64
        L.ho_align_batch.argtypes = [C.c_char_p, i64, C.c_char_p, i64, vp, vp, i64, i32, i32, i32, vp, i64, vp]
        L.ho_align_batch.restype = C.c_double
        L.ho_del_query.argtypes = [C.c_char_p, i64, vp, i64, vp, i64]
        L.ho_del_query.restype = i64
        L.ho_count_rows.argtypes = [vp, i64, i64, vp]
        L.ho_count_insertions.argtypes = [vp, i64, vp, i64]
        L.ho_pick_consensus.argtypes = [vp]
        L.ho_pick_consensus.restype = C.c_char
        L.ho_auto_band.argtypes = [i32, i32]
        L.ho_auto_band.restype = i32
        L.ho_log2_table.restype = C.POINTER(C.c_float)
        L.ho_last_ring_oob.restype = C.c_int64
        L.ho_cigar_has_insertion.argtypes = [vp, i64]
        L.ho_cigar_has_insertion.restype = i32
        L.ho_hash2bit.argtypes = [C.c_uint64, C.c_uint32]
        L.ho_hash2bit.restype = C.c_uint64
        L.ho_sketch.argtypes = [C.c_char_p, i64, i32, i64, i32, i32, vp]
        L.ho_sketch.restype = i64
        L.ho_jaccard.argtypes = [vp, i64, vp, i64]
        L.ho_jaccard.restype = C.c_double
        L.ho_best_reference.argtypes = [vp, i64, vp, vp, C.c_int32, vp]
        L.ho_best_reference.restype = C.c_int32

    def last_ring_oob(self) -> int:
        return int(self.lib.ho_last_ring_oob())

    def log2_table(self) -> np.ndarray:
        p = self.lib.ho_log2_table()
        return np.ctypeslib.as_array(p, shape=(513,)).copy()

    def extract_minimizer(self, seq, k=15, w=10, non_canonical=True):
        b = _bytes(seq)
        cap = len(b) + 1
        xs = np.zeros(cap, np.uint64)
        ys = np.zeros(cap, np.uint64)
        n = self.lib.ho_extract_minimizer(b, len(b), k, w, int(non_canonical), _p(xs), _p(ys), cap)
        assert n >= 0
        return xs[:n].copy(), ys[:n].copy()

    @staticmethod
    def _filter(filter_params):
        if filter_params is None:
            return None
        arr = np.zeros(1, np.dtype([("f", "<f8"), ("uf", "<u8"), ("uc", "<u8"), ("q", "<f8"), ("e", "<u8")]))
        arr[0] = tuple(filter_params)
        return arr

    def collect_anchors(self, rx, ry, qx, qy, filter_params=None):
        rx, ry, qx, qy = (np.ascontiguousarray(a, np.uint64) for a in (rx, ry, qx, qy))
        fp = self._filter(filter_params)
        cap = max(16, len(qx) * 4)
        while True:
            out = np.zeros(cap, ANCHOR_DTYPE)
            n = self.lib.ho_collect_anchors(_p(rx), _p(ry), len(rx), _p(qx), _p(qy), len(qx),
                                            _p(fp) if fp is not None else None, _p(out), cap)
            if n >= 0:
                return out[:n].copy()
            cap = -n

    @staticmethod
    def _chain_params(iparams, fparams):
        if iparams is None and fparams is None:
            return None
        arr = np.zeros(1, np.dtype([("i", "<i4", 7), ("f", "<f4", 2)]))
        arr["i"][0] = iparams if iparams is not None else [5000, 5000, 500, 25, 5000, 3, 40]
        arr["f"][0] = fparams if fparams is not None else [0.01, 0.01]
        return arr

    def chain_anchors(self, anchors, iparams=None, fparams=None):
        a = np.ascontiguousarray(anchors, ANCHOR_DTYPE).copy()
        out = np.zeros(max(1, len(a)), ANCHOR_DTYPE)
        prm = self._chain_params(iparams, fparams)
        n = self.lib.ho_chain_anchors(_p(a), len(a), _p(prm) if prm is not None else None, _p(out), len(out))
        assert n >= 0
        return a, out[:n].copy()

    def chain_anchors_fp(self, anchors, iparams=None, fparams=None):
        """chainAnchors plus its DP arrays: (sorted anchors, chain, f, p)."""
        a = np.ascontiguousarray(anchors, ANCHOR_DTYPE).copy()
        out = np.zeros(max(1, len(a)), ANCHOR_DTYPE)
        f = np.zeros(max(1, len(a)), np.int32)
        pr = np.zeros(max(1, len(a)), np.int64)
        prm = self._chain_params(iparams, fparams)
        n = self.lib.ho_chain_anchors_fp(_p(a), len(a), _p(prm) if prm is not None else None, _p(out), len(out),
                                         _p(f), _p(pr))
        assert n >= 0
        return a, out[:n].copy(), f[:len(a)].copy(), pr[:len(a)].copy()

    def chain_score(self, ai_ref, ai_qry, aj_ref, aj_qry, aj_span):
        a = np.zeros(2, ANCHOR_DTYPE)
        a[0]["pos_ref"], a[0]["pos_qry"] = ai_ref, ai_qry
        a[1]["pos_ref"], a[1]["pos_qry"], a[1]["span"] = aj_ref, aj_qry, aj_span
        prm = self._chain_params([5000, 5000, 500, 25, 5000, 3, 40], [0.01, 0.01])
        return int(self.lib.ho_chain_score(_p(a[0:1]), _p(a[1:2]), _p(prm)))

    def ksw_extz2(self, query_codes, target_codes, m, mat, q, e, w, zdrop, end_bonus, flag):
        qc = np.ascontiguousarray(query_codes, np.uint8)
        tc = np.ascontiguousarray(target_codes, np.uint8)
        mt = np.ascontiguousarray(mat, np.int8)
        ez = np.zeros(10, np.int32)
        cap = len(qc) + len(tc) + 4
        cig = np.zeros(cap, np.uint32)
        n = self.lib.ho_ksw_extz2(len(qc), _p(qc), len(tc), _p(tc), m, _p(mt), q, e, w, zdrop, end_bonus, flag,
                                  _p(ez), _p(cig), cap)
        assert n >= 0, n
        return ez, cig[:n].copy()

    def global_align_ksw2(self, ref, qry, flag=-1):
        r, q = _bytes(ref), _bytes(qry)
        cap = len(r) + len(q) + 4
        c = np.zeros(cap, np.uint32)
        n = self.lib.ho_global_align_ksw2(r, len(r), q, len(q), flag, _p(c), cap)
        assert n >= 0
        return c[:n].copy()

    def global_align_mm2(self, ref, qry, anchors):
        r, q = _bytes(ref), _bytes(qry)
        a = np.ascontiguousarray(anchors, ANCHOR_DTYPE)
        cap = len(r) + len(q) + 4
        c = np.zeros(cap, np.uint32)
        n = self.lib.ho_global_align_mm2(r, len(r), q, len(q), _p(a), len(a), _p(c), cap)
        assert n >= 0
        return c[:n].copy()

    def align_query(self, center_dp, cmx, cmy, qry, k=15, w=10):
        c_, q = _bytes(center_dp), _bytes(qry)
        cmx, cmy = np.ascontiguousarray(cmx, np.uint64), np.ascontiguousarray(cmy, np.uint64)
        cap = len(c_) + len(q) + 4
        c = np.zeros(cap, np.uint32)
        n = self.lib.ho_align_query(c_, len(c_), _p(cmx), _p(cmy), len(cmx), q, len(q), k, w, _p(c), cap)
        assert n >= 0
        return c[:n].copy()

    def align_batch(self, center_dp, center_raw, seqs: bytes, offsets, k=15, w=10, nthreads=1, cap_per_query=None):
        offsets = np.ascontiguousarray(offsets, np.int64)
        n = len(offsets) - 1
        if cap_per_query is None:
            cap_per_query = int(np.max(np.diff(offsets))) + len(center_dp) + 4 if n else 4
        cig = np.zeros(n * cap_per_query, np.uint32)
        ncig = np.zeros(n, np.int64)
        sb = np.frombuffer(seqs, np.uint8)
        cd, cr = _bytes(center_dp), _bytes(center_raw)
        t = self.lib.ho_align_batch(cd, len(cd), cr, len(cr), _p(sb), _p(offsets), n, k, w, nthreads, _p(cig),
                                    cap_per_query, _p(ncig))
        return t, [cig[i * cap_per_query: i * cap_per_query + ncig[i]].copy() for i in range(n)]

    def del_query(self, qry, cigar):
        q = _bytes(qry)
        c = np.ascontiguousarray(cigar, np.uint32)
        cap = len(q) + int(sum(int(x) >> 4 for x in c)) + 1
        out = np.zeros(cap, np.uint8)
        n = self.lib.ho_del_query(q, len(q), _p(c), len(c), _p(out), cap)
        assert n >= 0
        return out[:n].tobytes()

    def count_rows(self, rows: np.ndarray):
        rows = np.ascontiguousarray(rows, np.uint8)
        n, L = rows.shape
        cnt = np.zeros((L, 7), np.uint32)
        self.lib.ho_count_rows(_p(rows), n, L, _p(cnt))
        return cnt

    def count_insertions(self, cigar, L, ins=None):
        c = np.ascontiguousarray(cigar, np.uint32)
        if ins is None:
            ins = np.zeros(L + 1, np.uint32)
        self.lib.ho_count_insertions(_p(c), len(c), _p(ins), L)
        return ins

    def pick_consensus(self, counts7) -> str:
        k = np.ascontiguousarray(counts7, np.uint32)
        return self.lib.ho_pick_consensus(_p(k)).decode()

    def auto_band(self, qlen, tlen):
        return self.lib.ho_auto_band(qlen, tlen)

    def has_insertion(self, cigar) -> bool:
        c = np.ascontiguousarray(cigar, np.uint32)
        return bool(self.lib.ho_cigar_has_insertion(_p(c), len(c)))

    # ---- multi-reference mode (MinHash) ----
    def hash2bit(self, code: int, seed: int = 42) -> int:
        return int(self.lib.ho_hash2bit(code, seed))

    def sketch(self, seq, k=15, sketch_size=2000, noncanonical=True, seed=42) -> np.ndarray:
        b = _bytes(seq)
        out = np.zeros(max(1, min(sketch_size, len(b) + 1)), np.uint64)
        n = self.lib.ho_sketch(b, len(b), k, sketch_size, int(noncanonical), seed, _p(out))
        return out[:n].copy()

    def jaccard(self, a, b) -> float:
        a = np.ascontiguousarray(a, np.uint64)
        b = np.ascontiguousarray(b, np.uint64)
        return float(self.lib.ho_jaccard(_p(a), len(a), _p(b), len(b)))

    def best_reference(self, q, ref_sketches) -> tuple[int, float]:
        q = np.ascontiguousarray(q, np.uint64)
        flat = np.ascontiguousarray(np.concatenate([np.asarray(r, np.uint64) for r in ref_sketches] or
                                                   [np.zeros(0, np.uint64)]), np.uint64)
        off = np.zeros(len(ref_sketches) + 1, np.int64)
        np.cumsum([len(r) for r in ref_sketches], out=off[1:])
        bj = np.zeros(1, np.float64)
        r = self.lib.ho_best_reference(_p(q), len(q), _p(flat), _p(off), len(ref_sketches), _p(bj))
        return int(r), float(bj[0])


class Reference(_Common):
    """The unmodified reference sources (only where oracle/_ref was built)."""

    def __init__(self, path: Path | None = None):
        path = path or _build.build_ref()
        if path is None:
            raise FileNotFoundError("reference harness unavailable (no reference tree or not x86-64)")
        L = self.lib = C.CDLL(str(path))
        vp, i64, i32 = C.c_void_p, C.c_int64, C.c_int
        L.ref_extract_minimizer.argtypes = [C.c_char_p, i64, i32, i32, i32, vp, vp, i64]
        L.ref_extract_minimizer.restype = i64
        L.ref_collect_anchors.argtypes = [vp, vp, i64, vp, vp, i64, vp] + [vp] * 7 + [i64]
        L.ref_collect_anchors.restype = i64
        L.ref_chain_anchors.argtypes = [vp] * 7 + [i64, vp, vp] + [vp] * 7 + [i64]
        L.ref_chain_anchors.restype = i64
        L.ref_ksw_extz2.argtypes = [i32, vp, i32, vp, C.c_int8, vp, C.c_int8, C.c_int8, i32, i32, i32, i32, vp, vp,
                                    i64]
        L.ref_ksw_extz2.restype = i64
        L.ref_global_align_ksw2.argtypes = [C.c_char_p, i64, C.c_char_p, i64, i32, vp, i64]
        L.ref_global_align_ksw2.restype = i64
        L.ref_global_align_mm2.argtypes = [C.c_char_p, i64, C.c_char_p, i64] + [vp] * 7 + [i64, vp, i64]
        L.ref_global_align_mm2.restype = i64
        L.ref_align_query.argtypes = [C.c_char_p, i64, C.c_char_p, i64, i32, i32, vp, i64]
        L.ref_align_query.restype = i64
        L.ref_align_batch.argtypes = [C.c_char_p, i64, vp, vp, i64, i32, i32, i32, vp, i64, vp]
        L.ref_align_batch.restype = C.c_double
        L.ref_del_query.argtypes = [C.c_char_p, i64, vp, i64, vp, i64]
        L.ref_del_query.restype = i64
        L.ref_pick_consensus.argtypes = [vp]
        L.ref_pick_consensus.restype = C.c_char
        L.ref_auto_band.argtypes = [i32, i32]
        L.ref_auto_band.restype = i32
        L.ref_chain_score.argtypes = [C.c_uint32] * 5
        L.ref_chain_score.restype = C.c_int32
        L.ref_pad_query.argtypes = [C.c_char_p, i64, vp, i64, vp, i64]
        L.ref_pad_query.restype = i64
        L.ref_extend_align_ksw2.argtypes = [C.c_char_p, i64, C.c_char_p, i64, i32, vp, i64]
        L.ref_extend_align_ksw2.restype = i64
        L.ref_generate_consensus.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_uint64, i64, vp, i64]
        L.ref_generate_consensus.restype = i64
        L.ref_hash2bit.argtypes = [C.c_uint64, C.c_uint32]
        L.ref_hash2bit.restype = C.c_uint64
        L.ref_sketch.argtypes = [C.c_char_p, i64, i32, i64, i32, i32, vp, i64]
        L.ref_sketch.restype = i64
        L.ref_jaccard.argtypes = [vp, i64, vp, i64, i32]
        L.ref_jaccard.restype = C.c_double

    @staticmethod
    def _split(a):
        return [a[f] for f in ("hash", "rid_ref", "pos_ref", "rid_qry", "pos_qry", "span")]

    def hash2bit(self, code: int, seed: int = 42) -> int:
        return int(self.lib.ref_hash2bit(code, seed))

    def sketch(self, seq, k=15, sketch_size=2000, noncanonical=True, seed=42) -> np.ndarray:
        b = _bytes(seq)
        cap = max(1, min(sketch_size, len(b) + 1))
        out = np.zeros(cap, np.uint64)
        n = self.lib.ref_sketch(b, len(b), k, sketch_size, int(noncanonical), seed, _p(out), cap)
        assert n >= 0
        return out[:n].copy()

    def jaccard(self, a, b, k=15) -> float:
        a = np.ascontiguousarray(a, np.uint64)
        b = np.ascontiguousarray(b, np.uint64)
        return float(self.lib.ref_jaccard(_p(a), len(a), _p(b), len(b), k))

    def extract_minimizer(self, seq, k=15, w=10, non_canonical=True):
        b = _bytes(seq)
        cap = len(b) + 1
        xs = np.zeros(cap, np.uint64)
        ys = np.zeros(cap, np.uint64)
        n = self.lib.ref_extract_minimizer(b, len(b), k, w, int(non_canonical), _p(xs), _p(ys), cap)
        assert n >= 0
        return xs[:n].copy(), ys[:n].copy()

    def collect_anchors(self, rx, ry, qx, qy, filter_params=None):
        rx, ry, qx, qy = (np.ascontiguousarray(a, np.uint64) for a in (rx, ry, qx, qy))
        fp = None if filter_params is None else np.asarray(filter_params, np.float64)
        cap = max(16, len(qx) * 4)
        while True:
            cols = [np.zeros(cap, np.uint64)] + [np.zeros(cap, np.uint32) for _ in range(5)] + [np.zeros(cap, np.uint8)]
            n = self.lib.ref_collect_anchors(_p(rx), _p(ry), len(rx), _p(qx), _p(qy), len(qx),
                                             _p(fp) if fp is not None else None, *[_p(c) for c in cols], cap)
            if n >= 0:
                break
            cap = -n
        out = np.zeros(n, ANCHOR_DTYPE)
        for name, col in zip(ANCHOR_DTYPE.names, cols):
            out[name] = col[:n]
        return out

    def chain_anchors(self, anchors, iparams=None, fparams=None):
        a = np.ascontiguousarray(anchors, ANCHOR_DTYPE)
        n = len(a)
        cols = [np.ascontiguousarray(a[f]) .astype(np.uint64 if f == "hash" else np.uint32) for f in
                ("hash", "rid_ref", "pos_ref", "rid_qry", "pos_qry", "span")] + [a["is_rev"].astype(np.uint8)]
        cap = max(1, n)
        outs = [np.zeros(cap, np.uint64)] + [np.zeros(cap, np.uint32) for _ in range(5)] + [np.zeros(cap, np.uint8)]
        ip = None if iparams is None else np.asarray(iparams, np.int32)
        fpp = None if fparams is None else np.asarray(fparams, np.float32)
        if ip is None and fpp is not None:
            ip = np.array([5000, 5000, 500, 25, 5000, 3, 40], np.int32)
        m = self.lib.ref_chain_anchors(*[_p(c) for c in cols], n, _p(ip) if ip is not None else None,
                                       _p(fpp) if fpp is not None else None, *[_p(c) for c in outs], cap)
        assert m >= 0
        srt = np.zeros(n, ANCHOR_DTYPE)
        for name, col in zip(ANCHOR_DTYPE.names, cols):
            srt[name] = col
        res = np.zeros(m, ANCHOR_DTYPE)
        for name, col in zip(ANCHOR_DTYPE.names, outs):
            res[name] = col[:m]
        return srt, res

    def ksw_extz2(self, query_codes, target_codes, m, mat, q, e, w, zdrop, end_bonus, flag):
        qc = np.ascontiguousarray(query_codes, np.uint8)
        tc = np.ascontiguousarray(target_codes, np.uint8)
        mt = np.ascontiguousarray(mat, np.int8)
        ez = np.zeros(10, np.int32)
        cap = len(qc) + len(tc) + 4
        cig = np.zeros(cap, np.uint32)
        n = self.lib.ref_ksw_extz2(len(qc), _p(qc), len(tc), _p(tc), m, _p(mt), q, e, w, zdrop, end_bonus, flag,
                                   _p(ez), _p(cig), cap)
        assert n >= 0
        return ez, cig[:n].copy()

    def global_align_ksw2(self, ref, qry, flag=-1):
        r, q = _bytes(ref), _bytes(qry)
        cap = len(r) + len(q) + 4
        c = np.zeros(cap, np.uint32)
        n = self.lib.ref_global_align_ksw2(r, len(r), q, len(q), flag, _p(c), cap)
        assert n >= 0
        return c[:n].copy()

    def global_align_mm2(self, ref, qry, anchors):
        r, q = _bytes(ref), _bytes(qry)
        a = np.ascontiguousarray(anchors, ANCHOR_DTYPE)
        cols = [np.ascontiguousarray(a[f]).astype(np.uint64 if f == "hash" else np.uint32) for f in
                ("hash", "rid_ref", "pos_ref", "rid_qry", "pos_qry", "span")] + [a["is_rev"].astype(np.uint8)]
        cap = len(r) + len(q) + 4
        c = np.zeros(cap, np.uint32)
        n = self.lib.ref_global_align_mm2(r, len(r), q, len(q), *[_p(x) for x in cols], len(a), _p(c), cap)
        assert n >= 0
        return c[:n].copy()

    def align_query_full(self, center, qry, k=15, w=10):
        c_, q = _bytes(center), _bytes(qry)
        cap = len(c_) + len(q) + 4
        c = np.zeros(cap, np.uint32)
        n = self.lib.ref_align_query(c_, len(c_), q, len(q), k, w, _p(c), cap)
        assert n >= 0
        return c[:n].copy()

    def align_batch(self, center, seqs: bytes, offsets, k=15, w=10, nthreads=1, cap_per_query=None):
        offsets = np.ascontiguousarray(offsets, np.int64)
        n = len(offsets) - 1
        if cap_per_query is None:
            cap_per_query = int(np.max(np.diff(offsets))) + len(center) + 4 if n else 4
        cig = np.zeros(n * cap_per_query, np.uint32)
        ncig = np.zeros(n, np.int64)
        sb = np.frombuffer(seqs, np.uint8)
        c_ = _bytes(center)
        t = self.lib.ref_align_batch(c_, len(c_), _p(sb), _p(offsets), n, k, w, nthreads, _p(cig), cap_per_query,
                                     _p(ncig))
        return t, [cig[i * cap_per_query: i * cap_per_query + ncig[i]].copy() for i in range(n)]

    def del_query(self, qry, cigar):
        q = _bytes(qry)
        c = np.ascontiguousarray(cigar, np.uint32)
        cap = len(q) + int(sum(int(x) >> 4 for x in c)) + 1
        out = np.zeros(cap, np.uint8)
        n = self.lib.ref_del_query(q, len(q), _p(c), len(c), _p(out), cap)
        assert n >= 0
        return out[:n].tobytes()

    def pad_query(self, qry, cigar):
        q = _bytes(qry)
        c = np.ascontiguousarray(cigar, np.uint32)
        cap = len(q) + int(sum(int(x) >> 4 for x in c)) + 1
        out = np.zeros(cap, np.uint8)
        n = self.lib.ref_pad_query(q, len(q), _p(c), len(c), _p(out), cap)
        assert n >= 0
        return out[:n].tobytes()

    def extend_align_ksw2(self, ref, qry, zdrop=200):
        r, q = _bytes(ref), _bytes(qry)
        cap = len(r) + len(q) + 4
        c = np.zeros(cap, np.uint32)
        n = self.lib.ref_extend_align_ksw2(r, len(r), q, len(q), zdrop, _p(c), cap)
        assert n >= 0
        return c[:n].copy()

    def generate_consensus(self, aligned_fasta, out_fasta, out_json, seq_limit=0, batch_size=4096):
        cap = 1 << 24
        out = np.zeros(cap, np.uint8)
        n = self.lib.ref_generate_consensus(str(aligned_fasta).encode(), str(out_fasta).encode(),
                                            str(out_json).encode(), seq_limit, batch_size, _p(out), cap)
        assert n >= 0
        return out[:n].tobytes()

    def pick_consensus(self, counts7) -> str:
        k = np.ascontiguousarray(counts7, np.uint32)
        return self.lib.ref_pick_consensus(_p(k)).decode()

    def auto_band(self, qlen, tlen):
        return self.lib.ref_auto_band(qlen, tlen)

    def chain_score(self, ai_ref, ai_qry, aj_ref, aj_qry, aj_span):
        return self.lib.ref_chain_score(ai_ref, ai_qry, aj_ref, aj_qry, aj_span)


def reference_or_none():
    try:
        return Reference()
    except (FileNotFoundError, OSError, RuntimeError):
        return None
