// hg_output.cu - K7 stitch, K8 row projection, K9 per-column counters.
//
// K7 concatenates the segment CIGARs of a query in segment order (the small
// DP tier leaves its ops last-first, as its traceback produces them) with
// cigar::appendCigar semantics (src/align/cigar.cpp:302-329: zero lengths
// dropped, a run continuing the previous op merges into it, merged lengths
// above 2^28-1 are an error).  The op stream of all segments is flattened
// and merged with a warp segmented scan: op k starts a run iff its op code
// differs from op k-1; the run length is the segmented sum of lengths.
//
// K8 projects each query onto the center (cigar::delQueryToRefByCigar,
// src/align/cigar.cpp:212-299, as mergeConsensusAndSamToFasta calls it with
// keep=true): M copies the original query byte, D writes '-', I drops query
// bytes.  Rows are written column-parallel with a binary search over the op
// prefix sums, 16 columns per lane where they share one query offset and a
// lane per column where a group crosses an insertion or deletion; insertion
// events are counted at the center column they precede.
//
// K9 accumulates consensus::SiteCount (include/consensus.h:78-99, k_base_map
// :126-145) for every center column over all rows: each thread owns eight
// columns and a block of rows and adds its register totals once.
#include "hg_batch.cuh"

namespace hg {

constexpr int kStitchWarps = 4;

struct StitchState {
    uint32_t run_op;   // op of the open run (0xff = none)
    uint32_t run_len;
    int n_out;         // runs written so far (the open run is not counted)
    uint32_t ref_len, qry_len;
    bool ins, bad;
};

__global__ void __launch_bounds__(kStitchWarps * 32) stitch_kernel(IndexDev ix, BatchDev b)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    __shared__ uint32_t s_start[kStitchWarps][33];
    __shared__ uint32_t s_kind[kStitchWarps][32], s_slot[kStitchWarps][32], s_rl[kStitchWarps][32],
        s_ql[kStitchWarps][32];
    __shared__ int32_t s_nops[kStitchWarps][32];
    const uint32_t kMaxLen = (1u << 28) - 1u;
    for (;;) {
        int qi = 0;
        if (lane == 0) qi = (int)atomicAdd(&b.queues[4], 1u);
        qi = __shfl_sync(FULL, qi, 0);
        if (qi >= b.n) break;
        const int q = b.order ? b.order[qi] : qi;
        const int64_t sb = b.s_base[q];
        const int ns = b.s_n[q];
        const int64_t co = b.coff[q];
        const uint32_t* src = b.cig_seg + co;
        uint32_t* dst = b.cig + co;
        StitchState S{0xffu, 0, 0, 0, 0, false, false};
        bool global_seg = false;
        for (int s0 = 0; s0 < ns; s0 += 32) {
            const int s = s0 + lane;
            uint32_t cnt = 0;
            if (s < ns) {
                const Seg g = b.seg[sb + s];
                const uint32_t kind = g.kind & 0xffu;
                s_kind[wib][lane] = kind, s_slot[wib][lane] = g.slot, s_rl[wib][lane] = g.rl, s_ql[wib][lane] = g.ql;
                s_nops[wib][lane] = g.nops;
                if (kind == kSegIns || kind == kSegDel || kind == kSegMatch) cnt = 1;
                else if (seg_is_dp(kind)) cnt = g.nops < 0 ? 2u : (uint32_t)g.nops;
                if (kind == kSegGlobal) global_seg = true;
            }
            const uint32_t incl = warp_incl_sum(cnt);
            s_start[wib][lane] = incl - cnt;
            if (lane == 31) s_start[wib][32] = incl;
            __syncwarp();
            const uint32_t T = s_start[wib][32];
            const int nseg_chunk = min(32, ns - s0);
            for (uint32_t o0 = 0; o0 < T; o0 += 32) {
                const uint32_t o = o0 + lane;
                const bool act = o < T;
                uint32_t op = 0, len = 0;
                if (act) {
                    int lo = 0, hi = nseg_chunk - 1;  // last segment with start <= o
                    while (lo < hi) {
                        const int mid = (lo + hi + 1) >> 1;
                        if (s_start[wib][mid] <= o) lo = mid;
                        else hi = mid - 1;
                    }
                    const uint32_t rel = o - s_start[wib][lo];
                    const uint32_t kind = s_kind[wib][lo];
                    if (kind == kSegIns) op = 1, len = s_ql[wib][lo];
                    else if (kind == kSegDel) op = 2, len = s_rl[wib][lo];
                    else if (kind == kSegMatch) op = 0, len = s_rl[wib][lo];
                    else if (s_nops[wib][lo] < 0) {  // forced I(q) D(t) (src/align/align.cpp:248-256)
                        if (rel == 0) op = 1, len = s_ql[wib][lo];
                        else op = 2, len = s_rl[wib][lo];
                    } else {
                        // the small DP tier stores its ops last-first
                        const uint32_t at = (kind == kSegDpSmall || kind == kSegDpThin || kind == kSegDpSquare)
                                                  ? (uint32_t)s_nops[wib][lo] - 1u - rel
                                                  : rel;
                        const uint32_t c = src[s_slot[wib][lo] + at];
                        op = c & 0xfu, len = c >> 4;
                    }
                }
                // appendCigar drops zero lengths: they neither start nor break a run
                const bool live = act && len > 0;
                const bool open = S.run_op != 0xffu;
                const unsigned lm = __ballot_sync(FULL, live);
                const unsigned before = lm & ((1u << lane) - 1u);
                const int pl = before ? 31 - __clz(before) : 0;
                const uint32_t pop = __shfl_sync(FULL, op, pl);
                const uint32_t prev_op = before ? pop : S.run_op;
                const bool head = live && op != prev_op;
                const unsigned hm = __ballot_sync(FULL, head);
                // an open run ends when this sub-chunk's first live op starts a new run
                if (open && lm && ((hm >> (__ffs(lm) - 1)) & 1u)) {
                    if (lane == 0) dst[S.n_out] = (S.run_len << 4) | S.run_op;
                    if (S.run_len > kMaxLen) S.bad = true;
                }
                const unsigned upto = hm & ((2u << lane) - 1u);
                const int myhead = upto ? 31 - __clz(upto) : -1;
                uint32_t seg = live ? len : 0u;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const uint32_t nv = __shfl_up_sync(FULL, seg, d);
                    if (lane >= d && lane - d >= myhead) seg += nv;
                }
                if (myhead < 0) seg += S.run_len;  // still inside the open run
                const int m = __popc(upto);
                const int id = myhead < 0 ? S.n_out : S.n_out + (open ? 1 : 0) + m - 1;
                const unsigned after = lm & ~((2u << lane) - 1u);
                const bool next_head = after && ((hm >> (__ffs(after) - 1)) & 1u);
                if (live && next_head) dst[id] = (seg << 4) | op;
                if (__any_sync(FULL, live && next_head && seg > kMaxLen)) S.bad = true;
                if (lm) {
                    const int last = 31 - __clz(lm);
                    const int nh = __popc(hm);
                    S.run_len = __shfl_sync(FULL, seg, last);
                    S.run_op = __shfl_sync(FULL, op, last);
                    S.n_out += open ? nh : (nh > 0 ? nh - 1 : 0);
                }
                uint32_t rl = 0, ql = 0;
                if (live) {
                    if (op == 0 || op == 2 || op == 3 || op == 7 || op == 8) rl = len;
                    if (op == 0 || op == 1 || op == 4 || op == 7 || op == 8) ql = len;
                }
                S.ref_len += __reduce_add_sync(FULL, rl);
                S.qry_len += __reduce_add_sync(FULL, ql);
                if (__any_sync(FULL, live && op == 1)) S.ins = true;
            }
            __syncwarp();
        }
        global_seg = __any_sync(FULL, global_seg);
        if (S.run_op != 0xffu) {
            if (lane == 0) dst[S.n_out] = (S.run_len << 4) | S.run_op;
            if (S.run_len > kMaxLen) S.bad = true;
            S.n_out++;
        }
        if (lane == 0) {
            b.n_cig[q] = S.n_out;
            b.has_ins[q] = S.ins ? 1 : 0;
            uint32_t st = 0;
            if (S.bad) st |= kStCigarOverflow;
            // segments tile both sequences, so only a chainless alignment cut at
            // the band edge can leave them uncovered
            if (!global_seg && (S.ref_len != (uint32_t)ix.L || S.qry_len != (uint32_t)b.qlen[q]))
                st |= kStLengthMismatch;
            if (st) atomicOr(&b.status[q], st);
        }
    }
}

// K8: row projection, one warp per query (persistent CTAs of kRowWarps warps).
constexpr int kRowWarps = 8;
constexpr int kRowOps = 256;  // ops per chunk (per warp)

// One warp per query (no block barriers): each chunk of up to kRowOps ops
// gets its reference / query prefix sums by warp scans into the warp's shared
// arrays; columns are then written lane-parallel, 16 at a time with one
// packed-word decode where the 16 columns sit inside one op.
__global__ void __launch_bounds__(kRowWarps * 32) row_kernel(IndexDev ix, BatchDev b, int64_t row_stride)
{
    __shared__ uint32_t s_r_all[kRowWarps][kRowOps + 1], s_q_all[kRowWarps][kRowOps + 1];
    __shared__ uint32_t s_op_all[kRowWarps][kRowOps];
    __shared__ uint32_t lut[256];  // 4 packed 2-bit codes -> their 4 ASCII bases
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    uint32_t* s_r = s_r_all[wl];
    uint32_t* s_q = s_q_all[wl];
    uint32_t* s_op = s_op_all[wl];
    const int L = ix.L;
    for (int i = threadIdx.x; i < 256; i += kRowWarps * 32) {
        uint32_t v = 0;
        for (int k = 0; k < 4; ++k) v |= ((0x54474341u >> (8u * ((i >> (2 * k)) & 3))) & 0xffu) << (8 * k);
        lut[i] = v;
    }
    __syncthreads();
    for (;;) {
        int qi = 0;
        if (lane == 0) qi = (int)atomicAdd(&b.queues[5], 1u);
        qi = __shfl_sync(FULL, qi, 0);
        if (qi >= b.n) break;
        const int q = b.order ? b.order[qi] : qi;
        const int n = b.n_cig[q];
        const uint32_t* cg = b.cig + b.coff[q];
        const uint8_t* pk = b.packed + b.poff[q];
        const int64_t e0 = b.exc_off[q], e1 = b.exc_off[q + 1];
        uint8_t* row = b.rows + (int64_t)q * row_stride;
        uint32_t carry_r = 0, carry_q = 0;
        for (int c0 = 0; c0 < n; c0 += kRowOps) {
            const int cn = min(kRowOps, n - c0);
            // prefix sums of reference / query consumption: lane l takes ops 8l .. 8l+7
            constexpr int PER = kRowOps / 32;
            uint32_t lr[PER], lq[PER], sr = 0, sq = 0;
#pragma unroll
            for (int k = 0; k < PER; ++k) {
                const int i = lane * PER + k;
                uint32_t rr = 0, qq = 0;
                if (i < cn) {
                    const uint32_t c = cg[c0 + i];
                    const uint32_t op = c & 0xfu, len = c >> 4;
                    s_op[i] = c;
                    if (op == 0 || op == 2 || op == 3 || op == 7 || op == 8) rr = len;
                    if (op == 0 || op == 1 || op == 4 || op == 7 || op == 8) qq = len;
                }
                lr[k] = rr, lq[k] = qq, sr += rr, sq += qq;
            }
            const uint32_t ir = warp_incl_sum(sr), iq = warp_incl_sum(sq);
            uint32_t ar = carry_r + ir - sr, aq = carry_q + iq - sq;
#pragma unroll
            for (int k = 0; k < PER; ++k) {
                const int i = lane * PER + k;
                if (i < cn) {
                    s_r[i] = ar, s_q[i] = aq;
                    if ((s_op[i] & 0xfu) == 1 && ar <= (uint32_t)L) atomicAdd(&b.ins[ar], 1u);
                }
                ar += lr[k], aq += lq[k];
            }
            const uint32_t tot_r = __shfl_sync(FULL, ir, 31), tot_q = __shfl_sync(FULL, iq, 31);
            if (lane == 0) s_r[cn] = carry_r + tot_r, s_q[cn] = carry_q + tot_q;
            __syncwarp();
            const uint32_t col0 = s_r[0], col1 = max(col0, min(s_r[cn], (uint32_t)L));
            // exception-free query: 16 whole columns per lane, one 16-byte store
            uint32_t vb = col0, ve = col0;  // [vb, ve): columns written by the vector path
            if (e0 == e1) {
                vb = min((col0 + 15u) & ~15u, col1);
                ve = col1 & ~15u;
                if (ve < vb) ve = vb;
                for (uint32_t gb = vb; gb < ve; gb += 16u * 32u) {  // warp-uniform passes
                    const uint32_t g0 = gb + 16u * lane;
                    bool mixed = false;
                    int lo = 0;
                    if (g0 < ve) {
                        int hi = cn - 1;  // last op with s_r <= g0
                        while (lo < hi) {
                            const int mid = (lo + hi + 1) >> 1;
                            if (s_r[mid] <= g0) lo = mid;
                            else hi = mid - 1;
                        }
                        // 16 columns over copy ops only (M, =, X: one query offset, so 16
                        // consecutive query bases in one packed word) or over no copy op (16 gaps)
                        bool allcopy = true, nocopy = true;
                        for (int h = lo;; ++h) {
                            const uint32_t op = s_op[h] & 0xfu;
                            const bool cp = op == 0 || op == 7 || op == 8;
                            allcopy &= cp, nocopy &= !cp;
                            if (h >= cn - 1 || s_r[h + 1] >= g0 + 16u) break;
                        }
                        if (allcopy) {
                            const uint64_t base = (uint64_t)b.poff[q] * 4u + s_q[lo] + (g0 - s_r[lo]);
                            const uint32_t* W = reinterpret_cast<const uint32_t*>(b.packed) + (base >> 4);
                            const uint32_t sh = 2u * (uint32_t)(base & 15u);
                            const uint32_t w0 = W[0], w1 = W[1];
                            const uint32_t codes = sh ? (w0 >> sh) | (w1 << (32u - sh)) : w0;
                            *reinterpret_cast<uint4*>(row + g0) = make_uint4(
                                lut[codes & 0xffu], lut[(codes >> 8) & 0xffu], lut[(codes >> 16) & 0xffu], lut[codes >> 24]);
                        } else if (nocopy) {
                            *reinterpret_cast<uint4*>(row + g0) =
                                make_uint4(0x2d2d2d2du, 0x2d2d2d2du, 0x2d2d2d2du, 0x2d2d2d2du);
                        } else {
                            mixed = true;
                        }
                    }
                    // groups that cross an insertion, a deletion or a clip: two at a
                    // time, a half-warp per group and a lane per column
                    unsigned mm = __ballot_sync(FULL, mixed);
                    while (mm) {
                        const int l0 = __ffs(mm) - 1;
                        mm &= mm - 1u;
                        int l1 = -1;
                        if (mm) l1 = __ffs(mm) - 1, mm &= mm - 1u;
                        const int src = lane < 16 ? l0 : l1;
                        const uint32_t gg = __shfl_sync(FULL, g0, src < 0 ? l0 : src);
                        int glo = __shfl_sync(FULL, lo, src < 0 ? l0 : src);
                        if (src >= 0) {
                            const uint32_t col = gg + (uint32_t)(lane & 15);
                            while (glo < cn - 1 && s_r[glo + 1] <= col) ++glo;
                            const uint32_t op = s_op[glo] & 0xfu;
                            uint8_t ch = '-';
                            if (op == 0 || op == 7 || op == 8) ch = "ACGT"[packed_code(pk, s_q[glo] + (col - s_r[glo]))];
                            row[col] = ch;
                        }
                    }
                }
            }
            // the columns the vector path left: [col0, vb) and [ve, col1)
            const uint32_t head = vb - col0, nrest = head + (col1 - ve);
            for (uint32_t t = lane; t < nrest; t += 32) {
                const uint32_t col = t < head ? col0 + t : ve + (t - head);
                int lo = 0, hi = cn - 1;  // last op with s_r <= col and nonzero ref length
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (s_r[mid] <= col) lo = mid;
                    else hi = mid - 1;
                }
                while (lo < cn - 1 && s_r[lo + 1] <= col) ++lo;
                const uint32_t c = s_op[lo];
                const uint32_t op = c & 0xfu;
                uint8_t ch = '-';
                if (op == 0 || op == 7 || op == 8) {
                    const uint32_t qp = s_q[lo] + (col - s_r[lo]);
                    ch = "ACGT"[packed_code(pk, qp)];
                    if (e0 < e1) {
                        int64_t a = e0, z = e1;
                        while (a < z) {
                            const int64_t mid = (a + z) >> 1;
                            if ((uint32_t)b.exc[mid * 3] <= qp) a = mid + 1;
                            else z = mid;
                        }
                        if (a > e0) {
                            const int64_t r = a - 1;
                            if (qp < (uint32_t)(b.exc[r * 3] + b.exc[r * 3 + 1])) ch = (uint8_t)b.exc[r * 3 + 2];
                        }
                    }
                }
                row[col] = ch;
            }
            carry_r += tot_r, carry_q += tot_q;
            __syncwarp();
        }
        // a CIGAR that stops short of the center (chainless alignment cut at
        // the band edge) leaves a shorter row; pad so the buffer is defined
        const uint32_t done = carry_r;
        for (uint32_t col = done + lane; col < (uint32_t)L; col += 32) row[col] = '-';
        if (lane == 0 && done != (uint32_t)L) atomicOr(&b.status[q], kStLengthMismatch);
    }
}

// K9: SiteCount over rows [r0, r1) for 8 columns per thread.  Per 4-byte
// word and class, an exact zero-byte test marks the bytes of that class
// (letters case-folded: 'a' | 0x20 == 'A' | 0x20, and only those two bytes
// fold to it; '-' and '.' unfolded); the marks add into byte-lane counters
// flushed to 32-bit totals every 255 rows.  N (every other byte) is the
// row count minus the other classes.
__device__ __forceinline__ uint32_t zero_bytes(uint32_t x)  // 0x01 in each zero byte of x
{
    const uint32_t t = (x & 0x7F7F7F7Fu) + 0x7F7F7F7Fu;
    return (~(t | x | 0x7F7F7F7Fu)) >> 7;
}

constexpr int kCountCols = 8;

__global__ void __launch_bounds__(256) count_kernel(const uint8_t* rows, int64_t row_stride, int n_rows, int L,
                                                    int rows_per_block, uint32_t* counts)
{
    const int col = (blockIdx.x * 256 + threadIdx.x) * kCountCols;
    if (col >= L) return;
    const int r0 = blockIdx.y * rows_per_block, r1 = min(r0 + rows_per_block, n_rows);
    uint32_t tot[kCountCols][6];
#pragma unroll
    for (int c = 0; c < kCountCols; ++c)
#pragma unroll
        for (int k = 0; k < 6; ++k) tot[c][k] = 0;
    const uint32_t kA = 0x61616161u, kC = 0x63636363u, kG = 0x67676767u, kT = 0x74747474u, kU = 0x75757575u;
    for (int rb = r0; rb < r1; rb += 255) {
        const int re = min(rb + 255, r1);
        uint32_t acc[2][6];
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
            for (int k = 0; k < 6; ++k) acc[h][k] = 0;
#pragma unroll 4
        for (int r = rb; r < re; ++r) {
            const uint2 v = *reinterpret_cast<const uint2*>(rows + (int64_t)r * row_stride + col);
            const uint32_t wv[2] = {v.x, v.y};
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const uint32_t w = wv[h], f = w | 0x20202020u;
                acc[h][0] += zero_bytes(f ^ kA);
                acc[h][1] += zero_bytes(f ^ kC);
                acc[h][2] += zero_bytes(f ^ kG);
                acc[h][3] += zero_bytes(f ^ kT);
                acc[h][4] += zero_bytes(f ^ kU);
                acc[h][5] += zero_bytes(w ^ 0x2D2D2D2Du) + zero_bytes(w ^ 0x2E2E2E2Eu);
            }
        }
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
            for (int k = 0; k < 6; ++k)
#pragma unroll
                for (int bq = 0; bq < 4; ++bq) tot[h * 4 + bq][k] += (acc[h][k] >> (8 * bq)) & 0xffu;
    }
    const uint32_t nr = (uint32_t)(r1 - r0);
#pragma unroll
    for (int c = 0; c < kCountCols; ++c) {
        if (col + c >= L) break;
        uint32_t* cc = counts + (int64_t)(col + c) * 7;
        const uint32_t other = nr - tot[c][0] - tot[c][1] - tot[c][2] - tot[c][3] - tot[c][4] - tot[c][5];
        if (tot[c][0]) atomicAdd(cc + 0, tot[c][0]);
        if (tot[c][1]) atomicAdd(cc + 1, tot[c][1]);
        if (tot[c][2]) atomicAdd(cc + 2, tot[c][2]);
        if (tot[c][3]) atomicAdd(cc + 3, tot[c][3]);
        if (tot[c][4]) atomicAdd(cc + 4, tot[c][4]);
        if (other) atomicAdd(cc + 5, other);
        if (tot[c][5]) atomicAdd(cc + 6, tot[c][5]);
    }
}

}  // namespace hg

namespace hg {
// End of a sub-batch: OR of the per-query status words, and the work totals
// (anchors, segment records, DP segments) added to the context's counters.
__global__ void status_or_kernel(const uint32_t* status, int n, uint32_t* flags, const unsigned long long* ctl,
                                 const int32_t* s_n, unsigned long long* work)
{
    uint32_t v = 0;
    unsigned long long recs = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        v |= status[i];
        recs += (unsigned long long)max(s_n[i], 0);
    }
    v = __reduce_or_sync(0xffffffffu, v);
    for (int o = 16; o > 0; o >>= 1) recs += __shfl_xor_sync(0xffffffffu, recs, o);
    if ((threadIdx.x & 31) == 0 && v) atomicOr(flags, v);
    if ((threadIdx.x & 31) == 0 && recs) atomicAdd(&work[1], recs);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const uint32_t* c32 = reinterpret_cast<const uint32_t*>(ctl);
        atomicAdd(&work[0], ctl[4]);  // anchor cursor
        // small records, large, wavefront, CTA wavefront, thin, square list lengths
        atomicAdd(&work[2], (unsigned long long)c32[27] + c32[16] + c32[20] + c32[22] + c32[28] + c32[30]);
    }
}
}  // namespace hg

extern "C" cudaError_t hg_launch_status_or(const uint32_t* status, int n, uint32_t* flags,
                                           const unsigned long long* ctl, const int32_t* s_n, unsigned long long* work,
                                           cudaStream_t st)
{
    hg::status_or_kernel<<<4, 256, 0, st>>>(status, n, flags, ctl, s_n, work);
    return cudaGetLastError();
}

extern "C" cudaError_t hg_launch_stitch(const hg::IndexDev* ix, const hg::BatchDev* b, int grid, cudaStream_t st)
{
    hg::stitch_kernel<<<grid, hg::kStitchWarps * 32, 0, st>>>(*ix, *b);
    return cudaGetLastError();
}

extern "C" cudaError_t hg_launch_rows(const hg::IndexDev* ix, const hg::BatchDev* b, int64_t row_stride, int grid,
                                      cudaStream_t st)
{
    hg::row_kernel<<<grid, hg::kRowWarps * 32, 0, st>>>(*ix, *b, row_stride);
    return cudaGetLastError();
}

extern "C" cudaError_t hg_launch_count(const uint8_t* rows, int64_t row_stride, int n_rows, int L, uint32_t* counts,
                                       cudaStream_t st)
{
    if (n_rows <= 0) return cudaSuccess;
    const int rows_per_block = 512;
    dim3 grid((L + 256 * hg::kCountCols - 1) / (256 * hg::kCountCols), (n_rows + rows_per_block - 1) / rows_per_block);
    hg::count_kernel<<<grid, 256, 0, st>>>(rows, row_stride, n_rows, L, rows_per_block, counts);
    return cudaGetLastError();
}
