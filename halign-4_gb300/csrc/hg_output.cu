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
// prefix sums; insertion events are counted at the center column they
// precede.
//
// K9 accumulates consensus::SiteCount (include/consensus.h:78-99, k_base_map
// :126-145) for every center column over all rows: each thread owns four
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
                if (kind == kSegIns || kind == kSegDel) cnt = 1;
                else if (kind >= kSegDpSmall) cnt = g.nops < 0 ? 2u : (uint32_t)g.nops;
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
                    else if (s_nops[wib][lo] < 0) {  // forced I(q) D(t) (src/align/align.cpp:248-256)
                        if (rel == 0) op = 1, len = s_ql[wib][lo];
                        else op = 2, len = s_rl[wib][lo];
                    } else {
                        // the small DP tier stores its ops last-first
                        const uint32_t at = kind == kSegDpSmall ? (uint32_t)s_nops[wib][lo] - 1u - rel : rel;
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

// K8: row projection, one CTA per query (persistent).
constexpr int kRowThreads = 256;
constexpr int kRowOps = 1024;

__global__ void __launch_bounds__(kRowThreads) row_kernel(IndexDev ix, BatchDev b, int64_t row_stride)
{
    __shared__ uint32_t s_r[kRowOps + 1], s_q[kRowOps + 1];
    __shared__ uint32_t s_op[kRowOps];
    __shared__ int scan_s[33];
    __shared__ int s_qi;
    __shared__ uint32_t s_carry_r, s_carry_q;
    const int tid = threadIdx.x;
    const int L = ix.L;
    for (;;) {
        if (tid == 0) s_qi = (int)atomicAdd(&b.queues[5], 1u);
        __syncthreads();
        const int qi = s_qi;
        __syncthreads();
        if (qi >= b.n) break;
        const int q = b.order ? b.order[qi] : qi;
        const int n = b.n_cig[q];
        const uint32_t* cg = b.cig + b.coff[q];
        const uint8_t* pk = b.packed + b.poff[q];
        const int64_t e0 = b.exc_off[q], e1 = b.exc_off[q + 1];
        uint8_t* row = b.rows + (int64_t)q * row_stride;
        if (tid == 0) s_carry_r = 0, s_carry_q = 0;
        __syncthreads();
        for (int c0 = 0; c0 < n; c0 += kRowOps) {
            const int cn = min(kRowOps, n - c0);
            // prefix sums of reference / query consumption (4 ops per thread)
            uint32_t lr[4], lq[4], sr = 0, sq = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int i = tid * 4 + k;
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
            int tr, tq;
            const int er = block_excl_sum((int)sr, scan_s, &tr);
            const int eq = block_excl_sum((int)sq, scan_s, &tq);
            uint32_t ar = s_carry_r + (uint32_t)er, aq = s_carry_q + (uint32_t)eq;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int i = tid * 4 + k;
                if (i < cn) {
                    s_r[i] = ar, s_q[i] = aq;
                    const uint32_t c = s_op[i];
                    if ((c & 0xfu) == 1 && ar <= (uint32_t)L) atomicAdd(&b.ins[ar], 1u);
                }
                ar += lr[k], aq += lq[k];
            }
            if (tid == kRowThreads - 1) s_r[cn] = ar, s_q[cn] = aq;
            __syncthreads();
            const uint32_t col0 = s_r[0], col1 = s_r[cn];
            for (uint32_t col = col0 + tid; col < col1 && col < (uint32_t)L; col += kRowThreads) {
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
            __syncthreads();
            if (tid == 0) s_carry_r = s_r[cn], s_carry_q = s_q[cn];
            __syncthreads();
        }
        // a CIGAR that stops short of the center (chainless alignment cut at
        // the band edge) leaves a shorter row; pad so the buffer is defined
        const uint32_t done = s_carry_r;
        for (uint32_t col = done + tid; col < (uint32_t)L; col += kRowThreads) row[col] = '-';
        if (tid == 0 && done != (uint32_t)L) atomicOr(&b.status[q], kStLengthMismatch);
        __syncthreads();
    }
}

// K9: SiteCount over rows [r0, r1) for 4 columns per thread.
__global__ void __launch_bounds__(256) count_kernel(const uint8_t* rows, int64_t row_stride, int n_rows, int L,
                                                    int rows_per_block, uint32_t* counts)
{
    const int col = (blockIdx.x * 256 + threadIdx.x) * 4;
    if (col >= L) return;
    const int r0 = blockIdx.y * rows_per_block, r1 = min(r0 + rows_per_block, n_rows);
    uint32_t acc[4][7];
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
        for (int k = 0; k < 7; ++k) acc[c][k] = 0;
    for (int r = r0; r < r1; ++r) {
        const uint32_t wv = *reinterpret_cast<const uint32_t*>(rows + (int64_t)r * row_stride + col);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const uint32_t k = site_of((uint8_t)(wv >> (8 * c)));
#pragma unroll
            for (int z = 0; z < 7; ++z) acc[c][z] += (k == (uint32_t)z);
        }
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        if (col + c >= L) break;
#pragma unroll
        for (int k = 0; k < 7; ++k)
            if (acc[c][k]) atomicAdd(&counts[(int64_t)(col + c) * 7 + k], acc[c][k]);
    }
}

}  // namespace hg

namespace hg {
__global__ void status_or_kernel(const uint32_t* status, int n, uint32_t* flags)
{
    uint32_t v = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v |= status[i];
    v = __reduce_or_sync(0xffffffffu, v);
    if ((threadIdx.x & 31) == 0 && v) atomicOr(flags, v);
}
}  // namespace hg

extern "C" cudaError_t hg_launch_status_or(const uint32_t* status, int n, uint32_t* flags, cudaStream_t st)
{
    hg::status_or_kernel<<<4, 256, 0, st>>>(status, n, flags);
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
    hg::row_kernel<<<grid, hg::kRowThreads, 0, st>>>(*ix, *b, row_stride);
    return cudaGetLastError();
}

extern "C" cudaError_t hg_launch_count(const uint8_t* rows, int64_t row_stride, int n_rows, int L, uint32_t* counts,
                                       cudaStream_t st)
{
    if (n_rows <= 0) return cudaSuccess;
    const int rows_per_block = 512;
    dim3 grid((L + 1023) / 1024, (n_rows + rows_per_block - 1) / rows_per_block);
    hg::count_kernel<<<grid, 256, 0, st>>>(rows, row_stride, n_rows, L, rows_per_block, counts);
    return cudaGetLastError();
}
