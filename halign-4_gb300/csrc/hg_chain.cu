// hg_chain.cu - K3: anchor chaining DP + segmentation of the gap-fill.
//
// Chaining restates anchor::chainAnchors (src/seed/anchor.cpp:332-461) with
// chainScoreSimple (:254-301).  One warp owns one query.  For anchor i the
// reference scans j = i-1 down to iter_start and, in order, keeps the first
// strictly better total (max_f), decrements n_skip on every improvement and
// increments it when j was marked (t[j] == i, i.e. some scanned j' > j with a
// valid score has p[j'] == j), stopping once n_skip exceeds max_skip.  The
// warp scores 32 candidates at once and reproduces that serial order exactly:
//   * marks: every valid lane stores t[p[j]] = i before any lane tests t[j];
//     p[j'] < j' means a mark only ever targets a later-scanned j, and marks
//     from lanes past the stopping point target anchors this i never tests;
//   * improvements: lane l improves iff its total beats the running maximum
//     of max_f and all earlier valid totals (warp prefix max);
//   * n_skip: X_l = max(X_{l-1} + d_l, 0) with d = -1 (improvement), +1
//     (marked, not an improvement), 0 otherwise, has the closed form
//     X_l = S_l + max(X_in, -min_{m<=l} S_m) over the prefix sums S (warp
//     prefix sum + prefix min); the first +1 lane with X > max_skip stops it.
// The penalty 0.01*dd + 0.01*dg + 0.5*log2f(dd+1) is evaluated with
// round-to-nearest products and sums (no fused multiply-add), log2f from a
// host-built table, and truncated toward zero.
//
// Segmentation restates globalAlignMM2's segment walk (src/align/align.cpp:
// 189-305): the chain comes out of the backtrack strictly increasing in both
// coordinates, i.e. already sorted by (pos_qry, pos_ref).  Segment ends are
// clipped to the sequence ends and every segment starts where the previous one
// ended, so segment s covers [max_{m<s} end_m, max(end_s, start_s)) - a warp
// prefix max.  Whether a segment's DP consumes it never moves a later
// boundary, so all segments of all queries are independent work items.
#include "hg_batch.cuh"

namespace hg {

constexpr int kChainWarps = 4;

// chainScoreSimple; lg2 = log2f table (shared memory copy of ix.log2tab).
__device__ __forceinline__ int32_t chain_score(const IndexDev& ix, const float* lg2, uint32_t ri, uint32_t qi,
                                               uint32_t rj, uint32_t qj, int32_t span_j)
{
    const int32_t dq = (int32_t)qi - (int32_t)qj;
    const int32_t dr = (int32_t)ri - (int32_t)rj;
    const int32_t dd = dr > dq ? dr - dq : dq - dr;
    const bool ok = dq > 0 && dq <= ix.max_dist_x && dr > 0 && dr <= ix.max_dist_y && dd <= ix.bw;
    const int32_t dg = dr < dq ? dr : dq;
    int32_t sc = span_j < dg ? span_j : dg;
    // the reference subtracts when dd > 0 || dg > span_j; with dd == 0 the
    // penalty is 0 up to dg_nopen (>= span_j), so those lanes skip the float path
    if (ok && (dd > 0 || dg > ix.dg_nopen)) {
        const float lin = __fadd_rn(__fmul_rn(ix.gap_pen, (float)dd), __fmul_rn(ix.skip_pen, (float)dg));
        const float lg = dd >= 1 ? lg2[dd + 1] : 0.0f;
        sc -= __float2int_rz(__fadd_rn(lin, __fmul_rn(0.5f, lg)));
    }
    return ok ? sc : INT32_MIN;
}

constexpr int kLog2Max = 512;  // dd <= bw (500), index dd + 1

__global__ void __launch_bounds__(kChainWarps * 32, 8) chain_kernel(IndexDev ix, BatchDev b)
{
    __shared__ float lg2s[kLog2Max + 1];
    for (int k = threadIdx.x; k <= kLog2Max; k += blockDim.x) lg2s[k] = k < ix.n_log2 ? ix.log2tab[k] : 0.0f;
    __syncthreads();
    // a band wider than the shared copy (bw > kLog2Max - 1) reads the table in global memory
    const float* lg2 = ix.n_log2 <= kLog2Max + 1 ? lg2s : ix.log2tab;
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int32_t span = ix.k;
    // small-list entries come from a block this warp reserved (kSmallBlock at a
    // time: far fewer contended atomics); unused entries of a block are holes
    // (key kNoShape) that the sort skips
    uint32_t sm_base = 0, sm_left = 0;
    auto small_holes = [&]() {
        for (uint32_t k = (uint32_t)lane; k < sm_left; k += 32)
            if ((int64_t)(sm_base + k) < b.wcap) b.work_key[sm_base + k] = kNoShape;
    };
    for (;;) {
        int qi = 0;
        if (lane == 0) qi = (int)atomicAdd(&b.queues[2], 1u);
        qi = __shfl_sync(FULL, qi, 0);
        if (qi >= b.n) break;
        const int q = b.order ? b.order[qi] : qi;
        const int A = b.a_n[q];
        const int64_t base = b.a_base[q];
        const uint32_t* ar = b.a_ref + base;
        const uint32_t* aq = b.a_qry + base;
        int32_t* f = b.a_f + base;
        int32_t* p = b.a_p + base;
        int32_t* t = b.a_t + base;
        // ---- speculation: every anchor's predecessor is the previous anchor.
        // Then f is a (max, +) scan, f_i = max(span, f_{i-1} + s_i) with
        // s_i = score(i-1 -> i) (-inf when i-1 is not a candidate of i), and
        // p_i = i-1 exactly when f_{i-1} + s_i > span.  Anchors go in chunks
        // of 32 (lane l takes anchor 32c + l, so loads are coalesced): a warp
        // scan composes the steps x -> max(span, x + s) and applies them to the
        // last f of the previous chunk.
        // The pairs run in 32-bit values below 2^28 query bases (f <= query
        // length + span, so -2^29 stays below every f), in 64-bit above.
        auto speculate = [&](auto zero) {
            using T = decltype(zero);
            constexpr T kNeg = sizeof(T) == 4 ? (T)-(1 << 29) : (T) - ((int64_t)1 << 40);
            T carry = kNeg;
            uint32_t pr = 0, pqv = 0;  // positions of anchor c0 - 1 (the previous chunk's last)
            uint32_t nar = lane < A ? ar[lane] : 0u, naq = lane < A ? aq[lane] : 0u;  // chunk 0
            for (int c0 = 0; c0 < A; c0 += 32) {
                const int i = c0 + lane;
                const uint32_t ri = nar, qv = naq;
                nar = i + 32 < A ? ar[i + 32] : 0u;  // next chunk, loaded ahead
                naq = i + 32 < A ? aq[i + 32] : 0u;
                uint32_t rj = __shfl_up_sync(FULL, ri, 1), qj = __shfl_up_sync(FULL, qv, 1);
                if (lane == 0) rj = pr, qj = pqv;
                pr = __shfl_sync(FULL, ri, 31), pqv = __shfl_sync(FULL, qv, 31);
                T sv = kNeg;
                if (i > 0 && i < A) {
                    if ((int32_t)(ri - rj) <= ix.max_dist_x) {  // i-1 inside the window of i
                        const int32_t sc = chain_score(ix, lg2, ri, qv, rj, qj, span);
                        if (sc != INT32_MIN) sv = (T)sc;
                    }
                }
                T fa = i < A ? (T)span : kNeg, fb = i < A ? sv : (T)0;  // lanes past the end: identity
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {  // inclusive scan: compose left steps first
                    const T la = __shfl_up_sync(FULL, fa, o), lb = __shfl_up_sync(FULL, fb, o);
                    if (lane >= o) fa = max(fa, (T)(la + fb)), fb = max((T)(lb + fb), (T)(2 * kNeg));
                }
                const T fi = max(fa, (T)(carry + fb));
                // p_i = i-1 exactly when f_{i-1} + s_i > span, i.e. when f_i > span:
                // p is not stored, spec_p() derives it from f
                if (i < A) f[i] = (int32_t)fi;
                carry = __shfl_sync(FULL, fi, 31);
            }
        };
        if (b.qlen[q] < (1 << 28)) speculate((int32_t)0);
        else speculate((int64_t)0);
        __syncwarp();
        // the speculated predecessor of anchor j (f_j > span: j-1, else none)
        auto spec_p = [&](int j, int32_t fj) -> int32_t { return fj > span ? j - 1 : -1; };
        // ---- verification.  With the speculated f, anchor i's reference scan
        // keeps (f_i, p_i) unless some candidate j <= i-2 totals more than f_i
        // (ties do not improve; where the scan stops then does not matter).
        // A total is at most f_j + min(span, dg) (the gap penalty is >= 0), so
        // the candidates i-kNear1 .. i-2 are bounded one by one (scored exactly
        // only when the bound fails) and all older ones at once through the
        // prefix maximum of f; where that prefix bound fails, i-kNear ..
        // i-kNear1-1 are bounded one by one and the older ones through the
        // prefix maximum up to i-kNear-1.  An anchor the bounds do not clear
        // runs the reference's scan (lane l takes anchor ib + l; the first
        // anchor whose result differs ends it).
        constexpr int kNear1 = 4, kNear = 8;
        int bad = A;
        int32_t mcarry = INT32_MIN;  // max f over anchors 0 .. ib - kNear1 - 2
        int32_t pm1 = INT32_MIN;     // the previous chunk's mf1 (lane l: anchor ib - 32 + l)
        for (int ib = 0; ib < A && bad == A; ib += 32) {
            const int i = ib + lane;
            // mf1: max f over 0 .. i - kNear1 - 1; mf2: over 0 .. i - kNear - 1 (mf1 of anchor i - 4)
            const int jf = i - kNear1 - 1;
            int32_t mf1 = (jf >= 0 && jf < A) ? f[jf] : INT32_MIN;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int32_t v = __shfl_up_sync(FULL, mf1, o);
                if (lane >= o) mf1 = max(mf1, v);
            }
            mf1 = max(mf1, mcarry);
            mcarry = __shfl_sync(FULL, mf1, 31);
            const int32_t up4 = __shfl_up_sync(FULL, mf1, kNear - kNear1);
            const int32_t prev4 = __shfl_sync(FULL, pm1, (lane + 32 - (kNear - kNear1)) & 31);
            const int32_t mf2 = lane >= kNear - kNear1 ? up4 : prev4;
            pm1 = mf1;
            int mine = A;
            if (i > 0 && i < A) {
                const uint32_t ri = ar[i], qv = aq[i];
                const int32_t fi = f[i];
                // one near candidate: cleared by its bound or by its exact score
                auto near_ok = [&](uint32_t rc, uint32_t qc, int32_t fc) -> bool {
                    const int32_t dg = min((int32_t)(qv - qc), (int32_t)(ri - rc));
                    if ((int64_t)fc + min(span, dg) <= (int64_t)fi) return true;
                    const int32_t sc = chain_score(ix, lg2, ri, qv, rc, qc, span);
                    return sc == INT32_MIN || (int64_t)fc + sc <= (int64_t)fi;
                };
                // candidates i-2 .. i-kNear1 one by one (fields loaded before any is tested)
                uint32_t nr[kNear1 - 1], nq[kNear1 - 1];
                int32_t nf[kNear1 - 1];
#pragma unroll
                for (int d = 2; d <= kNear1; ++d) {
                    const int j = max(i - d, 0);
                    nr[d - 2] = ar[j], nq[d - 2] = aq[j], nf[d - 2] = f[j];
                }
                bool near = true;
#pragma unroll
                for (int d = 2; d <= kNear1; ++d)
                    if (i - d >= 0 && !near_ok(nr[d - 2], nq[d - 2], nf[d - 2])) near = false;
                // older candidates at once through mf1; where that bound fails,
                // i-kNear1-1 .. i-kNear one by one and the older ones through mf2
                bool ok = near && (mf1 == INT32_MIN || (int64_t)mf1 + span <= (int64_t)fi);
                if (near && !ok) {
                    ok = mf2 == INT32_MIN || (int64_t)mf2 + span <= (int64_t)fi;
                    uint32_t mr[kNear - kNear1], mq[kNear - kNear1];
                    int32_t mfv[kNear - kNear1];
#pragma unroll
                    for (int d = kNear1 + 1; d <= kNear; ++d) {
                        const int j = max(i - d, 0);
                        mr[d - kNear1 - 1] = ar[j], mq[d - kNear1 - 1] = aq[j], mfv[d - kNear1 - 1] = f[j];
                    }
#pragma unroll
                    for (int d = kNear1 + 1; d <= kNear; ++d)
                        if (i - d >= 0 && !near_ok(mr[d - kNear1 - 1], mq[d - kNear1 - 1], mfv[d - kNear1 - 1]))
                            ok = false;
                }
                if (!ok) {
                    const int jmin = max(0, i - ix.max_iter);
                    int32_t max_f = span;
                    int max_j = -1, n_skip = 0;
                    bool mark_next = false;
                    // candidate j's fields, the next candidate's loaded one step ahead
                    uint32_t rj = ar[i - 1], qj = aq[i - 1];
                    int32_t fj = f[i - 1], pj = spec_p(i - 1, fj);
                    for (int j = i - 1; j >= jmin; --j) {
                        const int jn = j > 0 ? j - 1 : 0;
                        const uint32_t rn = ar[jn], qn = aq[jn];
                        const int32_t fn = f[jn], pn = spec_p(jn, fn);
                        const uint32_t rc = rj, qc = qj;
                        const int32_t fc = fj, pc = pj;
                        rj = rn, qj = qn, fj = fn, pj = pn;
                        if ((int32_t)(ri - rc) > ix.max_dist_x) break;  // before the window start
                        const bool marked = mark_next;
                        mark_next = false;
                        const int32_t sc = chain_score(ix, lg2, ri, qv, rc, qc, span);
                        if (sc == INT32_MIN) continue;
                        const int32_t tot = fc + sc;
                        if (tot > max_f) {
                            max_f = tot, max_j = j;
                            if (n_skip > 0) --n_skip;
                        } else if (marked) {
                            if (++n_skip > ix.max_skip) break;
                        }
                        mark_next = pc == j - 1;
                    }
                    if (max_f != fi || max_j != spec_p(i, fi)) mine = i;
                }
            }
            bad = __reduce_min_sync(FULL, mine);
        }
        int st = 0, best = -1;
        int32_t best_f = 0;
        // ---- fallback from the first anchor the speculation got wrong: the
        // serial warp scan (register window of the 32 previous anchors)
        const int k0 = bad;
        if (k0 < A) {
            for (int i = lane; i < A; i += 32) t[i] = -1;
            __syncwarp();
        }
        // register windows: lane l holds candidate j = i-1-l (position pair,
        // f, p) and the positions of anchor i0 + l of the current 32-anchor block
        uint32_t w_ar = 0, w_aq = 0, nx_ar = 0, nx_aq = 0;
        int32_t w_f = 0, w_p = -1;
        if (k0 < A) {
            const int j = k0 - 1 - lane;
            if (j >= 0) w_ar = ar[j], w_aq = aq[j], w_f = f[j], w_p = spec_p(j, w_f);
            const int nb = k0 & ~31;
            nx_ar = nb + lane < A ? ar[nb + lane] : 0u;
            nx_aq = nb + lane < A ? aq[nb + lane] : 0u;
        }
        for (int i = k0; i < A; ++i) {
            if ((i & 31) == 0) {
                nx_ar = i + lane < A ? ar[i + lane] : 0u;
                nx_aq = i + lane < A ? aq[i + lane] : 0u;
            }
            const uint32_t ri = __shfl_sync(FULL, nx_ar, i & 31), qv = __shfl_sync(FULL, nx_aq, i & 31);
            if ((i & 31) == 0 && i > 0) {
                // the window holds anchors i-1 .. i-32: write their f and p back
                f[i - 1 - lane] = w_f;
                p[i - 1 - lane] = w_p;
            }
            // the window start st is brought up to date only when the window's
            // last candidate may be out of range; a stale (smaller) st changes
            // nothing in the first chunk, and later chunks refresh it first
            const uint32_t ar31 = __shfl_sync(FULL, w_ar, 31);
            if (i <= 32 || (int32_t)(ri - ar31) > ix.max_dist_x)
                while (st < i && (int32_t)(ri - ar[st]) > ix.max_dist_x) ++st;
            int it0 = (i - st > ix.max_iter) ? i - ix.max_iter : st;
            int32_t max_f = span;
            int max_j = -1;
            int n_skip = 0;
            bool done = true;
            if (i > it0) {
                // first chunk (j = i-1 .. i-32) from the register window
                const int j = i - 1 - lane;
                const int32_t sc = j >= it0 ? chain_score(ix, lg2, ri, qv, w_ar, w_aq, span) : INT32_MIN;
                const bool valid = sc != INT32_MIN;
                const int32_t tot = w_f + sc;
                const int32_t vt = valid ? tot : INT32_MIN;
                // marks: a valid lane marks p[j], i.e. lane i-1-p[j] (always a
                // later lane); marks past this chunk go to t[] for the next one
                uint32_t bits = 0;
                if (valid && w_p >= 0) {
                    const int tl = i - 1 - w_p;
                    if (tl < 32) bits = 1u << tl;
                    else t[w_p] = i;
                }
                const uint32_t vmask = __ballot_sync(FULL, valid);
                const uint32_t mk = __reduce_or_sync(FULL, bits) & vmask;
                const int32_t M = __reduce_max_sync(FULL, vt);
                const uint32_t lead = __ballot_sync(FULL, vt == M);
                if (M <= span) {
                    // no improvement: n_skip counts the marked lanes
                    const int cnt = __popc(mk);
                    done = cnt > ix.max_skip || i - 32 <= it0;
                    n_skip = cnt;
                } else if (lead & 1u) {
                    // lane 0 holds the maximum: the only improvement; after it
                    // n_skip = max(0 - 1, 0) = 0 and counts the marked lanes
                    max_f = __shfl_sync(FULL, tot, 0);
                    max_j = i - 1;
                    const int cnt = __popc(mk & ~1u);
                    done = cnt > ix.max_skip || i - 32 <= it0;
                    n_skip = cnt;
                } else {
                    const bool marked = (mk >> lane) & 1u;
                    const int32_t vmax = warp_incl_max(vt);
                    int32_t prev = __shfl_up_sync(FULL, vmax, 1);
                    if (lane == 0) prev = INT32_MIN;
                    const bool rec = valid && tot > max(prev, max_f);
                    const int d = rec ? -1 : (marked ? 1 : 0);
                    const int S = warp_incl_sum(d);
                    const int mS = warp_incl_min(S);
                    const int X = S + max(0, -mS);
                    const unsigned brk = __ballot_sync(FULL, d == 1 && X > ix.max_skip);
                    unsigned recm = __ballot_sync(FULL, rec);
                    if (brk) recm &= (1u << (__ffs(brk) - 1)) - 1u;
                    if (recm) {
                        const int L = 31 - __clz(recm);
                        max_f = __shfl_sync(FULL, tot, L);
                        max_j = i - 1 - L;
                    }
                    done = brk != 0 || i - 32 <= it0;
                    n_skip = __shfl_sync(FULL, X, 31);
                }
            }
            // later chunks: marks through t[], warp scans
            if (!done) {
                while (st < i && (int32_t)(ri - ar[st]) > ix.max_dist_x) ++st;
                it0 = (i - st > ix.max_iter) ? i - ix.max_iter : st;
                __syncwarp();
                for (int jb = i - 33; jb >= it0; jb -= 32) {
                    const int j = jb - lane;
                    int32_t sc = INT32_MIN;
                    if (j >= it0) sc = chain_score(ix, lg2, ri, qv, ar[j], aq[j], span);
                    const bool valid = sc != INT32_MIN;
                    int32_t fj = 0, pj = -1;
                    if (valid) fj = f[j], pj = j < k0 ? spec_p(j, fj) : p[j];
                    if (valid && pj >= 0) t[pj] = i;
                    __syncwarp();
                    const bool marked = valid && t[j] == i;
                    const int32_t tot = fj + sc;
                    const int32_t vmax = warp_incl_max(valid ? tot : INT32_MIN);
                    int32_t prev = __shfl_up_sync(FULL, vmax, 1);
                    if (lane == 0) prev = INT32_MIN;
                    prev = max(prev, max_f);
                    const bool rec = valid && tot > prev;
                    const int d = rec ? -1 : (marked ? 1 : 0);
                    const int S = warp_incl_sum(d);
                    const int mS = warp_incl_min(S);
                    const int X = S + max(n_skip, -mS);
                    const unsigned brk = __ballot_sync(FULL, d == 1 && X > ix.max_skip);
                    unsigned recm = __ballot_sync(FULL, rec);
                    if (brk) recm &= (1u << (__ffs(brk) - 1)) - 1u;
                    if (recm) {
                        const int L = 31 - __clz(recm);
                        max_f = __shfl_sync(FULL, tot, L);
                        max_j = __shfl_sync(FULL, j, L);
                    }
                    if (brk) break;
                    n_skip = __shfl_sync(FULL, X, 31);
                    __syncwarp();
                }
            }
            // shift the window: lane l takes lane l-1's anchor, lane 0 anchor i
            w_ar = __shfl_up_sync(FULL, w_ar, 1);
            w_aq = __shfl_up_sync(FULL, w_aq, 1);
            w_f = __shfl_up_sync(FULL, w_f, 1);
            w_p = __shfl_up_sync(FULL, w_p, 1);
            if (lane == 0) w_ar = ri, w_aq = qv, w_f = max_f, w_p = max_j;
        }
        if (k0 < A && A - 1 - lane >= 0) f[A - 1 - lane] = w_f, p[A - 1 - lane] = w_p;  // the last window
        __syncwarp();
        // best chain end: the first anchor with the largest f (strictly greater
        // than every earlier one, starting from 0)
        {
            int32_t mf = 0;
            int mi = -1;
            for (int i = lane; i < A; i += 32) {  // first index of this lane's maximum
                const int32_t fv = f[i];
                if (fv > mf) mf = fv, mi = i;
            }
            const int32_t gmax = __reduce_max_sync(FULL, mf);
            const int cand = (gmax > 0 && mf == gmax) ? mi : INT32_MAX;
            const int gi = __reduce_min_sync(FULL, cand);
            best_f = gmax;
            best = gi == INT32_MAX ? -1 : gi;
        }
        // backtrack: chain (reversed) into t[], read p[] 32 entries at a time
        int c = 0, s0c = -1;  // s0c >= 0: the chain is the run s0c .. s0c + c - 1 (t[] unused)
        if (!(best_f < ix.min_score || best < 0) && k0 == A) {
            // speculation held: every p is i-1 or -1, so the chain is the run
            // [s, best] with s the last anchor at or before best whose p is -1,
            // i.e. whose f is span (f_0 = span, so s exists)
            int sl = -1;
            for (int i = lane; i <= best; i += 32)
                if (f[i] <= span) sl = i;
            s0c = __reduce_max_sync(FULL, sl);
            c = best - s0c + 1;
            if (c < ix.min_cnt) c = 0;
        } else if (!(best_f < ix.min_score || best < 0)) {
            int cur = best;
            while (cur >= 0) {
                const int lo = max(cur - 31, 0);
                const int ip = lo + lane;
                const int pl = ip <= cur ? (ip < k0 ? spec_p(ip, f[ip]) : p[ip]) : -1;
                while (cur >= lo) {
                    if (lane == 0) t[c] = cur;
                    ++c;
                    cur = __shfl_sync(FULL, pl, cur - lo);
                }
            }
            if (c < ix.min_cnt) c = 0;
        }
        __syncwarp();
        // segmentation
        const int len = b.qlen[q];
        const int L = ix.L;
        const int nseg = c > 0 ? 2 * c + 1 : 1;
        unsigned long long sb = 0;
        if (lane == 0) {
            sb = atomicAdd(b.s_cursor, (unsigned long long)nseg);
            if ((int64_t)(sb + nseg) > b.scap) {
                atomicOr(&b.status[q], kStArenaOverflow);
                sb = ~0ull;
            }
        }
        sb = __shfl_sync(FULL, sb, 0);
        if (lane == 0) {
            b.n_chain[q] = c;
            if (b.chain_meta) b.chain_meta[2 * q] = best, b.chain_meta[2 * q + 1] = k0;
            b.s_base[q] = sb == ~0ull ? 0 : (int64_t)sb;
            b.s_n[q] = 0;
        }
        if (sb == ~0ull) continue;
        // empty segments (both lengths 0) contribute no op: only the others
        // are stored, in order
        uint32_t rpos = 0, qpos = 0, slot = 0, nkept = 0;
        // consecutive match segments (and anchor spans, which are match
        // segments) become one record of their summed length: their ops are
        // all M and merge in the CIGAR anyway.  Segments tile the center and
        // the query and a match is diagonal, so a run (empty segments inside
        // it included) spans from its first segment's start to its last
        // segment's end.  A run still open at the end of a 32-segment chunk is
        // carried (record id, start).
        bool open = false;
        uint32_t o_sid = 0, o_rs = 0, o_qs = 0;
        unsigned long long match_cells = 0;  // this lane's part, added to the cell total once per query
        auto put_match = [&](uint32_t id, uint32_t mrs, uint32_t mqs, uint32_t mlen) {
            Seg g;
            g.rs = mrs, g.qs = mqs, g.rl = mlen, g.ql = mlen;
            g.slot = 0;
            g.nops = 0;
            g.q = (uint32_t)q;
            g.kind = kSegMatch;
            b.seg[id] = g;
        };
        // Equal-length segments whose sides are identical A/C/G/T strings (the
        // span of an exact k-mer anchor after overlap clipping) align as rl M:
        // the diagonal scores 5 rl, any other path needs an insertion and a
        // deletion (>= 16 in gap costs) and has fewer matches, so every
        // diagonal cell's direction is M and the traceback from the corner
        // follows it.  Checked on 2-bit words of the query and the center.
        const bool plain = ix.center_plain && b.exc_off[q] == b.exc_off[q + 1];
        const uint64_t qbase = (uint64_t)b.poff[q] * 4u;
        auto same_bases = [&](uint64_t qp, uint32_t rp, uint32_t n) -> bool {
            auto window = [](const uint8_t* pk, uint64_t pos) -> uint64_t {
                const uint64_t wb = (pos >> 2) & ~(uint64_t)7;
                const uint64_t* w = reinterpret_cast<const uint64_t*>(pk + wb);
                const uint32_t sh = 2u * (uint32_t)(pos - wb * 4u);
                return sh ? (w[0] >> sh) | (w[1] << (64u - sh)) : w[0];
            };
            const uint64_t m = n >= 32 ? ~0ull : ((1ull << (2 * n)) - 1ull);
            return ((window(b.packed, qp) ^ window(ix.center2, rp)) & m) == 0;
        };
        // the x-th chain anchor in increasing order
        auto chain_at = [&](int x) -> int { return s0c >= 0 ? s0c + x : t[c - 1 - x]; };
        // raw end of segment s (before clipping and the prefix max)
        auto seg_end = [&](int s, int64_t& er, int64_t& eq, uint32_t& flags) {
            er = 0, eq = 0, flags = 0;
            if (s >= nseg) return;
            if (c == 0) {
                er = L, eq = len;
            } else if (s == 0) {
                const int a = chain_at(0);
                er = ar[a], eq = aq[a], flags = kSegLeft;
            } else if (s == 2 * c) {
                er = L, eq = len;
            } else if (s & 1) {
                const int a = chain_at((s - 1) / 2);
                er = (int64_t)ar[a] + span, eq = (int64_t)aq[a] + span;
            } else {
                const int a = chain_at(s / 2);
                er = ar[a], eq = aq[a];
            }
        };
        int64_t n_er, n_eq;
        uint32_t n_flags;
        seg_end(lane, n_er, n_eq, n_flags);
        for (int s0 = 0; s0 < nseg; s0 += 32) {
            const int s = s0 + lane;
            const bool act = s < nseg;
            const int64_t er = n_er, eq = n_eq;
            const uint32_t flags = n_flags;
            seg_end(s + 32, n_er, n_eq, n_flags);  // the next chunk's ends, loaded ahead
            const int cr = act ? (int)min(er, (int64_t)L) : 0;
            const int cq = act ? (int)min(eq, (int64_t)len) : 0;
            const int ir = max(warp_incl_max(cr), (int)rpos);
            const int iq = max(warp_incl_max(cq), (int)qpos);
            int pr = __shfl_up_sync(FULL, ir, 1), pq = __shfl_up_sync(FULL, iq, 1);
            if (lane == 0) pr = rpos, pq = qpos;
            const uint32_t rs = (uint32_t)pr, qs = (uint32_t)pq;
            const uint32_t rl = (uint32_t)ir - rs, ql = (uint32_t)iq - qs;
            uint32_t kind;
            if (rl == 0 && ql == 0) kind = kSegEmpty;
            else if (rl == 0) kind = kSegIns;
            else if (ql == 0) kind = kSegDel;
            else if (c == 0) kind = kSegGlobal;
            else if (rl == ql && rl <= 32 && plain && same_bases(qbase + qs, rs, rl))
                kind = kSegMatch;  // identical equal-length sides: the DP's CIGAR is rl M
            else if (small_tier_fits(rl, ql) || medium_tier_fits(rl, ql))
                kind = kSegDpSmall;
            else if (thin_tier_fits(rl, ql) && (int32_t)ql <= b.thin_max_inner)
                kind = kSegDpThin;
            else if (square_tier_fits(rl, ql) && (int64_t)rl * ql <= (int64_t)b.square_max_cells)
                kind = kSegDpSquare;
            else
                kind = kSegDpLarge;
            // the reference runs extz2 on a match segment too (full band: rl x rl
            // cells); count them so the cell total stays the reference's work unit
            if (act && kind == kSegMatch) match_cells += (unsigned long long)rl * rl;
            const bool keep = act && kind != kSegEmpty;
            const unsigned kmask = __ballot_sync(FULL, keep);
            const bool isM = keep && kind == kSegMatch;
            const unsigned mmask = __ballot_sync(FULL, isM);
            if (kmask == mmask) {  // every kept segment is a match (or none is kept): one run, no DP
                if (mmask && !open) {
                    const int h = __ffs(mmask) - 1;
                    o_rs = __shfl_sync(FULL, rs, h), o_qs = __shfl_sync(FULL, qs, h);
                    o_sid = (uint32_t)sb + nkept;
                    ++nkept;
                    open = true;
                }
                rpos = (uint32_t)__shfl_sync(FULL, ir, 31);
                qpos = (uint32_t)__shfl_sync(FULL, iq, 31);
                continue;
            }
            const unsigned below = (1u << lane) - 1u;
            const unsigned kb = kmask & below;
            const bool prev_m = kb ? ((mmask >> (31 - __clz(kb))) & 1u) != 0 : open;
            const bool cont = isM && prev_m;  // continues the match run before it
            const bool rec = keep && !cont;   // starts a record
            const unsigned rmask = __ballot_sync(FULL, rec);
            const uint32_t sid = (uint32_t)sb + nkept + (uint32_t)__popc(rmask & below);
            // a carried run ends where this chunk's first kept segment is not a match
            if (open && kmask && !((mmask >> (__ffs(kmask) - 1)) & 1u)) {
                if (lane == 0) put_match(o_sid, o_rs, o_qs, rpos - o_rs);
                open = false;
            }
            // match runs: this lane's run head (-1: the carried run)
            const unsigned hm = __ballot_sync(FULL, isM && !cont);
            const unsigned hup = hm & ((2u << lane) - 1u);
            const int h = hup ? 31 - __clz(hup) : -1;
            const int hs = h >= 0 ? h : 0;
            const uint32_t h_sid = __shfl_sync(FULL, sid, hs), h_rs = __shfl_sync(FULL, rs, hs),
                           h_qs = __shfl_sync(FULL, qs, hs);
            const uint32_t r_sid = h >= 0 ? h_sid : o_sid, r_rs = h >= 0 ? h_rs : o_rs, r_qs = h >= 0 ? h_qs : o_qs;
            const unsigned ka = kmask & ~((2u << lane) - 1u);  // kept segments after this one
            if (isM && ka && !((mmask >> (__ffs(ka) - 1)) & 1u)) put_match(r_sid, r_rs, r_qs, (uint32_t)ir - r_rs);
            if (kmask) {  // the chunk's last kept segment decides what is carried
                const int last = 31 - __clz(kmask);
                if ((mmask >> last) & 1u) {
                    o_sid = __shfl_sync(FULL, r_sid, last);
                    o_rs = __shfl_sync(FULL, r_rs, last);
                    o_qs = __shfl_sync(FULL, r_qs, last);
                    open = true;
                } else {
                    open = false;
                }
            }
            const uint32_t need = (seg_is_dp(kind) && act) ? rl + ql : 0;
            const unsigned mdp = __ballot_sync(FULL, need != 0);
            const uint32_t sincl = mdp ? warp_incl_sum(need) : 0u;
            const uint32_t my_slot = slot + sincl - need;
            if (rec && !isM) {
                Seg g;
                g.rs = rs, g.qs = qs, g.rl = rl, g.ql = ql;
                g.slot = my_slot;
                g.nops = 0;
                g.q = (uint32_t)q;
                g.kind = kind | flags;
                b.seg[sid] = g;
            }
            nkept += (uint32_t)__popc(rmask);
            // tier work lists (warp-aggregated appends): small, thin, one-warp
            // wavefront, CTA wavefront, exact; a chunk whose DP segments all
            // go to the small tier (the common case) skips the others
            const unsigned ms = __ballot_sync(FULL, act && kind == kSegDpSmall);
            if (ms) {
                const uint32_t nms = (uint32_t)__popc(ms);
                if (nms > sm_left) {
                    small_holes();
                    uint32_t nb = 0;
                    if (lane == 0) nb = atomicAdd(b.n_small, kSmallBlock);
                    sm_base = __shfl_sync(FULL, nb, 0), sm_left = kSmallBlock;
                }
                const uint32_t bs = sm_base;
                sm_base += nms, sm_left -= nms;
                if (ms >> lane & 1u) {
                    const unsigned w = bs + __popc(ms & below);
                    if ((int64_t)w < b.wcap) {
                        b.work_small[w] = sid;
                        if (b.work_key) {
                            Seg g;
                            g.rl = rl, g.ql = ql, g.kind = kind | flags;
                            b.work_key[w] = shape_key(g);
                        }
                    } else {
                        atomicOr(&b.status[q], kStArenaOverflow);
                    }
                }
                // (the small-tier shape histogram is counted from work_key by shape_hist_kernel)
            }
            if (mdp != ms) {
                const bool dp_big = act && (kind == kSegDpLarge || kind == kSegGlobal);
                const bool wv = dp_big && wave_eligible(rl, ql);
                const bool wv_warp = wv && min(rl, ql) <= (uint32_t)kWaveWarpMaxInner;
                const unsigned ml = __ballot_sync(FULL, dp_big && !wv);
                const unsigned mw = __ballot_sync(FULL, wv_warp);
                const unsigned mx = __ballot_sync(FULL, wv && !wv_warp);
                const unsigned mt = __ballot_sync(FULL, act && kind == kSegDpThin);
                const unsigned mq = __ballot_sync(FULL, act && kind == kSegDpSquare);
                unsigned bl = 0, bw = 0, bx = 0, bt = 0, bq = 0;
                if (lane == 0) {
                    if (mq) bq = atomicAdd(b.n_sq, (unsigned)__popc(mq));
                    if (mt) bt = atomicAdd(b.n_thin, (unsigned)__popc(mt));
                    if (ml) bl = atomicAdd(b.n_large, (unsigned)__popc(ml));
                    if (mw) bw = atomicAdd(b.n_wave, (unsigned)__popc(mw));
                    if (mx) bx = atomicAdd(b.n_wide, (unsigned)__popc(mx));
                }
                bl = __shfl_sync(FULL, bl, 0);
                bw = __shfl_sync(FULL, bw, 0);
                bx = __shfl_sync(FULL, bx, 0);
                bt = __shfl_sync(FULL, bt, 0);
                bq = __shfl_sync(FULL, bq, 0);
                if (ml >> lane & 1u) {
                    const unsigned w = bl + __popc(ml & below);
                    if ((int64_t)w < b.wcap) b.work_large[w] = sid;
                    else atomicOr(&b.status[q], kStArenaOverflow);
                }
                uint32_t wkey = 0xffffffffu;
                if (mw >> lane & 1u) {
                    const unsigned w = bw + __popc(mw & below);
                    wkey = wave_key(rl, ql, (flags & kSegLeft) != 0);
                    if ((int64_t)w < b.wcap) {
                        b.work_wave[w] = sid;
                        b.work_wave_key[w] = wkey;
                    } else {
                        atomicOr(&b.status[q], kStArenaOverflow);
                    }
                }
                if (mw) {
                    const unsigned peers = __match_any_sync(FULL, wkey);
                    if ((mw >> lane & 1u) && lane == __ffs(peers) - 1) atomicAdd(&b.wave_hist[wkey], __popc(peers));
                }
                if (mx >> lane & 1u) {
                    const unsigned w = bx + __popc(mx & below);
                    if ((int64_t)w < b.wcap) b.work_wide[w] = sid;
                    else atomicOr(&b.status[q], kStArenaOverflow);
                }
                uint32_t tkey = 0xffffffffu;  // counted in the histogram only when placed
                if (mt >> lane & 1u) {
                    const unsigned w = bt + __popc(mt & below);
                    if ((int64_t)w < b.wcap) {
                        tkey = thin_key(rl, ql, (flags & kSegLeft) != 0);
                        b.work_thin[w] = sid;
                        b.work_thin_key[w] = tkey;
                    } else {
                        atomicOr(&b.status[q], kStArenaOverflow);
                    }
                }
                if (mt) {
                    const unsigned peers = __match_any_sync(FULL, tkey);
                    if (tkey != 0xffffffffu && lane == __ffs(peers) - 1) atomicAdd(&b.thin_hist[tkey], __popc(peers));
                }
                if (mq) {
                    uint32_t qkey = 0xffffffffu;  // counted in the histogram only when placed
                    if (mq >> lane & 1u) {
                        const unsigned w = bq + __popc(mq & below);
                        if ((int64_t)w < b.wcap) {
                            qkey = square_key(rl, ql, (flags & kSegLeft) != 0);
                            b.work_sq[w] = sid;
                            b.work_sq_key[w] = qkey;
                        } else {
                            atomicOr(&b.status[q], kStArenaOverflow);
                        }
                    }
                    const unsigned peers = __match_any_sync(FULL, qkey);
                    if (qkey != 0xffffffffu && lane == __ffs(peers) - 1) atomicAdd(&b.sq_hist[qkey], __popc(peers));
                }
            }
            rpos = (uint32_t)__shfl_sync(FULL, ir, 31);
            qpos = (uint32_t)__shfl_sync(FULL, iq, 31);
            slot = slot + __shfl_sync(FULL, sincl, 31);
        }
        if (open && lane == 0) put_match(o_sid, o_rs, o_qs, rpos - o_rs);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) match_cells += __shfl_xor_sync(FULL, match_cells, o);
        if (lane == 0 && match_cells && b.cells) {
            atomicAdd(b.cells, match_cells);
            atomicAdd(b.match_cells, match_cells);
        }
        if (lane == 0) b.s_n[q] = (int32_t)nkept;
    }
    small_holes();  // the rest of this warp's last block
}

}  // namespace hg

extern "C" cudaError_t hg_launch_chain(const hg::IndexDev* ix, const hg::BatchDev* b, int grid, cudaStream_t st)
{
    hg::chain_kernel<<<grid, hg::kChainWarps * 32, 0, st>>>(*ix, *b);
    return cudaGetLastError();
}
