// hg_dp.cu - K5/K6: KSW2 extz2 gap-fill (src/align/ksw2_extz2_sse.c:23-304)
// and its traceback (ksw_backtrack, include/ksw2.h:129-161).
//
// Three tiers, all bit-exact with the SSE2 build of the reference:
//
// * Small tier (one thread per segment).  When the band w is at least
//   max(qlen, tlen) it never binds (globalAlignKSW2 sets w = 200 + ... for
//   segments up to 200 bp, or -1), and every cell the reference computes
//   outside [st0, en0] is either overwritten by a boundary before it is read
//   or never read by an in-band cell.  The DP is then exactly the per-cell
//   recurrence over the in-band cells: cell (t, j) takes x, v from (t-1, j),
//   u, y from (t, j-1), with the reference's boundaries x = 0, v = q (0 at the
//   corner) on the left and u = q (0 at the corner), y = 0 on top.  The thread
//   sweeps the longer side outermost, keeps the shorter side's byte state in
//   shared memory, applies ksw_lane (the SSE2 instruction sequence) per cell
//   and stores a 4-bit direction code per cell, word-interleaved across the
//   CTA so every shared-memory access is bank-conflict free.
//
// * Wavefront tier (one warp per segment): every other segment whose band
//   never binds and whose shorter side is at most 256; the small tier's
//   recurrence as a register wavefront across the lanes (see wave_segment).
//
// * Large tier (one warp per segment; also every single-call ksw_extz2).  An
//   exact emulation of the SIMD code: the anti-diagonal band rounded to whole
//   16-lane blocks, the per-target byte arrays u, v, x, y, s living across
//   anti-diagonals (so out-of-band lanes use stale state just as the SIMD
//   code does), the exact int32 H row with its 4-way interleaved arg-max,
//   z-drop, approximate-max mode and the band-exhaustion stop.  Lanes of a
//   diagonal run 32 at a time; the byte carried from the previous 32-lane
//   chunk plays the role of the SSE shift-in register.
#include <cstdio>
#include <type_traits>
#include <mutex>

#include "../../include/halign_gb300.h"
#include "hg_batch.cuh"
#include "hg_internal.h"

namespace hg {

constexpr int kDpSmallThreads = 128;

__device__ __forceinline__ uint32_t dna5_score(uint32_t a, uint32_t b)
{  // dna5_simd_mat (include/align.h:109-116)
    return (a == 4u || b == 4u) ? 0u : (a == b ? 5u : (uint32_t)(uint8_t)-4);
}

// DNA5 code of query base i (packed + exception runs).
__device__ __forceinline__ uint32_t query_dna5(const uint8_t* pk, const int32_t* exc, int64_t e0, int64_t e1, uint32_t i)
{
    uint32_t c = packed_code(pk, i);
    if (e0 < e1) {
        int64_t lo = e0, hi = e1;
        while (lo < hi) {  // first run starting after i
            const int64_t mid = (lo + hi) >> 1;
            if ((uint32_t)exc[mid * 3] <= i) lo = mid + 1;
            else hi = mid;
        }
        if (lo > e0) {
            const int64_t r = lo - 1;
            if (i < (uint32_t)(exc[r * 3] + exc[r * 3 + 1])) c = dna5_of((uint8_t)exc[r * 3 + 2]);
        }
    }
    return c;
}


struct CigarPush {
    uint32_t* out;
    int n, cap;
    uint32_t last;
    __device__ void push(uint32_t op, uint32_t len)
    {
        if (n > cap) return;
        if (n > 0 && (last & 0xfu) == op) {
            last += len << 4;
            out[n - 1] = last;
        } else if (n < cap) {
            last = len << 4 | op;
            out[n++] = last;
        } else {
            n = cap + 1;  // overflow marker
        }
    }
};

// One in-band cell in int32 arithmetic.  For segments the band never binds,
// the difference encoding keeps every byte value the SSE2 sequence touches in
// a range where 8-bit wrapping add/sub, unsigned max/min and signed compares
// equal plain int32 arithmetic (u, v in [0, 21], x, y in [0, q], z, a, b in
// [0, 27]); tests/dp_arith_equiv.c checks the two forms cell by cell.
template <int MODE>
__device__ __forceinline__ uint32_t lane_int(int s, int xt1, int vt1, int ut, int yt, int& u, int& v, int& x, int& y)
{
    int z = s + 16;
    const int a0 = xt1 + vt1, b0 = yt + ut;
    uint32_t d;
    if (MODE == 1) {  // left-aligned gaps: ties go to H, then E
        d = a0 > z ? 1u : 0u;
        z = max(z, a0);
        if (b0 > z) d = 2u;
    } else {          // right-aligned gaps: ties go to F, then E
        d = z > a0 ? 0u : 1u;
        z = max(z, a0);
        if (!(z > b0)) d = 2u;
    }
    z = min(max(z, b0), 21);
    u = z - vt1;
    v = z - ut;
    const int zq = z - 6;
    const int a = a0 - zq, b = b0 - zq;
    if (MODE == 1) {
        x = max(a, 0), y = max(b, 0);
        d |= (a > 0 ? 4u : 0u) | (b > 0 ? 8u : 0u);   // 4-bit code: E/F continuation bits
    } else {
        x = max(a, 0), y = max(b, 0);
        d |= (a >= 0 ? 4u : 0u) | (b >= 0 ? 8u : 0u);
    }
    return d;  // bits 0-1 state, bit 2 E continuation, bit 3 F continuation
}

// lane_int with the score already offset: z0 = score + 16, and the max
// with the column-side term taken first so the row-carried term (xt1 + vt1)
// is the last input on the dependency chain.
template <int MODE>
__device__ __forceinline__ uint32_t lane_int_z(int z0, int xt1, int vt1, int ut, int yt, int& u, int& v, int& x,
                                               int& y)
{
    const int a0 = xt1 + vt1, b0 = yt + ut;
    uint32_t d;
    if (MODE == 1) {
        d = a0 > z0 ? 1u : 0u;
        if (b0 > max(z0, a0)) d = 2u;
    } else {
        d = z0 > a0 ? 0u : 1u;
        if (!(max(z0, a0) > b0)) d = 2u;
    }
    const int z = min(max(max(z0, b0), a0), 21);
    u = z - vt1;
    v = z - ut;
    const int zq = z - 6;
    const int a = a0 - zq, b = b0 - zq;
    x = max(a, 0), y = max(b, 0);
    if (MODE == 1) d |= (a > 0 ? 4u : 0u) | (b > 0 ? 8u : 0u);
    else d |= (a >= 0 ? 4u : 0u) | (b >= 0 ? 8u : 0u);
    return d;
}

// Two independent cells at once, one per 16-bit half (two segments of the
// same shape and gap mode side by side): lane_int_z's recurrence on both
// halves of 32-bit words.  Every value carries a bias of kPB per half, so
// each half stays non-negative and below 0x8000 (real values lie in
// [-32, 64]); plain 32-bit adds and subtracts then act on both halves at
// once with no carry or borrow crossing between them, and the unsigned
// 16x2 max / min order biased values as the signed ones would.  A
// comparison p > q (p >= q) is bit 15 of a half of 0x7fff + p - q
// (0x8000 + p - q).  Returns the two 4-bit direction codes at bits 0-3
// (low half) and 16-19 (high half).
constexpr uint32_t kPB = 64;
constexpr uint32_t kPB2 = kPB * 0x00010001u;

template <int MODE>
__device__ __forceinline__ uint32_t lane16x2(uint32_t z0, uint32_t xt1, uint32_t vt1, uint32_t ut, uint32_t yt,
                                             uint32_t& u, uint32_t& v, uint32_t& x, uint32_t& y)
{
    const uint32_t a0 = xt1 + vt1 - kPB2, b0 = yt + ut - kPB2;
    const uint32_t m = __vmaxu2(z0, a0);
    const uint32_t z = __vminu2(__vmaxu2(m, b0), (21u + kPB) * 0x00010001u);  // min(., 21)
    u = z + kPB2 - vt1;
    v = z + kPB2 - ut;
    const uint32_t a = a0 - z + (6u + kPB) * 0x00010001u;  // a0 - (z - q)
    const uint32_t b = b0 - z + (6u + kPB) * 0x00010001u;
    x = __vmaxu2(a, kPB2);
    y = __vmaxu2(b, kPB2);
    // MODE 1 (left-aligned): strict compares; MODE 2 (right-aligned): ties
    // go the other way, i.e. >=
    constexpr uint32_t K = MODE == 1 ? 0x7fff7fffu : 0x80008000u;
    const uint32_t fa = a0 + K - z0;   // a0 > z0
    const uint32_t fc = b0 + K - m;    // b0 > max(z0, a0)
    const uint32_t fe = a + K - kPB2;  // a > 0
    const uint32_t ff = b + K - kPB2;  // b > 0
    constexpr uint32_t H = 0x80008000u;
    return ((fc & H) >> 14) | ((fa & ~fc & H) >> 15) | ((fe & H) >> 13) | ((ff & H) >> 12);
}

// 64 bases of 2-bit codes from base `pos` of a packed stream (base i at bits
// 2(i&3) of byte i>>2): base pos+m at bits 2m of lo (m < 32) / 2(m-32) of hi.
// The stream is 8-byte aligned and readable 24 bytes past byte (pos/4 & ~7).
__device__ __forceinline__ void load_bases64(const uint8_t* pk, uint64_t pos, uint64_t& lo, uint64_t& hi)
{
    const uint64_t wb = (pos >> 2) & ~(uint64_t)7;
    const uint64_t* w = reinterpret_cast<const uint64_t*>(pk + wb);
    const uint64_t w0 = w[0], w1 = w[1], w2 = w[2];
    const uint32_t sh = 2u * (uint32_t)(pos - wb * 4u);  // 0 .. 62
    lo = sh ? (w0 >> sh) | (w1 << (64u - sh)) : w0;
    hi = sh ? (w1 >> sh) | (w2 << (64u - sh)) : w1;
}

// Segment DP for one thread.  TINNER: the target is the shorter (inner) side;
// rows run over the query.  Direction codes: row o, inner position i at word
// o*stride + i/8, nibble i%8, words interleaved across the CTA.  FAST: the
// query has no exception bytes and the center is all A/C/G/T, so both sides
// come from 2-bit packed words held in registers.  The traceback writes each
// op run once, last-first (the stitch reads small-tier segments backwards).
template <bool TINNER, int MODE, bool FAST, int IMAX, int T>
__device__ __forceinline__ void small_segment(const IndexDev& ix, const BatchDev& b, const SmallRec& r,
                                              uint32_t* dirs, int tid)
{
    // IMAX: unroll bound of the inner side (4, 8, 16 or 32 >= inner), so short
    // segments do not pay for wider guarded rows; T: threads per CTA (the
    // direction words of a row are interleaved across them)
    constexpr int NW = (IMAX + 7) / 8;  // direction words per row at most
    const int qn = (int)((r.shape >> 8) & 0xffu), tn = (int)(r.shape & 0xffu);
    const int inner = TINNER ? tn : qn, outer = TINNER ? qn : tn;
    const int stride = (inner + 7) >> 3;
    // off the fast path: query-relative positions, exception runs
    const uint32_t qs = FAST ? 0u : (uint32_t)(r.qpos - (uint64_t)b.poff[r.q] * 4u);
    const uint8_t* pk = FAST ? b.packed : b.packed + b.poff[r.q];
    const int64_t e0 = FAST ? 0 : b.exc_off[r.q], e1 = FAST ? 0 : b.exc_off[r.q + 1];
    const bool plain_q = e0 == e1;
    const uint8_t* tc = ix.center + r.rs;
    int ic[IMAX], s1[IMAX], s2[IMAX];
    uint64_t olo = 0, ohi = 0;
    if (FAST) {
        uint64_t qlo, qhi, tlo, thi;
        load_bases64(b.packed, r.qpos, qlo, qhi);
        load_bases64(ix.center2, r.rs, tlo, thi);
        const uint64_t ilo = TINNER ? tlo : qlo;
        olo = TINNER ? qlo : tlo;
        ohi = TINNER ? qhi : thi;
#pragma unroll
        for (int i = 0; i < IMAX; ++i) ic[i] = (int)((ilo >> (2 * i)) & 3u);
    } else {
#pragma unroll
        for (int i = 0; i < IMAX; ++i) {
            ic[i] = 0;
            if (i < inner) {
                if (TINNER) ic[i] = tc[i];
                else ic[i] = plain_q ? (int)packed_code(pk, qs + i) : (int)query_dna5(pk, b.exc, e0, e1, qs + i);
            }
        }
    }
#pragma unroll
    for (int i = 0; i < IMAX; ++i) s1[i] = 0, s2[i] = 0;
    for (int o = 0; o < outer; ++o) {
        int oc;
        if (FAST) {
            oc = (int)(((o < 32 ? olo : ohi) >> (2 * (o & 31))) & 3u);
        } else {
            if (TINNER) oc = plain_q ? (int)packed_code(pk, qs + o) : (int)query_dna5(pk, b.exc, e0, e1, qs + o);
            else oc = tc[o];
        }
        // TINNER: carried x, v along the row, s1/s2 = u, y of the previous row.
        // !TINNER: carried u, y along the column, s1/s2 = x, v of the previous column.
        int c1 = 0, c2 = o ? 6 : 0;
        uint32_t wd[NW];
#pragma unroll
        for (int k = 0; k < NW; ++k) wd[k] = 0;
#pragma unroll
        for (int i = 0; i < IMAX; ++i) {
            if (i < inner) {
                const int z0 = FAST ? (ic[i] == oc ? 21 : 12)
                                    : ((ic[i] == 4 || oc == 4) ? 16 : (ic[i] == oc ? 21 : 12));
                int u, v, x, y;
                uint32_t d;
                if (TINNER) {
                    const int ut = o ? s1[i] : (i ? 6 : 0), yt = o ? s2[i] : 0;
                    d = lane_int_z<MODE>(z0, c1, c2, ut, yt, u, v, x, y);
                    c1 = x, c2 = v, s1[i] = u, s2[i] = y;
                } else {
                    const int xt = o ? s1[i] : 0, vt = o ? s2[i] : (i ? 6 : 0);
                    const int ut = i ? c1 : (o ? 6 : 0), yt = i ? c2 : 0;
                    d = lane_int_z<MODE>(z0, xt, vt, ut, yt, u, v, x, y);
                    c1 = u, c2 = y, s1[i] = x, s2[i] = v;
                }
                wd[i >> 3] |= d << (4 * (i & 7));
            }
        }
#pragma unroll
        for (int k = 0; k < NW; ++k)
            if (k < stride) dirs[(o * stride + k) * T + tid] = wd[k];
    }
    // traceback from (tlen-1, qlen-1); runs written once, last-first
    uint32_t* out = b.cig_seg + r.out;
    int n = 0;
    uint32_t run_op = 0xffu, run_len = 0;
    auto push = [&](uint32_t op, uint32_t len) {
        if (op == run_op) {
            run_len += len;
        } else {
            if (run_len) out[n++] = run_len << 4 | run_op;
            run_op = op, run_len = len;
        }
    };
    int ti = tn - 1, qj = qn - 1, state = 0;
    while (ti >= 0 && qj >= 0) {
        const int o = TINNER ? qj : ti, i = TINNER ? ti : qj;
        const uint32_t nib = (dirs[(o * stride + (i >> 3)) * T + tid] >> ((i & 7) * 4)) & 0xfu;
        if (state == 0) state = nib & 3u;
        else if (!((nib >> (state + 1)) & 1u)) state = 0;
        if (state == 0) state = nib & 3u;
        if (state == 0) push(0, 1), --ti, --qj;
        else if (state == 1) push(2, 1), --ti;
        else push(1, 1), --qj;
    }
    if (ti >= 0) push(2, (uint32_t)(ti + 1));
    if (qj >= 0) push(1, (uint32_t)(qj + 1));
    if (run_len) out[n++] = run_len << 4 | run_op;
    b.seg[r.sid].nops = n;
}

// Two FAST records of identical shape in one thread, one per 16-bit half
// (lane16x2).  Direction codes: row o, inner position i at word
// o * stride + i / 4, byte i % 4, the low nibble the first record's and the
// high nibble the second's; words interleaved across the CTA as in
// small_segment.  Each record's traceback then runs as small_segment's.
template <bool TINNER, int MODE, int IMAX, int T>
__device__ __forceinline__ void small_pair(const IndexDev& ix, const BatchDev& b, const SmallRec& r0,
                                           const SmallRec& r1, uint32_t* dirs, int tid)
{
    constexpr int NW = (IMAX + 3) / 4;  // direction words per row at most
    const int qn = (int)((r0.shape >> 8) & 0xffu), tn = (int)(r0.shape & 0xffu);
    const int inner = TINNER ? tn : qn, outer = TINNER ? qn : tn;
    const int stride = (inner + 3) >> 2;
    uint32_t icp[IMAX], s1[IMAX], s2[IMAX];
    uint64_t olo[2], ohi[2];
    {
        uint64_t qlo, qhi, tlo, thi, ilo[2];
        for (int h = 0; h < 2; ++h) {
            const SmallRec& r = h ? r1 : r0;
            load_bases64(b.packed, r.qpos, qlo, qhi);
            load_bases64(ix.center2, r.rs, tlo, thi);
            ilo[h] = TINNER ? tlo : qlo;
            olo[h] = TINNER ? qlo : tlo;
            ohi[h] = TINNER ? qhi : thi;
        }
#pragma unroll
        for (int i = 0; i < IMAX; ++i)
            icp[i] = (uint32_t)((ilo[0] >> (2 * i)) & 3u) | (uint32_t)((ilo[1] >> (2 * i)) & 3u) << 16;
    }
    // (biased by kPB per half: lane16x2's representation)
#pragma unroll
    for (int i = 0; i < IMAX; ++i) s1[i] = kPB2, s2[i] = kPB2;
    const uint32_t k6 = (6u + kPB) * 0x00010001u, k0 = kPB2;
    for (int o = 0; o < outer; ++o) {
        const int sh = 2 * (o & 31);
        const uint32_t ocp = (uint32_t)(((o < 32 ? olo[0] : ohi[0]) >> sh) & 3u) |
                             (uint32_t)(((o < 32 ? olo[1] : ohi[1]) >> sh) & 3u) << 16;
        uint32_t c1 = k0, c2 = o ? k6 : k0;
        uint32_t wd[NW];
#pragma unroll
        for (int k = 0; k < NW; ++k) wd[k] = 0;
#pragma unroll
        for (int i = 0; i < IMAX; ++i) {
            if (i < inner) {
                // z0 = 21 on a match, 12 on a mismatch, per half (biased):
                // mismatch flag t in {0, 1}, z0 = 21 + kPB - 9 t
                const uint32_t t = __vminu2(icp[i] ^ ocp, 0x00010001u);
                const uint32_t z0 = (21u + kPB) * 0x00010001u - 9u * t;
                uint32_t u, v, x, y, d;
                if (TINNER) {
                    const uint32_t ut = o ? s1[i] : (i ? k6 : k0), yt = o ? s2[i] : k0;
                    d = lane16x2<MODE>(z0, c1, c2, ut, yt, u, v, x, y);
                    c1 = x, c2 = v, s1[i] = u, s2[i] = y;
                } else {
                    const uint32_t xt = o ? s1[i] : k0, vt = o ? s2[i] : (i ? k6 : k0);
                    const uint32_t ut = i ? c1 : (o ? k6 : k0), yt = i ? c2 : k0;
                    d = lane16x2<MODE>(z0, xt, vt, ut, yt, u, v, x, y);
                    c1 = u, c2 = y, s1[i] = x, s2[i] = v;
                }
                wd[i >> 2] |= ((d | (d >> 12)) & 0xffu) << (8 * (i & 3));
            }
        }
#pragma unroll
        for (int k = 0; k < NW; ++k)
            if (k < stride) dirs[(o * stride + k) * T + tid] = wd[k];
    }
    // both tracebacks step together: two independent dependency chains
    // (direction reads and state updates) in flight per thread
    uint32_t* out[2] = {b.cig_seg + r0.out, b.cig_seg + r1.out};
    int n[2] = {0, 0}, ti[2] = {tn - 1, tn - 1}, qj[2] = {qn - 1, qn - 1}, state[2] = {0, 0};
    uint32_t run_op[2] = {0xffu, 0xffu}, run_len[2] = {0, 0};
    auto push = [&](int h, uint32_t op, uint32_t len) {
        if (op == run_op[h]) {
            run_len[h] += len;
        } else {
            if (run_len[h]) out[h][n[h]++] = run_len[h] << 4 | run_op[h];
            run_op[h] = op, run_len[h] = len;
        }
    };
    for (;;) {
        const bool act0 = ti[0] >= 0 && qj[0] >= 0, act1 = ti[1] >= 0 && qj[1] >= 0;
        if (!act0 && !act1) break;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if (!(h ? act1 : act0)) continue;
            const int o = TINNER ? qj[h] : ti[h], i = TINNER ? ti[h] : qj[h];
            const uint32_t nib = (dirs[(o * stride + (i >> 2)) * T + tid] >> (8 * (i & 3) + 4 * h)) & 0xfu;
            int st = state[h];
            if (st == 0) st = nib & 3u;
            else if (!((nib >> (st + 1)) & 1u)) st = 0;
            if (st == 0) st = nib & 3u;
            state[h] = st;
            if (st == 0) push(h, 0, 1), --ti[h], --qj[h];
            else if (st == 1) push(h, 2, 1), --ti[h];
            else push(h, 1, 1), --qj[h];
        }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        if (ti[h] >= 0) push(h, 2, (uint32_t)(ti[h] + 1));
        if (qj[h] >= 0) push(h, 1, (uint32_t)(qj[h] + 1));
        if (run_len[h]) out[h][n[h]++] = run_len[h] << 4 | run_op[h];
        b.seg[(h ? r1 : r0).sid].nops = n[h];
    }
}

template <int IMAX, int T>
__device__ __forceinline__ void pair_dispatch(const IndexDev& ix, const BatchDev& b, const SmallRec& r0,
                                              const SmallRec& r1, uint32_t* dirs, int tid, bool tinner, bool left)
{
    if (tinner) {
        if (left) small_pair<true, 1, IMAX, T>(ix, b, r0, r1, dirs, tid);
        else small_pair<true, 2, IMAX, T>(ix, b, r0, r1, dirs, tid);
    } else {
        if (left) small_pair<false, 1, IMAX, T>(ix, b, r0, r1, dirs, tid);
        else small_pair<false, 2, IMAX, T>(ix, b, r0, r1, dirs, tid);
    }
}

template <bool FAST, int IMAX, int T>
__device__ __forceinline__ void small_dispatch(const IndexDev& ix, const BatchDev& b, const SmallRec& r,
                                               uint32_t* dirs, int tid, bool tinner, bool left)
{
    if (tinner) {
        if (left) small_segment<true, 1, FAST, IMAX, T>(ix, b, r, dirs, tid);
        else small_segment<true, 2, FAST, IMAX, T>(ix, b, r, dirs, tid);
    } else {
        if (left) small_segment<false, 1, FAST, IMAX, T>(ix, b, r, dirs, tid);
        else small_segment<false, 2, FAST, IMAX, T>(ix, b, r, dirs, tid);
    }
}

// Small tier, one record per thread (int32 lanes).
__global__ void __launch_bounds__(kDpSmallThreads) dp_small_kernel(IndexDev ix, BatchDev b)
{
    __shared__ uint32_t dirs[kSmallDirWords * kDpSmallThreads];
    const int tid = threadIdx.x;
    const unsigned total = min(b.queues2[1], b.queues2[3]);  // small shapes only
    unsigned long long cell_sum = 0;
    const unsigned wspan = (total + 31u) & ~31u;  // whole warps iterate together for the shuffle
    for (unsigned w = blockIdx.x * kDpSmallThreads + tid; w < wspan; w += gridDim.x * kDpSmallThreads) {
        if (w >= total) continue;
        const SmallRec r = b.work_rec[w];
        const uint32_t rl = r.shape & 0xffu, ql = (r.shape >> 8) & 0xffu;
        const bool tinner = rl <= ql;
        const bool left = (r.shape & kRecLeft) != 0;
        const uint32_t inner = tinner ? rl : ql;
        if (r.shape & kRecFast) {
            if (inner <= 4) small_dispatch<true, 4, kDpSmallThreads>(ix, b, r, dirs, tid, tinner, left);
            else if (inner <= 8) small_dispatch<true, 8, kDpSmallThreads>(ix, b, r, dirs, tid, tinner, left);
            else small_dispatch<true, 16, kDpSmallThreads>(ix, b, r, dirs, tid, tinner, left);
        } else {
            small_dispatch<false, 16, kDpSmallThreads>(ix, b, r, dirs, tid, tinner, left);
        }
        cell_sum += (unsigned long long)(rl * ql);
    }
    for (int o = 16; o > 0; o >>= 1) cell_sum += __shfl_xor_sync(0xffffffffu, cell_sum, o);
    if ((tid & 31) == 0 && cell_sum && b.cells) atomicAdd(b.cells, cell_sum);
}

// Small tier, two records per thread: consecutive records of the
// shape-sorted list share their shape (rl, ql, gap mode, FAST) except at the
// boundary between shapes, so a thread takes records 2w and 2w+1 and runs
// them in the two halves of int16x2 registers (small_pair); a pair whose
// shapes differ, or that has a record off the FAST path, runs as two single
// records (small_segment).  Half the instructions per cell of the int32
// form, but half the warps per SM for the same direction store: on the
// mito workload it measured 5% slower (latency-bound at that occupancy), so
// it is a launch knob (HG_LAUNCH_KNOBS entry 8) the autotuner can choose.
constexpr int kDpSmallPairThreads = 64;

__global__ void __launch_bounds__(kDpSmallPairThreads) dp_small_pair_kernel(IndexDev ix, BatchDev b)
{
    constexpr int T = kDpSmallPairThreads;
    __shared__ uint32_t dirs[2 * kSmallDirWords * T];
    const int tid = threadIdx.x;
    const unsigned total = min(b.queues2[1], b.queues2[3]);  // small shapes only
    const unsigned npair = (total + 1u) / 2u;
    unsigned long long cell_sum = 0;
    const unsigned wspan = (npair + 31u) & ~31u;  // whole warps iterate together for the shuffle
    for (unsigned w = blockIdx.x * T + tid; w < wspan; w += gridDim.x * T) {
        if (w >= npair) continue;
        const SmallRec r0 = b.work_rec[2 * w];
        const bool has1 = 2 * w + 1 < total;
        SmallRec r1 = r0;
        if (has1) r1 = b.work_rec[2 * w + 1];
        const uint32_t rl = r0.shape & 0xffu, ql = (r0.shape >> 8) & 0xffu;
        const bool tinner = rl <= ql;
        const bool left = (r0.shape & kRecLeft) != 0;
        const uint32_t inner = tinner ? rl : ql;
        if (has1 && r1.shape == r0.shape && (r0.shape & kRecFast)) {
            if (inner <= 4) pair_dispatch<4, T>(ix, b, r0, r1, dirs, tid, tinner, left);
            else if (inner <= 8) pair_dispatch<8, T>(ix, b, r0, r1, dirs, tid, tinner, left);
            else pair_dispatch<16, T>(ix, b, r0, r1, dirs, tid, tinner, left);
            cell_sum += 2ull * rl * ql;
            continue;
        }
        for (int h = 0; h < (has1 ? 2 : 1); ++h) {
            const SmallRec& r = h ? r1 : r0;
            const uint32_t hrl = r.shape & 0xffu, hql = (r.shape >> 8) & 0xffu;
            const bool ht = hrl <= hql, hl = (r.shape & kRecLeft) != 0;
            const uint32_t hin = ht ? hrl : hql;
            if (r.shape & kRecFast) {
                if (hin <= 4) small_dispatch<true, 4, T>(ix, b, r, dirs, tid, ht, hl);
                else if (hin <= 8) small_dispatch<true, 8, T>(ix, b, r, dirs, tid, ht, hl);
                else small_dispatch<true, 16, T>(ix, b, r, dirs, tid, ht, hl);
            } else {
                small_dispatch<false, 16, T>(ix, b, r, dirs, tid, ht, hl);
            }
            cell_sum += (unsigned long long)(hrl * hql);
        }
    }
    for (int o = 16; o > 0; o >>= 1) cell_sum += __shfl_xor_sync(0xffffffffu, cell_sum, o);
    if ((tid & 31) == 0 && cell_sum && b.cells) atomicAdd(b.cells, cell_sum);
}

// Medium shapes of the small tier (shorter side 17..32): the same thread-
// per-segment DP with up to four direction words per row, 64 threads per CTA
// so the per-thread store (kMedDirWords) fits shared memory.  Its records
// follow every small shape in the sorted list.
constexpr int kDpMedThreads = 64;

__global__ void __launch_bounds__(kDpMedThreads) dp_medium_kernel(IndexDev ix, BatchDev b)
{
    __shared__ uint32_t dirs[kMedDirWords * kDpMedThreads];
    const int tid = threadIdx.x;
    const unsigned total = b.queues2[3];  // small-tier records (the list without holes)
    const unsigned first = min(b.queues2[1], total);
    unsigned long long cell_sum = 0;
    const unsigned span = ((total - first) + 31u) & ~31u;
    for (unsigned k = blockIdx.x * kDpMedThreads + tid; k < span; k += gridDim.x * kDpMedThreads) {
        const unsigned w = first + k;
        if (w >= total) continue;
        const SmallRec r = b.work_rec[w];
        const uint32_t rl = r.shape & 0xffu, ql = (r.shape >> 8) & 0xffu;
        const bool tinner = rl <= ql;
        const bool left = (r.shape & kRecLeft) != 0;
        if (r.shape & kRecFast) small_dispatch<true, 32, kDpMedThreads>(ix, b, r, dirs, tid, tinner, left);
        else small_dispatch<false, 32, kDpMedThreads>(ix, b, r, dirs, tid, tinner, left);
        cell_sum += (unsigned long long)(rl * ql);
    }
    for (int o = 16; o > 0; o >>= 1) cell_sum += __shfl_xor_sync(0xffffffffu, cell_sum, o);
    if ((tid & 31) == 0 && cell_sum && b.cells) atomicAdd(b.cells, cell_sum);
}

// lane_int_z with the gap mode as a value: nl = 0 left-aligned (MODE 1),
// nl = 1 right-aligned (MODE 2); "> t - 1" is ">= t" for integers.
__device__ __forceinline__ uint32_t lane_int_nl(int z0, int xt1, int vt1, int ut, int yt, int nl, int& u, int& v,
                                                int& x, int& y)
{
    const int a0 = xt1 + vt1, b0 = yt + ut;
    const int m = max(z0, a0);
    uint32_t d = a0 > z0 - nl ? 1u : 0u;
    if (b0 > m - nl) d = 2u;
    const int z = min(max(m, b0), 21);
    u = z - vt1;
    v = z - ut;
    const int zq = z - 6;
    const int a = a0 - zq, b = b0 - zq;
    x = max(a, 0), y = max(b, 0);
    d |= (a > -nl ? 4u : 0u) | (b > -nl ? 8u : 0u);
    return d;
}

// Thin tier: G = floor(32 / W) segments of query length <= W per warp (W is
// the query length up to 16, and 32 above), lane j of group g owns query
// column j of the group's segment and computes cell (s - j, j) at step s.
// A cell takes its left neighbour's outputs of the previous step by one
// shuffle (u, y and the row's center code, packed), its own previous outputs
// as the cell above, and lane 0 of a group reads the center base of a new
// row.  Direction nibbles of 8 steps make one word per lane in the warp's
// scratch; the traceback copies blocks of kThinBlockSteps steps back to
// shared memory and each group's lane 0 walks its segment there, writing op
// runs last-first (as the small tier does).  A deletion run (the bulk of a
// thin segment's path) stays in one column, so its nibbles sit side by side
// in one word: the walk takes all of a word's continuing ones at once.
constexpr int kThinWarps = 4;
constexpr int kThinBlockSteps = 512;
constexpr int kThinBlockWords = kThinBlockSteps / 8 * 32;  // per warp
constexpr size_t kThinSmemBytes = (size_t)kThinWarps * kThinBlockWords * sizeof(uint32_t);

template <int W>
__device__ __forceinline__ void thin_group(const IndexDev& ix, const BatchDev& b, unsigned first, unsigned cnt,
                                           uint32_t* scratch, uint32_t* buf, unsigned long long& cells)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, j = lane % W, g = lane / W;
    const bool has = (unsigned)g < cnt;  // cnt <= 32 / W
    uint32_t sid = 0;
    Seg sg;
    sg.rs = sg.qs = sg.rl = sg.ql = sg.slot = sg.q = sg.kind = 0;
    if (has) {
        sid = b.work_thin_sorted[first + g];
        sg = b.seg[sid];
    }
    const int inner = (int)sg.ql, outer = (int)sg.rl;
    const int nl = (sg.kind & kSegLeft) ? 0 : 1;
    int smax = has ? outer + inner - 1 : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) smax = max(smax, __shfl_xor_sync(FULL, smax, o));
    // z0 by the row's center code (0..4, at 5 bits each) for this lane's query base
    uint32_t tab = 0;
    {
        int ic = 0;
        if (has && j < inner) {
            const uint8_t* pk = b.packed + b.poff[sg.q];
            const int64_t e0 = b.exc_off[sg.q], e1 = b.exc_off[sg.q + 1];
            ic = e0 == e1 ? (int)packed_code(pk, sg.qs + j) : (int)query_dna5(pk, b.exc, e0, e1, sg.qs + j);
        }
#pragma unroll
        for (int oc = 0; oc < 5; ++oc) tab |= (uint32_t)((ic == 4 || oc == 4) ? 16 : (ic == oc ? 21 : 12)) << (5 * oc);
    }
    const uint8_t* tc = ix.center + sg.rs;
    int s1 = 0, s2 = j ? 6 : 0;  // x, v of the cell above row 0
    uint32_t outp = 0;           // u | y << 8 | 5 x center code << 16, toward the right neighbour
    uint32_t chunk = 0, acc = 0;
    const unsigned span = has ? (unsigned)outer : 0u;  // cell (s - j, j) exists for s - j in [0, span)
    for (int s = 0, sm = 0; s < smax; ++s) {
        if (sm == 0) {
            const int o = s + j;
            chunk = (has && o < outer) ? 5u * (uint32_t)tc[o] : 0u;
        }
        const uint32_t fresh = __shfl_sync(FULL, chunk, g * W + sm);
        const uint32_t inp = __shfl_sync(FULL, outp, lane - 1);  // lane 0 of a group ignores it
        sm = sm == W - 1 ? 0 : sm + 1;
        int c1, c2, c5;
        if (j == 0) {
            c1 = s ? 6 : 0, c2 = 0, c5 = (int)fresh;  // left of column 0 on row s
        } else {
            c1 = (int)(inp & 0xffu), c2 = (int)((inp >> 8) & 0xffu), c5 = (int)(inp >> 16);
        }
        const int z0 = (int)((tab >> c5) & 31u);
        int u, v, x, y;
        const uint32_t d = lane_int_nl(z0, s1, s2, c1, c2, nl, u, v, x, y);
        if ((unsigned)(s - j) < span) {
            s1 = x, s2 = v;
            outp = (uint32_t)u | (uint32_t)y << 8 | (uint32_t)c5 << 16;
            acc |= d << (4 * (s & 7));
        }
        if ((s & 7) == 7 || s == smax - 1) {
            scratch[(size_t)(s >> 3) * 32 + lane] = acc;
            acc = 0;
        }
    }
    __syncwarp();
    // traceback from (rl-1, ql-1), block by block from the last
    const bool lead = has && j == 0;
    uint32_t* out = b.cig_seg + (has ? b.coff[sg.q] + sg.slot : 0);
    int n = 0;
    uint32_t run_op = 0xffu, run_len = 0;
    auto push = [&](uint32_t op, uint32_t len) {
        if (op == run_op) {
            run_len += len;
        } else {
            if (run_len) out[n++] = run_len << 4 | run_op;
            run_op = op, run_len = len;
        }
    };
    int ti = outer - 1, qj = inner - 1, state = 0;
    for (int bk = (smax - 1) / kThinBlockSteps; bk >= 0; --bk) {
        const int base = bk * kThinBlockSteps;
        const int need = (lead && ti >= 0 && qj >= 0) ? ti + qj : -1;
        int mx = need;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(FULL, mx, o));
        if (mx < 0) break;
        if (mx < base) continue;
        const int rows = (min(smax, base + kThinBlockSteps) - base + 7) / 8;
        const uint32_t* src = scratch + (size_t)(base / 8) * 32;
        for (int w = lane; w < rows * 32; w += 32) buf[w] = src[w];
        __syncwarp();
        if (lead) {
            while (ti >= 0 && qj >= 0) {
                const int s = ti + qj;
                if (s < base) break;
                const uint32_t word = buf[((s - base) >> 3) * 32 + g * W + qj];
                const int p = s & 7;
                if (state == 1) {  // nibbles p, p-1, .. with the E bit set continue the deletion
                    const uint32_t stop = ~word & (0x44444444u >> (4 * (7 - p)));
                    int run = stop ? p - ((31 - __clz(stop)) >> 2) : p + 1;
                    run = min(run, ti + 1);
                    if (run > 0) {
                        push(2, (uint32_t)run);
                        ti -= run;
                        continue;
                    }
                }
                const uint32_t nib = (word >> (4 * p)) & 0xfu;
                if (state == 0) state = nib & 3u;
                else if (!((nib >> (state + 1)) & 1u)) state = 0;
                if (state == 0) state = nib & 3u;
                if (state == 0) push(0, 1), --ti, --qj;
                else if (state == 1) push(2, 1), --ti;
                else push(1, 1), --qj;
            }
        }
        __syncwarp();
    }
    if (lead) {
        if (ti >= 0) push(2, (uint32_t)(ti + 1));
        if (qj >= 0) push(1, (uint32_t)(qj + 1));
        if (run_len) out[n++] = run_len << 4 | run_op;
        b.seg[sid].nops = n;
        cells += (unsigned long long)sg.rl * sg.ql;
    }
}

// Persistent warps; warp gw owns thin scratch region gw.
// Each warp starts on query length gw % 32 + 1 and moves on when that queue
// is drained; a queue hands out G consecutive entries of its length's range
// of the sorted list (longest first).
template <int W>
__device__ __forceinline__ void thin_drain(const IndexDev& ix, const BatchDev& b, int cls, unsigned lo, unsigned hi,
                                           uint32_t* scratch, uint32_t* buf, unsigned long long& cells)
{
    constexpr unsigned G = 32 / W;
    for (;;) {
        unsigned t = 0;
        if ((threadIdx.x & 31) == 0) t = atomicAdd(&b.thin_q[cls], 1u);
        t = __shfl_sync(0xffffffffu, t, 0);
        const unsigned long long f = (unsigned long long)lo + (unsigned long long)t * G;
        if (f >= hi) break;
        thin_group<W>(ix, b, (unsigned)f, min(G, hi - (unsigned)f), scratch, buf, cells);
    }
}

__global__ void __launch_bounds__(kThinWarps * 32, 4) dp_thin_kernel(IndexDev ix, BatchDev b)
{
    extern __shared__ uint32_t thin_smem[];
    __shared__ unsigned rng[kThinMaxInner + 1];
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    const int gw = blockIdx.x * kThinWarps + wl;
    if (threadIdx.x < 32) {  // per-length ranges of the sorted list from the key counters
        constexpr int per = kThinBins / kThinMaxInner;  // lane c covers length c + 1
        static_assert(kThinMaxInner == 32, "one lane per query length");
        unsigned incl = 0;
        for (int k = 0; k < per; ++k) incl += b.thin_hist[lane * per + k];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned v = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += v;
        }
        if (lane == 0) rng[0] = 0;
        rng[lane + 1] = incl;
    }
    __syncthreads();
    if (gw >= b.thin_nwarps) return;
    uint32_t* scratch = reinterpret_cast<uint32_t*>(b.thin_scratch + (size_t)gw * kThinWarpBytes);
    uint32_t* buf = thin_smem + wl * kThinBlockWords;
    unsigned long long cells = 0;
    for (int k = 0; k < kThinMaxInner; ++k) {
        const int c = (gw + k) % kThinMaxInner;
        const unsigned lo = rng[c], hi = rng[c + 1];
        if (lo >= hi) continue;
        switch (c + 1) {
        case 1: thin_drain<1>(ix, b, c, lo, hi, scratch, buf, cells); break;
        case 2: thin_drain<2>(ix, b, c, lo, hi, scratch, buf, cells); break;
        case 3: thin_drain<3>(ix, b, c, lo, hi, scratch, buf, cells); break;
        case 4: thin_drain<4>(ix, b, c, lo, hi, scratch, buf, cells); break;
        case 5: thin_drain<5>(ix, b, c, lo, hi, scratch, buf, cells); break;
        case 6: thin_drain<6>(ix, b, c, lo, hi, scratch, buf, cells); break;
        case 7: thin_drain<7>(ix, b, c, lo, hi, scratch, buf, cells); break;
        case 8: thin_drain<8>(ix, b, c, lo, hi, scratch, buf, cells); break;
        case 9: thin_drain<9>(ix, b, c, lo, hi, scratch, buf, cells); break;
        case 10: thin_drain<10>(ix, b, c, lo, hi, scratch, buf, cells); break;
        case 11: thin_drain<11>(ix, b, c, lo, hi, scratch, buf, cells); break;
        case 12: thin_drain<12>(ix, b, c, lo, hi, scratch, buf, cells); break;
        case 13: thin_drain<13>(ix, b, c, lo, hi, scratch, buf, cells); break;
        case 14: thin_drain<14>(ix, b, c, lo, hi, scratch, buf, cells); break;
        case 15: thin_drain<15>(ix, b, c, lo, hi, scratch, buf, cells); break;
        case 16: thin_drain<16>(ix, b, c, lo, hi, scratch, buf, cells); break;
        default: thin_drain<32>(ix, b, c, lo, hi, scratch, buf, cells); break;
        }
    }
    for (int o = 16; o > 0; o >>= 1) cells += __shfl_xor_sync(FULL, cells, o);
    if (lane == 0 && cells && b.cells) atomicAdd(b.cells, cells);
}

// Square tier: one thread per segment the band never binds, shorter side up
// to 128.  The row state (s1, s2: one byte per column, 4 columns per word)
// and the inner side's base codes live in shared memory, the thread's words
// interleaved across the CTA; a row is swept 8 columns (one direction word)
// at a time.  Directions go to the warp's scratch slot, interleaved by lane
// (word (o * stride + k) of lane l at [(o * stride + k) * 32 + l]); the
// traceback reads them back there and writes op runs last-first as the small
// tier does.  Values stay in bytes: u, v in [0, 21], x, y in [0, 6].
constexpr int kSquareWarps = 4;
constexpr int kSquareStateWords = kSquareMaxInner / 4;  // per thread and array
constexpr size_t kSquareSmemBytes = (size_t)3 * kSquareStateWords * kSquareWarps * 32 * sizeof(uint32_t);

template <bool TINNER, int MODE>
__device__ __forceinline__ void square_segment(const IndexDev& ix, const BatchDev& b, const Seg& g, uint32_t sid,
                                               uint32_t* S1, uint32_t* S2, uint32_t* IC, uint32_t* dirs)
{
    constexpr int T = kSquareWarps * 32;
    const int qn = (int)g.ql, tn = (int)g.rl;
    const int inner = TINNER ? tn : qn, outer = TINNER ? qn : tn;
    const int stride = (inner + 7) >> 3;
    const uint8_t* pk = b.packed + b.poff[g.q];
    const int64_t e0 = b.exc_off[g.q], e1 = b.exc_off[g.q + 1];
    const bool plain_q = e0 == e1;
    const uint8_t* tc = ix.center + g.rs;
    auto qbase = [&](int j) -> uint32_t {
        return plain_q ? packed_code(pk, g.qs + j) : query_dna5(pk, b.exc, e0, e1, g.qs + j);
    };
    for (int w = 0; w < 2 * stride; ++w) {
        uint32_t v = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int i = 4 * w + k;
            const uint32_t c = i < inner ? (TINNER ? (uint32_t)tc[i] : qbase(i)) : 0u;
            v |= c << (8 * k);
        }
        IC[w * T] = v, S1[w * T] = 0, S2[w * T] = 0;
    }
    for (int o = 0; o < outer; ++o) {
        const int oc = TINNER ? (int)qbase(o) : (int)tc[o];
        int c1 = 0, c2 = o ? 6 : 0;
        for (int k8 = 0; k8 < stride; ++k8) {
            uint32_t dw = 0;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int w = 2 * k8 + h;
                const uint32_t icw = IC[w * T], s1w = S1[w * T], s2w = S2[w * T];
                uint32_t n1 = 0, n2 = 0;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int i = 4 * w + k;
                    if (i < inner) {
                        const int ic = (int)((icw >> (8 * k)) & 0xffu);
                        const int s1 = (int)((s1w >> (8 * k)) & 0xffu), s2 = (int)((s2w >> (8 * k)) & 0xffu);
                        const int z0 = (ic == 4 || oc == 4) ? 16 : (ic == oc ? 21 : 12);
                        int u, v, x, y;
                        uint32_t d;
                        if (TINNER) {
                            const int ut = o ? s1 : (i ? 6 : 0), yt = o ? s2 : 0;
                            d = lane_int_z<MODE>(z0, c1, c2, ut, yt, u, v, x, y);
                            c1 = x, c2 = v;
                            n1 |= (uint32_t)u << (8 * k), n2 |= (uint32_t)y << (8 * k);
                        } else {
                            const int xt = o ? s1 : 0, vt = o ? s2 : (i ? 6 : 0);
                            const int ut = i ? c1 : (o ? 6 : 0), yt = i ? c2 : 0;
                            d = lane_int_z<MODE>(z0, xt, vt, ut, yt, u, v, x, y);
                            c1 = u, c2 = y;
                            n1 |= (uint32_t)x << (8 * k), n2 |= (uint32_t)v << (8 * k);
                        }
                        dw |= d << (4 * (4 * h + k));
                    }
                }
                S1[w * T] = n1, S2[w * T] = n2;
            }
            dirs[(size_t)(o * stride + k8) * 32] = dw;
        }
    }
    // traceback from (tlen-1, qlen-1); runs written once, last-first
    uint32_t* out = b.cig_seg + b.coff[g.q] + g.slot;
    int n = 0;
    uint32_t run_op = 0xffu, run_len = 0;
    auto push = [&](uint32_t op, uint32_t len) {
        if (op == run_op) {
            run_len += len;
        } else {
            if (run_len) out[n++] = run_len << 4 | run_op;
            run_op = op, run_len = len;
        }
    };
    int ti = tn - 1, qj = qn - 1, state = 0;
    while (ti >= 0 && qj >= 0) {
        const int o = TINNER ? qj : ti, i = TINNER ? ti : qj;
        const uint32_t nib = (dirs[(size_t)(o * stride + (i >> 3)) * 32] >> ((i & 7) * 4)) & 0xfu;
        if (state == 0) state = nib & 3u;
        else if (!((nib >> (state + 1)) & 1u)) state = 0;
        if (state == 0) state = nib & 3u;
        if (state == 0) push(0, 1), --ti, --qj;
        else if (state == 1) push(2, 1), --ti;
        else push(1, 1), --qj;
    }
    if (ti >= 0) push(2, (uint32_t)(ti + 1));
    if (qj >= 0) push(1, (uint32_t)(qj + 1));
    if (run_len) out[n++] = run_len << 4 | run_op;
    b.seg[sid].nops = n;
}

// Persistent warps take 32 consecutive entries of the sorted square list at a
// time (queue queues2[2]); warp gw owns scratch slot gw.
__global__ void __launch_bounds__(kSquareWarps * 32, 4) dp_square_kernel(IndexDev ix, BatchDev b)
{
    extern __shared__ uint32_t sq_smem[];
    const unsigned FULL = 0xffffffffu;
    const int tid = threadIdx.x, lane = tid & 31, wl = tid >> 5;
    const int gw = blockIdx.x * kSquareWarps + wl;
    if (gw >= b.dp_nslots) return;
    constexpr int T = kSquareWarps * 32;
    uint32_t* S1 = sq_smem + tid;
    uint32_t* S2 = sq_smem + kSquareStateWords * T + tid;
    uint32_t* IC = sq_smem + 2 * kSquareStateWords * T + tid;
    uint32_t* dirs = reinterpret_cast<uint32_t*>(b.dp_slots + (size_t)gw * b.dp_slot_bytes) + lane;
    const unsigned total = min(*b.n_sq, (unsigned)b.wcap);
    unsigned long long cells = 0;
    for (;;) {
        unsigned t = 0;
        if (lane == 0) t = atomicAdd(&b.queues2[2], 1u);
        t = __shfl_sync(FULL, t, 0);
        if ((unsigned long long)t * 32u >= total) break;
        const unsigned w = t * 32u + (unsigned)lane;
        if (w < total) {
            const uint32_t sid = b.work_sq_sorted[w];
            const Seg g = b.seg[sid];
            const bool tinner = g.rl <= g.ql, left = (g.kind & kSegLeft) != 0;
            if (tinner) {
                if (left) square_segment<true, 1>(ix, b, g, sid, S1, S2, IC, dirs);
                else square_segment<true, 2>(ix, b, g, sid, S1, S2, IC, dirs);
            } else {
                if (left) square_segment<false, 1>(ix, b, g, sid, S1, S2, IC, dirs);
                else square_segment<false, 2>(ix, b, g, sid, S1, S2, IC, dirs);
            }
            cells += (unsigned long long)g.rl * g.ql;
        }
    }
    for (int o = 16; o > 0; o >>= 1) cells += __shfl_xor_sync(FULL, cells, o);
    if (lane == 0 && cells && b.cells) atomicAdd(b.cells, cells);
}

// Histogram of the small-tier shape keys (the chain kernel writes one key
// per work-list entry): per-CTA counters in shared memory, one global atomic
// per non-empty bin and CTA.
constexpr int kShapeHistThreads = 512;
__global__ void __launch_bounds__(kShapeHistThreads) shape_hist_kernel(BatchDev b)
{
    __shared__ uint32_t h[kShapeBins];
    for (int i = threadIdx.x; i < (int)kShapeBins; i += kShapeHistThreads) h[i] = 0;
    __syncthreads();
    const unsigned total = min(*b.n_small, (unsigned)b.wcap);
    for (unsigned w = blockIdx.x * kShapeHistThreads + threadIdx.x; w < total; w += gridDim.x * kShapeHistThreads) {
        const uint32_t key = b.work_key[w];
        if (key != kNoShape) atomicAdd(&h[key], 1u);  // holes carry kNoShape
    }
    __syncthreads();
    for (int i = threadIdx.x; i < (int)kShapeBins; i += kShapeHistThreads)
        if (h[i]) atomicAdd(&b.shape_hist[i], h[i]);
}

// Counting sort of the small-tier work list by shape_key: the chain kernel
// writes each entry's key, shape_hist_kernel the histogram; scan + scatter
// follow.
__global__ void shape_scan_kernel(BatchDev b)
{
    __shared__ uint32_t part[1024];
    const int tid = threadIdx.x;
    const int per = kShapeBins / 1024;
    uint32_t s = 0;
    for (int i = 0; i < per; ++i) s += b.shape_hist[tid * per + i];
    part[tid] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const uint32_t v = tid >= o ? part[tid - o] : 0u;
        __syncthreads();
        part[tid] += v;
        __syncthreads();
    }
    uint32_t run = part[tid] - s;
    for (int i = 0; i < per; ++i) {
        const uint32_t c = b.shape_hist[tid * per + i];
        if ((uint32_t)(tid * per + i) == kShapeMedium) b.queues2[1] = run;  // first medium record
        b.shape_hist[kShapeBins + tid * per + i] = run;  // cursor = bucket start
        run += c;
    }
    if (tid == 1023) b.queues2[3] = run;  // all records
}

// Scatter into shape order.  CTA c takes a contiguous chunk of the chain-
// ordered list, counts its keys in shared memory, reserves one range per
// non-empty key with a single global atomic, then places its items; each
// item becomes a SmallRec (the segment record is read here, in chain order,
// so mostly coalesced).
constexpr int kScatterThreads = 512;

__global__ void __launch_bounds__(kScatterThreads) shape_scatter_kernel(IndexDev ix, BatchDev b)
{
    extern __shared__ uint32_t sh[];  // [kShapeBins] counts, then [kShapeBins] reserved bases
    uint32_t* cnt = sh;
    uint32_t* base = sh + kShapeBins;
    const unsigned total = min(*b.n_small, (unsigned)b.wcap);
    const unsigned chunk = (total + gridDim.x - 1) / gridDim.x;
    const unsigned w0 = blockIdx.x * chunk, w1 = min(w0 + chunk, total);
    if (w0 >= w1) return;
    for (int i = threadIdx.x; i < kShapeBins; i += kScatterThreads) cnt[i] = 0;
    __syncthreads();
    for (unsigned w = w0 + threadIdx.x; w < w1; w += kScatterThreads) {
        const uint32_t key = b.work_key[w];
        if (key != kNoShape) atomicAdd(&cnt[key], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kShapeBins; i += kScatterThreads) {
        const uint32_t c = cnt[i];
        base[i] = c ? atomicAdd(&b.shape_hist[kShapeBins + i], c) : 0u;
        cnt[i] = 0;
    }
    __syncthreads();
    for (unsigned w = w0 + threadIdx.x; w < w1; w += kScatterThreads) {
        const uint32_t key = b.work_key[w];
        if (key == kNoShape) continue;  // a hole of a chain warp's block
        const uint32_t sid = b.work_small[w];
        const uint32_t pos = base[key] + atomicAdd(&cnt[key], 1u);
        const Seg g = b.seg[sid];
        SmallRec r;
        r.qpos = (uint64_t)b.poff[g.q] * 4u + g.qs;
        r.sid = sid;
        r.out = (uint32_t)(b.coff[g.q] + g.slot);
        r.rs = g.rs;
        const bool fast = ix.center_plain && b.exc_off[g.q] == b.exc_off[g.q + 1];
        r.shape = g.rl | g.ql << 8 | ((g.kind & kSegLeft) ? kRecLeft : 0u) | (fast ? kRecFast : 0u);
        r.q = g.q;
        r.pad = 0;
        b.work_rec[pos] = r;
    }
}

constexpr size_t kScatterSmem = 2 * sizeof(uint32_t) * (size_t)kShapeBins;

// ---------------------------------------------------------------- large tier

struct KswArgs {
    int qlen, tlen;
    const uint8_t* query;   // DNA5 codes (or nullptr: read from the packed query)
    const uint8_t* target;
    const uint8_t* pk;      // packed query + exceptions, when query == nullptr
    const int32_t* exc;
    int64_t e0, e1;
    uint32_t qoff;          // query base offset inside the packed query
    int m;
    const int8_t* mat;      // m*m
    int q, e, w, zdrop, end_bonus, flag;
};

struct KswResult {
    int32_t max, zdropped, max_q, max_t, mqe, mqe_t, mte, mte_q, score, reach_end;
    int n_cigar;
    long long cells;  // sum over computed anti-diagonals of (en0 - st0 + 1)
};

__device__ __forceinline__ size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

__host__ __device__ inline size_t ksw_scratch_bytes(int qlen, int tlen, int w, int flag)
{
    if (qlen <= 0 || tlen <= 0) return 0;
    if (w < 0) w = tlen > qlen ? tlen : qlen;
    const size_t tl16 = (size_t)((tlen + 15) / 16) * 16;
    int n_col = qlen < tlen ? qlen : tlen;
    n_col = ((n_col < w + 1 ? n_col : w + 1) + 15) / 16 + 1;
    size_t s = ((tl16 * 5 + 15) & ~(size_t)15) + ((tl16 * 4 + 15) & ~(size_t)15);
    if (!(flag & kEzScoreOnly)) {
        s += ((((size_t)(qlen + tlen - 1) * n_col + 1) * 16 + 15) & ~(size_t)15);
        s += (((size_t)(qlen + tlen - 1) * 8 + 15) & ~(size_t)15);
    }
    return s;
}

__device__ __forceinline__ uint32_t ksw_qcode(const KswArgs& a, int j)
{
    return a.query ? a.query[j] : query_dna5(a.pk, a.exc, a.e0, a.e1, a.qoff + (uint32_t)j);
}

// Warp-cooperative ksw_extz2_sse.  All 32 lanes call it; returns the same
// KswResult in every lane.  The CIGAR (cap entries) goes to `cig`.
__device__ KswResult ksw_extz2_warp(const KswArgs& a, uint8_t* scratch, uint32_t* cig, int cap)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    KswResult R;
    R.max_q = R.max_t = R.mqe_t = R.mte_q = -1;
    R.max = 0, R.score = R.mqe = R.mte = kNegInf;
    R.zdropped = 0, R.reach_end = 0, R.n_cigar = 0, R.cells = 0;
    const int qlen = a.qlen, tlen = a.tlen, m = a.m, q = a.q, e = a.e;
    if (m <= 0 || qlen <= 0 || tlen <= 0) return R;
    const int qe = q + e, with_cigar = !(a.flag & kEzScoreOnly), approx_max = !!(a.flag & kEzApproxMax);
    const int mode = !with_cigar ? 0 : ((a.flag & kEzRight) ? 2 : 1);
    const uint32_t qe2 = (uint32_t)((q + e) * 2) & 0xffu, max_sc = (uint32_t)(a.mat[0] + (q + e) * 2) & 0xffu;
    int w = a.w;
    if (w < 0) w = tlen > qlen ? tlen : qlen;
    const int wl = w, wr = w;
    const int tlen_ = (tlen + 15) / 16;
    int n_col_ = qlen < tlen ? qlen : tlen;
    n_col_ = ((n_col_ < w + 1 ? n_col_ : w + 1) + 15) / 16 + 1;
    int min_sc = a.mat[1];
    for (int t = 1; t < m * m; ++t) min_sc = min(min_sc, (int)a.mat[t]);
    if (-min_sc > 2 * (q + e)) return R;
    const size_t Lb = (size_t)tlen_ * 16;
    uint8_t* u = scratch;
    uint8_t* v = u + Lb;
    uint8_t* x = v + Lb;
    uint8_t* y = x + Lb;
    uint8_t* s = y + Lb;
    int32_t* H = reinterpret_cast<int32_t*>(scratch + align16(Lb * 5));
    uint8_t* p = scratch + align16(Lb * 5) + align16(Lb * 4);
    const size_t ncol = (size_t)n_col_ * 16;
    const size_t nd = (size_t)(qlen + tlen - 1);
    int* off = reinterpret_cast<int*>(p + align16((nd * n_col_ + 1) * 16));
    int* off_end = off + nd;
    for (size_t i = lane; i < Lb * 5; i += 32) u[i] = 0;
    if (!approx_max)
        for (size_t i = lane; i < Lb; i += 32) H[i] = kNegInf;
    __syncwarp();
    int32_t H0 = 0, last_H0_t = 0;
    int last_st = -1, last_en = -1;
    for (int r = 0; r < qlen + tlen - 1; ++r) {
        int st = 0, en = tlen - 1;
        if (st < r - qlen + 1) st = r - qlen + 1;
        if (en > r) en = r;
        if (st < (r - wr + 1) >> 1) st = (r - wr + 1) >> 1;
        if (en > (r + wl) >> 1) en = (r + wl) >> 1;
        if (st > en) {
            R.zdropped = 1;
            break;
        }
        const int st0 = st, en0 = en;
        R.cells += en0 - st0 + 1;
        st = st / 16 * 16, en = (en + 16) / 16 * 16 - 1;
        uint32_t x1, v1;
        if (st > 0) {
            if (st - 1 >= last_st && st - 1 <= last_en) x1 = x[st - 1], v1 = v[st - 1];
            else x1 = v1 = 0;
        } else
            x1 = 0, v1 = r ? (uint32_t)q : 0u;
        const uint32_t x1e = (x1 & 0x80u) ? 0xffu : 0u, v1e = (v1 & 0x80u) ? 0xffu : 0u;
        __syncwarp();
        if (lane == 0 && en >= r) y[r] = 0, u[r] = (uint8_t)(r ? q : 0);
        if (a.flag & kEzGenericSc) {
            for (int t = st0 + lane; t <= en0; t += 32) s[t] = (uint8_t)a.mat[a.target[t] * m + ksw_qcode(a, r - t)];
        } else {
            // match/mismatch scoring with symbol m-1 as the wildcard
            // (ksw2_extz2_sse.c:123-137): the reference fills whole 16-byte
            // blocks from st0, so lanes past en0 up to the block end get a
            // score too, from what its buffers hold there - the target copy's
            // zero padding up to Lb, then the reversed query (zeros past its
            // end).  Those lanes are stale state for later anti-diagonals.
            // Lanes at or past Lb are never computed, so they are not stored.
            const int mch = a.mat[0], mis = a.mat[1];
            const int scn = a.mat[m * m - 1] == 0 ? -e : a.mat[m * m - 1];
            const int tend = min(st0 + ((en0 - st0) / 16 + 1) * 16 - 1, (int)Lb - 1);
            for (int t = st0 + lane; t <= tend; t += 32) {
                int sq;  // the target copy at t
                if (t < tlen) sq = a.target[t];
                else if (t < (int)Lb) sq = 0;
                else sq = t - (int)Lb < qlen ? ksw_qcode(a, qlen - 1 - (t - (int)Lb)) : 0;
                const int kq = qlen - 1 - r + t;  // the reversed query at qlen-1-r+t
                const int sr = kq < qlen ? ksw_qcode(a, qlen - 1 - kq) : 0;
                int sc = sq == sr ? mch : mis;
                if (sq == m - 1 || sr == m - 1) sc = scn;
                s[t] = (uint8_t)sc;
            }
        }
        __syncwarp();
        if (with_cigar && lane == 0) off[r] = st, off_end[r] = en;
        uint8_t* pr = with_cigar ? p + (size_t)r * ncol : nullptr;
        uint32_t cx = x1, cv = v1;
        for (int c0 = st; c0 <= en; c0 += 32) {
            const int t = c0 + lane;
            const bool act = t <= en;
            const uint32_t xo = act ? x[t] : 0u, vo = act ? v[t] : 0u, ut = act ? u[t] : 0u, yt = act ? y[t] : 0u,
                           sv = act ? s[t] : 0u;
            uint32_t xt1 = __shfl_up_sync(FULL, xo, 1), vt1 = __shfl_up_sync(FULL, vo, 1);
            if (lane == 0) xt1 = cx, vt1 = cv;
            if (c0 == st && lane >= 1 && lane <= 3) xt1 |= x1e, vt1 |= v1e;
            cx = __shfl_sync(FULL, xo, 31);
            cv = __shfl_sync(FULL, vo, 31);
            __syncwarp();
            if (act) {
                const LaneOut o = ksw_lane(sv, xt1, vt1, ut, yt, qe2, max_sc, (uint32_t)q & 0xffu, mode);
                u[t] = o.u, v[t] = o.v, x[t] = o.x, y[t] = o.y;
                if (with_cigar) pr[t - st] = o.d;
            }
            __syncwarp();
        }
        if (!approx_max) {
            int32_t max_H, max_t;
            if (r > 0) {
                int32_t hen = 0;
                if (lane == 0) hen = en0 > 0 ? H[en0 - 1] + (int32_t)u[en0] - qe : H[en0] + (int32_t)v[en0] - qe;
                hen = __shfl_sync(FULL, hen, 0);
                __syncwarp();
                if (lane == 0) H[en0] = hen;
                max_H = hen, max_t = en0;
                const int en1 = st0 + (en0 - st0) / 4 * 4;
                // lanes t = st0 + lane + 32k: SIMD lane (t - st0) & 3 == lane & 3
                int32_t gh = max_H, gt = max_t;
                for (int t = st0 + lane; t < en0; t += 32) {
                    const int32_t h = H[t] + (int32_t)v[t] - qe;
                    H[t] = h;
                    if (t < en1 && h > gh) gh = h, gt = t;
                }
                // reduce within each SIMD-lane group: larger H, then smaller t
#pragma unroll
                for (int o = 4; o < 32; o <<= 1) {
                    const int32_t oh = __shfl_xor_sync(FULL, gh, o), ot = __shfl_xor_sync(FULL, gt, o);
                    const bool og = oh > max_H;   // the other side moved off the initial value
                    const bool mg = gh > max_H;
                    if (og && (!mg || oh > gh || (oh == gh && ot < gt))) gh = oh, gt = ot;
                }
                __syncwarp();
                // combine the four groups in order, then the scalar tail
                for (int g = 0; g < 4; ++g) {
                    const int32_t oh = __shfl_sync(FULL, gh, g), ot = __shfl_sync(FULL, gt, g);
                    if (max_H < oh) max_H = oh, max_t = ot;
                }
                for (int t = en1; t < en0; ++t) {
                    const int32_t h = H[t];
                    if (h > max_H) max_H = h, max_t = t;
                }
            } else {
                if (lane == 0) H[0] = (int32_t)v[0] - qe - qe;
                __syncwarp();
                max_H = H[0], max_t = 0;
            }
            __syncwarp();
            if (en0 == tlen - 1 && H[en0] > R.mte) R.mte = H[en0], R.mte_q = r - en;
            if (r - st0 == qlen - 1 && H[st0] > R.mqe) R.mqe = H[st0], R.mqe_t = st0;
            // ksw_apply_zdrop (include/ksw2.h:191-207)
            bool stop = false;
            if (max_H > R.max) {
                R.max = max_H, R.max_t = max_t, R.max_q = r - max_t;
            } else if (max_t >= R.max_t && r - max_t >= R.max_q) {
                const int tl = max_t - R.max_t, ql = (r - max_t) - R.max_q;
                const int l = tl > ql ? tl - ql : ql - tl;
                if (a.zdrop >= 0 && R.max - max_H > a.zdrop + l * e) R.zdropped = 1, stop = true;
            }
            if (stop) break;
            if (r == qlen + tlen - 2 && en0 == tlen - 1) R.score = H[tlen - 1];
        } else {
            __syncwarp();
            if (r > 0) {
                if (last_H0_t >= st0 && last_H0_t <= en0 && last_H0_t + 1 >= st0 && last_H0_t + 1 <= en0) {
                    const int32_t d0 = (int32_t)v[last_H0_t] - qe, d1 = (int32_t)u[last_H0_t + 1] - qe;
                    if (d0 > d1) H0 += d0;
                    else H0 += d1, ++last_H0_t;
                } else if (last_H0_t >= st0 && last_H0_t <= en0) {
                    H0 += (int32_t)v[last_H0_t] - qe;
                } else {
                    ++last_H0_t, H0 += (int32_t)u[last_H0_t] - qe;
                }
                if (a.flag & kEzApproxDrop) {
                    bool stop = false;
                    if (H0 > R.max) {
                        R.max = H0, R.max_t = last_H0_t, R.max_q = r - last_H0_t;
                    } else if (last_H0_t >= R.max_t && r - last_H0_t >= R.max_q) {
                        const int tl = last_H0_t - R.max_t, ql = (r - last_H0_t) - R.max_q;
                        const int l = tl > ql ? tl - ql : ql - tl;
                        if (a.zdrop >= 0 && R.max - H0 > a.zdrop + l * e) R.zdropped = 1, stop = true;
                    }
                    if (stop) break;
                }
            } else
                H0 = (int32_t)v[0] - qe - qe, last_H0_t = 0;
            if (r == qlen + tlen - 2 && en0 == tlen - 1) R.score = H0;
        }
        last_st = st, last_en = en;
        __syncwarp();
    }
    __syncwarp();
    if (with_cigar) {
        int i0 = -1, j0 = -1;
        if (!R.zdropped && !(a.flag & kEzExtzOnly)) i0 = tlen - 1, j0 = qlen - 1;
        else if (!R.zdropped && (a.flag & kEzExtzOnly) && R.mqe + a.end_bonus > R.max) R.reach_end = 1, i0 = R.mqe_t, j0 = qlen - 1;
        else if (R.max_t >= 0 && R.max_q >= 0) i0 = R.max_t, j0 = R.max_q;
        if (i0 >= 0 || j0 >= 0) {
            int n = 0;
            if (lane == 0) {
                CigarPush cp{cig, 0, cap, 0};
                int i = i0, j = j0, state = 0;
                while (i >= 0 && j >= 0) {
                    const int rr = i + j;
                    int force = -1;
                    uint32_t tmp;
                    if (i < off[rr]) force = 2;
                    if (i > off_end[rr]) force = 1;
                    tmp = force < 0 ? p[(size_t)rr * ncol + (size_t)(i - off[rr])] : 0u;
                    if (state == 0) state = tmp & 7;
                    else if (!(tmp >> (state + 2) & 1)) state = 0;
                    if (state == 0) state = tmp & 7;
                    if (force >= 0) state = force;
                    if (state == 0) cp.push(0, 1), --i, --j;
                    else if (state == 1 || state == 3) cp.push(2, 1), --i;
                    else cp.push(1, 1), --j;
                }
                if (i >= 0) cp.push(2, (uint32_t)(i + 1));
                if (j >= 0) cp.push(1, (uint32_t)(j + 1));
                if (cp.n <= cap && !(a.flag & kEzRevCigar))
                    for (int k = 0; k < cp.n / 2; ++k) {
                        const uint32_t tt = cig[k];
                        cig[k] = cig[cp.n - 1 - k];
                        cig[cp.n - 1 - k] = tt;
                    }
                n = cp.n;
            }
            R.n_cigar = __shfl_sync(FULL, n, 0);
        }
    }
    return R;
}

// ------------------------------------------------------------------------
// Wavefront tiers.  For every segment whose band never binds (auto_band < 0
// or >= both lengths) the DP is the small tier's per-cell int32 recurrence
// (lane_int), so it needs neither the anti-diagonal byte arrays nor the H row
// of the exact emulation.  A group of GW warps (1, or a 16-warp CTA for wide
// segments) runs it as a register wavefront over anti-diagonals: virtual
// lane v = 32 x warp + lane owns the P consecutive columns c = vP .. vP+P-1
// of the shorter side, and cell (o, c) runs at step o + c, so the P cells a
// lane computes per step are independent.  The pair carried along a row and
// the row's outer base move one column per step: inside a lane through
// registers, to the next lane through a shuffle, across a warp boundary
// through a shared-memory ring (the warps run 32-step windows with a barrier
// between windows, warp k one window behind warp k-1).  Column 0 takes the
// boundary column and a fresh outer base.
//
// Direction nibbles: one word holds 8/P steps x P columns of one virtual
// lane; step group t of lane v is word t x LDW + v (LDW = lanes that hold
// columns).  The traceback walks K-step blocks held in shared memory, from
// the last block to the first (the step index o + c never increases along
// the path).  A segment of one block computes straight into shared memory.
// A longer one either writes every word to global scratch during the single
// forward pass and copies each block back for the walk, or - when no scratch
// of that size is left - saves each warp's state at every block start
// (per column: its state and its last outputs) and recomputes
// each block from its saved state for the walk.
constexpr int kWaveWarpDirWords = 2048;   // one-warp groups: 8 KB per warp
constexpr int kWaveCtaWarps = 16;
constexpr int kWaveCtaDirWords = 32768;   // CTA group: 128 KB
constexpr int kWaveRing = 128;            // ring entries per warp boundary (4 windows)

struct WaveGeom {
    int P, lanes, nw, K, S, nblk, ckw;  // cols/lane, column lanes, active warps, steps/block, steps, blocks, ckpt words
};

__host__ __device__ __forceinline__ WaveGeom wave_geom(int inner, int outer, int P, int dir_words)
{
    WaveGeom G;
    G.P = P;
    G.lanes = (inner + P - 1) / P;
    G.nw = (G.lanes + 31) / 32;
    G.K = ((dir_words / G.lanes) * (8 / P)) & ~31;   // steps per block, a multiple of 32
    G.S = outer + inner - 1;                          // cell (o, c) runs at step o + c
    G.nblk = (G.S + G.K - 1) / G.K;
    G.ckw = (5 * P + 3) / 4;
    return G;
}

// Global direction words of a segment (every step group x column lanes).
__host__ __device__ __forceinline__ size_t wave_gdir_bytes(const WaveGeom& G)
{
    const int spw = 8 / G.P;
    return G.nblk > 1 ? (size_t)((G.S + spw - 1) / spw) * G.lanes * sizeof(uint32_t) : 0;
}

// Checkpoint bytes: one record (ckw words x 32 lanes per active warp) per
// block; blocks 0 and nblk-1 need none but keep their slots for indexing.
__host__ __device__ __forceinline__ size_t wave_ckpt_bytes(const WaveGeom& G)
{
    return G.nblk > 2 ? (size_t)G.nblk * G.nw * G.ckw * 32 * sizeof(uint32_t) : 0;
}

template <int GW>
__device__ __forceinline__ void wave_sync()
{
    if (GW == 1) __syncwarp();
    else __syncthreads();
}

template <int GW, int P, bool TINNER, int MODE>
__device__ __forceinline__ void wave_segment(const IndexDev& ix, const BatchDev& b, uint32_t sid, const Seg& g,
                                             uint32_t* dirs, int dir_words, uint32_t* ring, uint32_t* scratch,
                                             bool gmode, int* flag)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int wk = GW == 1 ? 0 : (int)(threadIdx.x >> 5);
    constexpr int SPW = 8 / P;                       // steps per direction word
    constexpr int CKW = (5 * P + 3) / 4;             // checkpoint words per lane (5 bytes per column)
    const int qn = (int)g.ql, tn = (int)g.rl;
    const int inner = TINNER ? tn : qn, outer = TINNER ? qn : tn;
    const WaveGeom G = wave_geom(inner, outer, P, dir_words);
    const int NW = G.nw, K = G.K, S = G.S, nblk = G.nblk, LDW = G.lanes;
    const bool active = wk < NW;
    const int v = wk * 32 + lane;                    // virtual lane; columns v*P .. v*P+P-1
    const bool holds = v < LDW;                      // this lane owns columns
    const uint8_t* pk = b.packed + b.poff[g.q];
    const int64_t e0 = b.exc_off[g.q], e1 = b.exc_off[g.q + 1];
    const bool plain_q = e0 == e1;
    const uint8_t* tc = ix.center + g.rs;
    // per column: score table (z0 = score + 16 at bit 5 x outer code), column
    // state from the row above (s1, s2) and the column's outputs of the last
    // step (r1, r2: carried pair; r5: 5 x the row's outer code)
    uint32_t tab[P];
    int s1[P], s2[P], r1[P], r2[P], r5[P];
#pragma unroll
    for (int p = 0; p < P; ++p) {
        const int c = v * P + p;
        s1[p] = s2[p] = r1[p] = r2[p] = r5[p] = 0;
        int ic = 0;
        if (active && c < inner) {
            if (TINNER) ic = tc[c];
            else ic = plain_q ? (int)packed_code(pk, g.qs + c) : (int)query_dna5(pk, b.exc, e0, e1, g.qs + c);
        }
        uint32_t t = 0;
#pragma unroll
        for (int oc = 0; oc < 5; ++oc) t |= (uint32_t)((ic == 4 || oc == 4) ? 16 : (ic == oc ? 21 : 12)) << (5 * oc);
        tab[p] = t;
    }
    auto pack_last = [&]() -> uint32_t {
        return (uint32_t)r1[P - 1] | (uint32_t)r2[P - 1] << 8 | (uint32_t)r5[P - 1] << 16;
    };
    auto init_state = [&]() {
#pragma unroll
        for (int p = 0; p < P; ++p) {
            const int c = v * P + p;
            if (TINNER) s1[p] = c ? 6 : 0, s2[p] = 0;   // u, y above row 0
            else s1[p] = 0, s2[p] = c ? 6 : 0;          // x, v left of column 0
            r1[p] = r2[p] = r5[p] = 0;
        }
    };
    // checkpoint: 5 bytes per column (s1, s2, r1, r2, r5)
    auto ck = [&](int bk, int w) -> uint32_t& { return scratch[((bk * NW + wk) * CKW + w) * 32 + lane]; };
    auto byte_of = [&](int k) -> int {
        const int p = k % P, f = k / P;
        return f == 0 ? s1[p] : f == 1 ? s2[p] : f == 2 ? r1[p] : f == 3 ? r2[p] : r5[p];
    };
    auto set_byte = [&](int k, int val) {
        const int p = k % P, f = k / P;
        if (f == 0) s1[p] = val;
        else if (f == 1) s2[p] = val;
        else if (f == 2) r1[p] = val;
        else if (f == 3) r2[p] = val;
        else r5[p] = val;
    };
    auto save = [&](int bk) {
#pragma unroll
        for (int w = 0; w < CKW; ++w) {
            uint32_t wd = 0;
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (4 * w + j < 5 * P) wd |= (uint32_t)byte_of(4 * w + j) << (8 * j);
            ck(bk, w) = wd;
        }
    };
    auto restore = [&](int bk) {
#pragma unroll
        for (int w = 0; w < CKW; ++w) {
            const uint32_t wd = ck(bk, w);
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (4 * w + j < 5 * P) set_byte(4 * w + j, (int)((wd >> (8 * j)) & 0xffu));
        }
    };
    // 5 x outer code of row o (0 past the end)
    auto outer_code5 = [&](int o) -> uint32_t {
        if (o >= outer) return 0u;
        uint32_t c;
        if (TINNER) c = plain_q ? packed_code(pk, g.qs + o) : query_dna5(pk, b.exc, e0, e1, g.qs + o);
        else c = tc[o];
        return 5u * c;
    };
    // One step at s: column p of lane v computes row s - (v*P + p), so the P
    // cells of a lane are independent.  Column p takes the pair carried from
    // column p-1's previous step (column 0: from the lane below by shuffle,
    // across a warp boundary from the ring; virtual lane 0: the boundary and
    // a fresh outer base).  `chunk`/`ringv` hold window values at lane s & 31.
    auto step = [&](auto guard_tag, int s, uint32_t chunk, uint32_t ringv) -> uint32_t {
        constexpr bool GUARD = decltype(guard_tag)::value;
        int c1 = __shfl_up_sync(FULL, r1[P - 1], 1);
        int c2 = __shfl_up_sync(FULL, r2[P - 1], 1);
        int c5 = __shfl_up_sync(FULL, r5[P - 1], 1);
        const uint32_t fresh = __shfl_sync(FULL, chunk, s & 31);
        if (GW > 1) {
            const uint32_t rv = __shfl_sync(FULL, ringv, s & 31);
            if (lane == 0 && wk > 0) c1 = (int)(rv & 0xffu), c2 = (int)((rv >> 8) & 0xffu), c5 = (int)(rv >> 16);
        }
        if (v == 0) {
            const int ob = s ? 6 : 0;
            c1 = TINNER ? 0 : ob;
            c2 = TINNER ? ob : 0;
            c5 = (int)fresh;
        }
        uint32_t dn = 0;
#pragma unroll
        for (int p = P - 1; p >= 0; --p) {  // descending: column p reads column p-1's previous outputs
            const int i1 = p ? r1[p - 1] : c1, i2 = p ? r2[p - 1] : c2, i5 = p ? r5[p - 1] : c5;
            const int o = s - (v * P + p);
            if (!GUARD || (o >= 0 && o < outer && v * P + p < inner)) {
                const int z0 = (int)((tab[p] >> i5) & 31u);
                int u, vv, x, y;
                uint32_t d;
                if (TINNER) {
                    d = lane_int_z<MODE>(z0, i1, i2, s1[p], s2[p], u, vv, x, y);
                    r1[p] = x, r2[p] = vv, s1[p] = u, s2[p] = y;
                } else {
                    d = lane_int_z<MODE>(z0, s1[p], s2[p], i1, i2, u, vv, x, y);
                    r1[p] = u, r2[p] = y, s1[p] = x, s2[p] = vv;
                }
                r5[p] = i5;
                dn |= d << (4 * p);
            }
        }
        if (GW > 1 && lane == 31) ring[wk * kWaveRing + (s & (kWaveRing - 1))] = pack_last();
        return dn;
    };
    // Steps [sb, se) of every active warp, sb a multiple of 32; whole 32-step
    // windows run (steps past the segment's last are inactive in every
    // column, and recomputed blocks end on a window boundary).  Words of step
    // groups >= dbase go to shared memory (the block it holds starts at
    // dbase); with to_global every word goes to global scratch instead; with
    // save_ck each warp saves its state at the block starts below the last.
    auto run = [&](int sb, int se, int dbase, bool to_global, bool save_ck) {
        const int nwin = (se - sb + 31) / 32 + (GW > 1 ? NW - 1 : 0);
        const int clo = wk * 32 * P, chi = min(LDW, wk * 32 + 32) * P - 1;  // this warp's columns
        uint32_t chunk_next = (active && wk == 0) ? outer_code5(sb + lane) : 0u;
        for (int j = 0; j < nwin; ++j) {
            const int s0 = sb + (j - wk) * 32;
            if (active && s0 >= sb && s0 < se) {
                if (save_ck && s0 > 0 && s0 % K == 0 && s0 / K <= nblk - 2) save(s0 / K);
                const uint32_t chunk = chunk_next;
                if (wk == 0) chunk_next = outer_code5(s0 + 32 + lane);
                uint32_t ringv = 0;
                if (GW > 1 && wk > 0) ringv = ring[(wk - 1) * kWaveRing + ((s0 - 1 + lane) & (kWaveRing - 1))];
                // every real column of the warp on a row inside the segment for the
                // whole window (columns past the last only feed columns past the last)
                const bool fast = s0 - min(chi, inner - 1) >= 0 && s0 + 31 - clo <= outer - 1;
                for (int gq = 0; gq < 32 / SPW; ++gq) {
                    const int sg = s0 + gq * SPW;
                    uint32_t acc = 0;
                    if (fast) {
#pragma unroll
                        for (int k = 0; k < SPW; ++k)
                            acc |= step(std::false_type{}, sg + k, chunk, ringv) << (4 * P * k);
                    } else {
#pragma unroll
                        for (int k = 0; k < SPW; ++k)
                            acc |= step(std::true_type{}, sg + k, chunk, ringv) << (4 * P * k);
                    }
                    if (holds && sg < se) {
                        if (to_global) scratch[(size_t)(sg / SPW) * LDW + v] = acc;
                        else if (sg >= dbase) dirs[((sg - dbase) / SPW) * LDW + v] = acc;
                    }
                }
            }
            if (GW > 1) __syncthreads();
        }
    };
    init_state();
    const bool ckmode = nblk > 1 && !gmode;
    run(0, S, (nblk - 1) * K, gmode && nblk > 1, ckmode && nblk > 2);
    wave_sync<GW>();
    // traceback from (tlen-1, qlen-1) by the group's first thread
    const bool lead = wk == 0 && lane == 0;
    CigarPush cp{b.cig_seg + b.coff[g.q] + g.slot, 0, tn + qn, 0};
    int ti = tn - 1, qj = qn - 1, state = 0;
    for (int bk = nblk - 1;;) {
        if (gmode && nblk > 1) {  // bring block bk's words back from global scratch
            const int w0 = (bk * K / SPW) * LDW;
            const int w1 = ((min((bk + 1) * K, S) + SPW - 1) / SPW) * LDW;
            for (int i = wk * 32 + lane; i < w1 - w0; i += GW * 32) dirs[i] = scratch[(size_t)w0 + i];
            wave_sync<GW>();
        }
        int done = 0;
        if (lead) {
            const int base = bk * K;
            while (ti >= 0 && qj >= 0) {
                const int o = TINNER ? qj : ti, c = TINNER ? ti : qj;
                const int s = o + c;
                if (s < base) break;
                const uint32_t word = dirs[((s - base) / SPW) * LDW + c / P];
                const uint32_t nib = (word >> (4 * (P * (s % SPW) + c % P))) & 0xfu;
                if (state == 0) state = nib & 3u;
                else if (!((nib >> (state + 1)) & 1u)) state = 0;
                if (state == 0) state = nib & 3u;
                if (state == 0) cp.push(0, 1), --ti, --qj;
                else if (state == 1) cp.push(2, 1), --ti;
                else cp.push(1, 1), --qj;
            }
            done = !(ti >= 0 && qj >= 0);
            if (GW > 1) *flag = done;
        }
        if (GW == 1) {
            done = __shfl_sync(FULL, done, 0);
        } else {
            __syncthreads();
            done = *flag;
        }
        if (done || bk == 0) break;
        --bk;
        wave_sync<GW>();
        if (!gmode) {  // recompute block bk from its saved state
            if (active) {
                if (bk == 0) init_state();
                else restore(bk);
                if (GW > 1 && lane == 31 && bk > 0) ring[wk * kWaveRing + ((bk * K - 1) & (kWaveRing - 1))] = pack_last();
            }
            wave_sync<GW>();
            run(bk * K, (bk + 1) * K, bk * K, false, false);
            wave_sync<GW>();
        }
    }
    if (lead) {
        if (ti >= 0) cp.push(2, (uint32_t)(ti + 1));
        if (qj >= 0) cp.push(1, (uint32_t)(qj + 1));
        for (int i = 0; i < cp.n / 2; ++i) {
            const uint32_t a = cp.out[i];
            cp.out[i] = cp.out[cp.n - 1 - i];
            cp.out[cp.n - 1 - i] = a;
        }
        b.seg[sid].nops = cp.n;
        if (b.cells) atomicAdd(b.cells, (unsigned long long)g.rl * g.ql);
    }
    wave_sync<GW>();
}

template <int GW, bool TINNER, int MODE>
__device__ __forceinline__ void wave_dispatch_p(const IndexDev& ix, const BatchDev& b, uint32_t sid, const Seg& g,
                                                int P, uint32_t* dirs, int dir_words, uint32_t* ring,
                                                uint32_t* scratch, bool gmode, int* flag)
{
    if (P == 1) wave_segment<GW, 1, TINNER, MODE>(ix, b, sid, g, dirs, dir_words, ring, scratch, gmode, flag);
    else if (P == 2) wave_segment<GW, 2, TINNER, MODE>(ix, b, sid, g, dirs, dir_words, ring, scratch, gmode, flag);
    else if (P == 4) wave_segment<GW, 4, TINNER, MODE>(ix, b, sid, g, dirs, dir_words, ring, scratch, gmode, flag);
    else wave_segment<GW, 8, TINNER, MODE>(ix, b, sid, g, dirs, dir_words, ring, scratch, gmode, flag);
}

template <int GW>
__device__ __forceinline__ void wave_dispatch(const IndexDev& ix, const BatchDev& b, uint32_t sid, const Seg& g,
                                              int P, uint32_t* dirs, int dir_words, uint32_t* ring,
                                              uint32_t* scratch, bool gmode, int* flag)
{
    const bool tinner = g.rl <= g.ql;
    const bool left = (g.kind & kSegLeft) != 0;
    if (tinner) {
        if (left) wave_dispatch_p<GW, true, 1>(ix, b, sid, g, P, dirs, dir_words, ring, scratch, gmode, flag);
        else wave_dispatch_p<GW, true, 2>(ix, b, sid, g, P, dirs, dir_words, ring, scratch, gmode, flag);
    } else {
        if (left) wave_dispatch_p<GW, false, 1>(ix, b, sid, g, P, dirs, dir_words, ring, scratch, gmode, flag);
        else wave_dispatch_p<GW, false, 2>(ix, b, sid, g, P, dirs, dir_words, ring, scratch, gmode, flag);
    }
}

// Scratch of a wavefront segment, decided by the group's leader: direction
// words in the group's reusable slot or in the bump arena when they fit
// (gmode), else checkpoints in the slot or the arena, else the status gets
// kStArenaOverflow.  code: 0 none needed, 1 slot, 2 arena (offset in *off),
// 3 overflow; bit 2 set = gmode.
__device__ __forceinline__ uint32_t wave_scratch_plan(const BatchDev& b, const WaveGeom& G, int slot,
                                                      unsigned long long* off)
{
    if (G.nblk <= 1) return 0;
    const bool slot_ok = slot < b.dp_nslots;
    const size_t gbytes = wave_gdir_bytes(G), cbytes = wave_ckpt_bytes(G);
    if (slot_ok && (int64_t)gbytes <= b.dp_slot_bytes) return 1 | 4;
    const unsigned long long ga = (gbytes + 255) & ~(size_t)255;
    if (*(volatile unsigned long long*)b.dp_cursor + ga <= (unsigned long long)b.dp_cap) {  // likely room: claim it
        const unsigned long long o = atomicAdd(b.dp_cursor, ga);
        if (o + gbytes <= (unsigned long long)b.dp_cap) {
            *off = o;
            return 2 | 4;
        }
    }
    if (!cbytes) return 0;
    if (slot_ok && (int64_t)cbytes <= b.dp_slot_bytes) return 1;
    const unsigned long long o = atomicAdd(b.dp_cursor, (unsigned long long)((cbytes + 255) & ~(size_t)255));
    if (o + cbytes <= (unsigned long long)b.dp_cap) {
        *off = o;
        return 2;
    }
    return 3;
}

__device__ __forceinline__ uint32_t* wave_scratch_ptr(const BatchDev& b, uint32_t code, int slot,
                                                      unsigned long long off)
{
    if ((code & 3u) == 1u) return reinterpret_cast<uint32_t*>(b.dp_slots + (size_t)slot * b.dp_slot_bytes);
    if ((code & 3u) == 2u) return reinterpret_cast<uint32_t*>(b.dp_arena + off);
    return nullptr;
}

// Counting-sort placement of a work list by key (the chain kernel built the
// key histogram): bucket starts by a block scan of the counters, then one
// atomic per run of equal keys in a warp.  Cursors follow the counters.
constexpr int kKeyScatterThreads = 256;
__global__ void __launch_bounds__(kKeyScatterThreads)
    key_scatter_kernel(const uint32_t* list, const uint32_t* keys, uint32_t* hist, uint32_t* sorted,
                       const unsigned* n_list, int64_t wcap, int bins)
{
    __shared__ uint32_t start[kThinBins];
    __shared__ uint32_t part[kKeyScatterThreads];
    const int per = (bins + kKeyScatterThreads - 1) / kKeyScatterThreads;
    uint32_t s = 0;
    for (int k = 0; k < per; ++k) {
        const int i = threadIdx.x * per + k;
        if (i < bins) s += hist[i];
    }
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < kKeyScatterThreads; o <<= 1) {
        const uint32_t v = (int)threadIdx.x >= o ? part[threadIdx.x - o] : 0u;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t run = part[threadIdx.x] - s;
    for (int k = 0; k < per; ++k) {
        const int i = threadIdx.x * per + k;
        if (i < bins) start[i] = run, run += hist[i];
    }
    __syncthreads();
    const unsigned total = *n_list;
    const unsigned span = (total + 31u) & ~31u;
    for (unsigned w = blockIdx.x * blockDim.x + threadIdx.x; w < span; w += gridDim.x * blockDim.x) {
        const bool act = w < total && (int64_t)w < wcap;
        const uint32_t key = act ? keys[w] : 0xffffffffu;
        const unsigned peers = __match_any_sync(0xffffffffu, key);
        const int leader = __ffs(peers) - 1;
        uint32_t base = 0;
        if (act && (int)(threadIdx.x & 31) == leader) base = atomicAdd(&hist[bins + key], __popc(peers));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (act) sorted[start[key] + base + __popc(peers & ((1u << (threadIdx.x & 31)) - 1u))] = list[w];
    }
}

// One-warp wavefront tier: 4 independent warps per CTA.
__global__ void __launch_bounds__(128, 4) dp_wave_kernel(IndexDev ix, BatchDev b)
{
    __shared__ uint32_t dirs[4][kWaveWarpDirWords];
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    const int gw = blockIdx.x * 4 + wl;
    const unsigned total = min(*b.n_wave, (unsigned)b.wcap);
    for (;;) {
        unsigned wi = 0;
        if (lane == 0) wi = atomicAdd(&b.queues[6], 1u);
        wi = __shfl_sync(FULL, wi, 0);
        if (wi >= total) break;
        const uint32_t sid = b.work_wave_sorted[wi];
        const Seg g = b.seg[sid];
        const int inner = (int)min(g.rl, g.ql), outer = (int)max(g.rl, g.ql);
        const int P = wave_warp_cols(inner);
        const WaveGeom G = wave_geom(inner, outer, P, kWaveWarpDirWords);
        unsigned long long off = 0;
        uint32_t code = 0;
        if (lane == 0) code = wave_scratch_plan(b, G, gw, &off);
        code = __shfl_sync(FULL, code, 0);
        off = __shfl_sync(FULL, off, 0);
        if (code == 3u) {
            if (lane == 0) {
                atomicOr(&b.status[g.q], kStArenaOverflow);
                b.seg[sid].nops = 0;
            }
            continue;
        }
        wave_dispatch<1>(ix, b, sid, g, P, dirs[wl], kWaveWarpDirWords, nullptr, wave_scratch_ptr(b, code, gw, off),
                         (code & 4u) != 0, nullptr);
    }
}

// CTA wavefront tier: one 16-warp CTA per segment (shorter side 257..4096);
// CTA i uses checkpoint slot dp_nslots - gridDim.x + i.
__global__ void __launch_bounds__(kWaveCtaWarps * 32, 1) dp_wave_cta_kernel(IndexDev ix, BatchDev b)
{
    extern __shared__ uint32_t wsm[];
    uint32_t* dirs = wsm;
    uint32_t* ring = wsm + kWaveCtaDirWords;
    __shared__ unsigned s_item;
    __shared__ int s_flag;
    __shared__ uint32_t s_code;
    __shared__ unsigned long long s_off;
    const unsigned total = min(*b.n_wide, (unsigned)b.wcap);
    const int slot = b.dp_nslots - (int)gridDim.x + (int)blockIdx.x;
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(&b.queues[7], 1u);
        __syncthreads();
        const unsigned wi = s_item;
        __syncthreads();
        if (wi >= total) break;
        const uint32_t sid = b.work_wide[wi];
        const Seg g = b.seg[sid];
        const int inner = (int)min(g.rl, g.ql), outer = (int)max(g.rl, g.ql);
        const int P = wave_cta_cols(inner);
        const WaveGeom G = wave_geom(inner, outer, P, kWaveCtaDirWords);
        if (threadIdx.x == 0) {
            unsigned long long off = 0;
            s_code = wave_scratch_plan(b, G, slot, &off);
            s_off = off;
            if (s_code == 3u) {
                atomicOr(&b.status[g.q], kStArenaOverflow);
                b.seg[sid].nops = 0;
            }
        }
        __syncthreads();
        const uint32_t code = s_code;
        const unsigned long long off = s_off;
        __syncthreads();
        if (code == 3u) continue;
        wave_dispatch<kWaveCtaWarps>(ix, b, sid, g, P, dirs, kWaveCtaDirWords, ring,
                                     wave_scratch_ptr(b, code, slot, off), (code & 4u) != 0, &s_flag);
    }
}

constexpr size_t kWaveCtaSmemBytes = sizeof(uint32_t) * ((size_t)kWaveCtaDirWords + (size_t)kWaveCtaWarps * kWaveRing);

__device__ const int8_t c_dna5_mat[25] = {5, -4, -4, -4, 0, -4, 5, -4, -4, 0, -4, -4, 5, -4, 0,
                                          -4, -4, -4, 5, 0, 0, 0, 0, 0, 0};

// Large tier of the batch: one warp per segment from the work list.
__global__ void __launch_bounds__(128) dp_large_kernel(IndexDev ix, BatchDev b)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int gw = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const unsigned total = *b.n_large;
    for (;;) {
        unsigned wi = 0;
        if (lane == 0) wi = atomicAdd(&b.queues[3], 1u);
        wi = __shfl_sync(FULL, wi, 0);
        if (wi >= total) break;
        const uint32_t sid = b.work_large[wi];
        const Seg g = b.seg[sid];
        const bool global = (g.kind & 0xffu) == kSegGlobal;
        KswArgs a;
        a.qlen = (int)g.ql, a.tlen = (int)g.rl;
        a.query = nullptr;
        a.target = ix.center + g.rs;
        a.pk = b.packed + b.poff[g.q];
        a.exc = b.exc;
        a.e0 = b.exc_off[g.q], a.e1 = b.exc_off[g.q + 1];
        a.qoff = g.qs;
        a.m = 5, a.mat = c_dna5_mat, a.q = 6, a.e = 2;
        a.w = auto_band((int)g.rl, (int)g.ql);
        a.zdrop = -1, a.end_bonus = 0;
        // the left end uses left-aligned gaps; the exact max is only needed
        // when a chainless global alignment stops at the band edge
        a.flag = kEzGenericSc | ((g.kind & kSegLeft) ? 0 : kEzRight) | (global ? 0 : kEzApproxMax);
        const size_t need = ksw_scratch_bytes(a.qlen, a.tlen, a.w, a.flag);
        uint8_t* scratch;
        if ((int64_t)need <= b.dp_slot_bytes && gw < b.dp_nslots) {
            scratch = b.dp_slots + (size_t)gw * b.dp_slot_bytes;  // this warp's reusable slot
        } else {
            unsigned long long off = 0;
            if (lane == 0) {
                off = atomicAdd(b.dp_cursor, (unsigned long long)((need + 255) & ~(size_t)255));
                if ((int64_t)(off + need) > b.dp_cap) off = ~0ull;
            }
            off = __shfl_sync(FULL, off, 0);
            if (off == ~0ull) {
                if (lane == 0) {
                    atomicOr(&b.status[g.q], kStArenaOverflow);
                    b.seg[sid].nops = 0;
                }
                continue;
            }
            scratch = b.dp_arena + off;
        }
        uint32_t* out = b.cig_seg + b.coff[g.q] + g.slot;
        const KswResult R = ksw_extz2_warp(a, scratch, out, (int)(g.rl + g.ql));
        if (lane == 0 && b.cells) atomicAdd(b.cells, (unsigned long long)R.cells);
        if (lane == 0) {
            if (global) {
                b.seg[sid].nops = R.n_cigar;
                if (R.zdropped) atomicOr(&b.status[g.q], kStPartialCigar);
            } else {
                // a segment whose CIGAR does not consume it becomes I(q) D(t)
                // (src/align/align.cpp:243-261); only a band stop can cause it
                b.seg[sid].nops = R.zdropped ? -1 : R.n_cigar;
            }
        }
    }
}

// Single-call ksw_extz2 entry point: one warp.
__global__ void ksw_single_kernel(KswArgs a, uint8_t* scratch, uint32_t* cig, int cap, KswResult* res)
{
    if (threadIdx.x >= 32) return;
    const KswResult R = ksw_extz2_warp(a, scratch, cig, cap);
    if (threadIdx.x == 0) *res = R;
}

}  // namespace hg

extern "C" cudaError_t hg_launch_dp_small(const hg::IndexDev* ix, const hg::BatchDev* b, int grid, cudaStream_t st)
{
    hg::shape_hist_kernel<<<grid / 4 > 0 ? grid / 4 : 1, hg::kShapeHistThreads, 0, st>>>(*b);
    hg::shape_scan_kernel<<<1, 1024, 0, st>>>(*b);
    hg::shape_scatter_kernel<<<grid / 4 > 0 ? grid / 4 : 1, hg::kScatterThreads, hg::kScatterSmem, st>>>(*ix, *b);
    if (b->small_pair)  // half the threads per CTA of the single-record form, twice the CTAs
        hg::dp_small_pair_kernel<<<2 * grid, hg::kDpSmallPairThreads, 0, st>>>(*ix, *b);
    else
        hg::dp_small_kernel<<<grid, hg::kDpSmallThreads, 0, st>>>(*ix, *b);
    hg::dp_medium_kernel<<<grid, hg::kDpMedThreads, 0, st>>>(*ix, *b);
    return cudaGetLastError();
}

extern "C" cudaError_t hg_launch_dp_large(const hg::IndexDev* ix, const hg::BatchDev* b, int grid, cudaStream_t st)
{
    hg::dp_large_kernel<<<grid, 128, 0, st>>>(*ix, *b);
    return cudaGetLastError();
}

// Thin tier: sort, then one warp per thin scratch region.
extern "C" cudaError_t hg_launch_dp_thin(const hg::IndexDev* ix, const hg::BatchDev* b, int grid, cudaStream_t st)
{
    hg::key_scatter_kernel<<<grid, hg::kKeyScatterThreads, 0, st>>>(b->work_thin, b->work_thin_key, b->thin_hist,
                                                                    b->work_thin_sorted, b->n_thin, b->wcap,
                                                                    hg::kThinBins);
    const int tgrid = (b->thin_nwarps + hg::kThinWarps - 1) / hg::kThinWarps;
    hg::dp_thin_kernel<<<tgrid, hg::kThinWarps * 32, hg::kThinSmemBytes, st>>>(*ix, *b);
    return cudaGetLastError();
}

// Square tier (sort, then grid CTAs of 4 warps; warp i uses slot i), then the
// one-warp wavefront tier (sort, then grid CTAs of 4 warps; warp i uses slot
// i): one after the other on one stream, as they share the slots.
extern "C" cudaError_t hg_launch_dp_wave(const hg::IndexDev* ix, const hg::BatchDev* b, int grid, cudaStream_t st)
{
    hg::key_scatter_kernel<<<grid, hg::kKeyScatterThreads, 0, st>>>(b->work_sq, b->work_sq_key, b->sq_hist,
                                                                    b->work_sq_sorted, b->n_sq, b->wcap,
                                                                    hg::kSquareBins);
    hg::dp_square_kernel<<<grid, hg::kSquareWarps * 32, hg::kSquareSmemBytes, st>>>(*ix, *b);
    hg::key_scatter_kernel<<<grid, hg::kKeyScatterThreads, 0, st>>>(b->work_wave, b->work_wave_key, b->wave_hist,
                                                                    b->work_wave_sorted, b->n_wave, b->wcap,
                                                                    hg::kWaveBins);
    hg::dp_wave_kernel<<<grid, 128, 0, st>>>(*ix, *b);
    return cudaGetLastError();
}

// CTA wavefront tier: grid CTAs (at most one per SM); CTA i uses checkpoint
// slot dp_nslots - grid + i, above every slot the warp tiers use, so it may
// run concurrently with them.
extern "C" cudaError_t hg_launch_dp_wide(const hg::IndexDev* ix, const hg::BatchDev* b, int grid, cudaStream_t st)
{
    hg::dp_wave_cta_kernel<<<grid, hg::kWaveCtaWarps * 32, hg::kWaveCtaSmemBytes, st>>>(*ix, *b);
    return cudaGetLastError();
}

extern "C" cudaError_t hg_prepare_dp_kernels()
{
    cudaError_t e = cudaFuncSetAttribute(hg::dp_wave_cta_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)hg::kWaveCtaSmemBytes);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(hg::dp_thin_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)hg::kThinSmemBytes);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(hg::dp_square_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)hg::kSquareSmemBytes);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(hg::shape_scatter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)hg::kScatterSmem);
}

extern "C" size_t hg_ksw_scratch_bytes(int qlen, int tlen, int w, int flag)
{
    return hg::ksw_scratch_bytes(qlen, tlen, w, flag);
}

extern "C" cudaError_t hg_launch_ksw_single(int qlen, const uint8_t* d_query, int tlen, const uint8_t* d_target, int m,
                                            const int8_t* d_mat, int q, int e, int w, int zdrop, int end_bonus,
                                            int flag, uint8_t* d_scratch, uint32_t* d_cig, int cap, void* d_res,
                                            cudaStream_t st)
{
    hg::KswArgs a{};
    a.qlen = qlen, a.tlen = tlen, a.query = d_query, a.target = d_target;
    a.m = m, a.mat = d_mat, a.q = q, a.e = e, a.w = w, a.zdrop = zdrop, a.end_bonus = end_bonus, a.flag = flag;
    hg::ksw_single_kernel<<<1, 32, 0, st>>>(a, d_scratch, d_cig, cap, static_cast<hg::KswResult*>(d_res));
    return cudaGetLastError();
}

// ------------------------------------------------------------------------
// Allocation-free ksw_extz2 for callers that cannot allocate device memory.
//
// Some callers must not allocate: code whose device memory is owned by a
// pool or caching allocator that has to account for every byte, and
// latency-sensitive loops that cannot afford the device-wide
// synchronisation cudaFree implies.  hg_ksw_extz2 allocates its scratch per
// call, so those callers use this entry point instead: the caller passes
// device buffers for the inputs and the outputs, and the DP scratch is a
// fixed array compiled into this library.
//
// Limits and sharing rules:
//   * the scratch is kNoAllocScratchBytes (1 MiB) per GPU; every GPU that
//     loads the library keeps it until the process exits;
//   * a call whose DP needs more scratch (hg_ksw_scratch_bytes) is rejected
//     with HG_ERR_CAPACITY before anything is launched;
//   * every call on a GPU uses the same array.  The kernel clears the parts
//     that must start at zero itself, so a call never sees the previous
//     call's data, but two calls that can overlap on the GPU (different
//     streams, or different host threads) race on the array: serialise them.
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) with that device current; make that first call
//     before any stream capture.  The address is kept per device ordinal for
//     the process's primary context: it is not valid in another driver
//     context of that device, nor after cudaDeviceReset.
constexpr size_t kNoAllocScratchBytes = (size_t)1 << 20;
static_assert(kNoAllocScratchBytes == HG_NOALLOC_SCRATCH_BYTES, "scratch size and its public limit disagree");
static __device__ __align__(256) uint8_t g_noalloc_scratch[kNoAllocScratchBytes];

namespace hg {
__global__ void ksw_noalloc_kernel(KswArgs a, uint8_t* scratch, uint32_t* cig, int cap, int32_t* res)
{
    if (threadIdx.x >= 32) return;
    // The sequences are device memory, so the host cannot check them: a
    // symbol >= m would index past the m x m matrix.  Such a call computes
    // nothing, leaves the CIGAR buffer untouched and reports length -1.
    bool bad = false;
    for (int i = threadIdx.x; i < a.qlen; i += 32) bad |= a.query[i] >= a.m;
    for (int i = threadIdx.x; i < a.tlen; i += 32) bad |= a.target[i] >= a.m;
    if (__any_sync(0xffffffffu, bad)) {
        if (threadIdx.x == 0) {
            res[0] = 0, res[1] = 0, res[2] = -1, res[3] = -1, res[4] = kNegInf;
            res[5] = -1, res[6] = kNegInf, res[7] = -1, res[8] = kNegInf, res[9] = 0;
            res[10] = -1;
        }
        return;
    }
    const KswResult R = ksw_extz2_warp(a, scratch, cig, cap);
    if (threadIdx.x == 0) {
        res[0] = R.max, res[1] = R.zdropped, res[2] = R.max_q, res[3] = R.max_t, res[4] = R.mqe;
        res[5] = R.mqe_t, res[6] = R.mte, res[7] = R.mte_q, res[8] = R.score, res[9] = R.reach_end;
        res[10] = R.n_cigar;
    }
}
}  // namespace hg

namespace {
constexpr int kMaxNoAllocDevices = 64;
uint8_t* g_noalloc_ptr[kMaxNoAllocDevices] = {};
std::mutex g_noalloc_mu;

int noalloc_fail(char* err, int64_t err_cap, int code, const char* fmt, size_t a = 0, size_t b = 0)
{
    if (err && err_cap > 0) std::snprintf(err, (size_t)err_cap, fmt, a, b);
    return code;
}
}  // namespace

extern "C" int hg_ksw_extz2_noalloc(int qlen, const uint8_t* d_query, int tlen, const uint8_t* d_target, int8_t m,
                                    const int8_t* d_mat, int8_t q, int8_t e, int w, int zdrop, int end_bonus,
                                    int flag, int32_t* d_ez, uint32_t* d_cigar, int64_t cap, void* stream,
                                    char* err, int64_t err_cap)
{
    if (err && err_cap > 0) err[0] = 0;
    if (m <= 0 || m > 16 || !d_mat || !d_ez || (qlen > 0 && !d_query) ||
        (tlen > 0 && !d_target) || cap < 0 || cap > INT32_MAX || (cap > 0 && !d_cigar))
        return noalloc_fail(err, err_cap, 2, "hg_ksw_extz2_noalloc: bad arguments");  // HG_ERR_ARG
    const size_t need = hg_ksw_scratch_bytes(qlen, tlen, w, flag);
    if (need > kNoAllocScratchBytes)
        return noalloc_fail(err, err_cap, 4,  // HG_ERR_CAPACITY
                            "hg_ksw_extz2_noalloc: this alignment needs %zu scratch bytes, above the %zu-byte "
                            "static limit; use hg_ksw_extz2",
                            need, kNoAllocScratchBytes);
    int dev = 0;
    cudaError_t ce = cudaGetDevice(&dev);
    if (ce != cudaSuccess || dev < 0 || dev >= kMaxNoAllocDevices)
        return noalloc_fail(err, err_cap, 1, "hg_ksw_extz2_noalloc: no usable CUDA device");  // HG_ERR_CUDA
    uint8_t* scratch;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!g_noalloc_ptr[dev]) {
            void* p = nullptr;
            ce = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (ce != cudaSuccess || !p)
                return noalloc_fail(err, err_cap, 1, "hg_ksw_extz2_noalloc: cudaGetSymbolAddress failed");
            g_noalloc_ptr[dev] = static_cast<uint8_t*>(p);
        }
        scratch = g_noalloc_ptr[dev];
    }
    hg::KswArgs a{};
    a.qlen = qlen, a.tlen = tlen, a.query = d_query, a.target = d_target;
    a.m = m, a.mat = d_mat, a.q = q, a.e = e, a.w = w, a.zdrop = zdrop, a.end_bonus = end_bonus, a.flag = flag;
    hg::ksw_noalloc_kernel<<<1, 32, 0, static_cast<cudaStream_t>(stream)>>>(a, scratch, d_cigar, (int)cap, d_ez);
    if (cudaGetLastError() != cudaSuccess) return noalloc_fail(err, err_cap, 1, "hg_ksw_extz2_noalloc: launch failed");
    return 0;
}

// ------------------------------------------------------------------------
// Self-test of the packed cell: lane16x2 against lane_int_z over every input
// the band-free tiers can feed a cell (z0 in {12, 16, 21}, x and y of the
// neighbours in [0, 6], u and v in [0, 21]), both gap modes, each input in
// the low half paired with another input in the high half.  Returns the
// number of disagreeing (input, half) cases.
namespace hg {
__global__ void lane16x2_selftest_kernel(unsigned* bad)
{
    constexpr int NZ = 3, NX = 7, NV = 22;
    const int total = NZ * NX * NV * NV * NX;
    const int zs[NZ] = {12, 16, 21};
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < 2 * total; idx += gridDim.x * blockDim.x) {
        const int mode = idx >= total ? 2 : 1;
        int k = idx % total;
        const int lo[5] = {zs[k % NZ], (k / NZ) % NX, (k / (NZ * NX)) % NV, (k / (NZ * NX * NV)) % NV,
                           (k / (NZ * NX * NV * NV)) % NX};
        k = (k * 7919 + 17) % total;  // another input for the high half
        const int hi[5] = {zs[k % NZ], (k / NZ) % NX, (k / (NZ * NX)) % NV, (k / (NZ * NX * NV)) % NV,
                           (k / (NZ * NX * NV * NV)) % NX};
        uint32_t pk[5];
        for (int j = 0; j < 5; ++j) pk[j] = (uint32_t)(lo[j] + (int)kPB) | (uint32_t)(hi[j] + (int)kPB) << 16;
        uint32_t u2, v2, x2, y2;
        const uint32_t d2 = mode == 1 ? lane16x2<1>(pk[0], pk[1], pk[2], pk[3], pk[4], u2, v2, x2, y2)
                                      : lane16x2<2>(pk[0], pk[1], pk[2], pk[3], pk[4], u2, v2, x2, y2);
        for (int h = 0; h < 2; ++h) {
            const int* in = h ? hi : lo;
            int u, v, x, y;
            const uint32_t d = mode == 1 ? lane_int_z<1>(in[0], in[1], in[2], in[3], in[4], u, v, x, y)
                                         : lane_int_z<2>(in[0], in[1], in[2], in[3], in[4], u, v, x, y);
            const int sh = 16 * h;
            auto val = [&](uint32_t w) { return (int)((w >> sh) & 0xffffu) - (int)kPB; };
            const bool ok = ((d2 >> sh) & 0xfu) == d && val(u2) == u && val(v2) == v && val(x2) == x &&
                            val(y2) == y;
            if (!ok) atomicAdd(bad, 1u);
        }
    }
}
}  // namespace hg

extern "C" int hg_dp_lane_selftest(uint32_t* mismatches)
{
    if (!mismatches) return hg::set_error(HG_ERR_ARG, "hg_dp_lane_selftest: bad arguments");
    unsigned* d = nullptr;
    HG_CUDA(cudaMalloc(&d, sizeof(unsigned)));
    cudaMemset(d, 0, sizeof(unsigned));
    hg::lane16x2_selftest_kernel<<<304, 256>>>(d);
    const cudaError_t e = cudaMemcpy(mismatches, d, sizeof(unsigned), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return hg::cuda_error(e, "hg_dp_lane_selftest");
    return HG_OK;
}
