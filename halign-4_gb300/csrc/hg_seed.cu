// hg_seed.cu - K1: minimizer extraction + center-index lookup.
//
// Restates minimizer::extractMinimizer (src/seed/minimizer.cpp:103-177) as a
// data-parallel tile computation.  For k-mer start p the reference emits
//   m(p) = argmin h(q) over the valid k-mers q in [p-win+1, p] that share p's
//          N-free run, ties to the largest q ("latest equal hash wins"),
// at every p with a valid k-mer and p+1 >= win, whenever m(p) differs from
// what it emitted at p-1 (an N clears that memory).  m(p) is monotone inside
// a run, so the emitted list is the de-duplicated m(p) sequence in scan order.
//
// One CTA owns one query at a time (persistent, queue ordered longest first)
// and sweeps it in tiles of kSeedTile k-mer positions:
//   1. stream the packed bases of the tile (+ halo) with aligned uint4 loads,
//      overlay exception bytes (N, U, lowercase ...), decode to nt4 codes;
//   2. hash every k-mer (splitmix64 of the 2-bit forward code, >> 8);
//   3. window minimum per position, emission flags;
//   4. block-scan compaction in position order; matched hits (hash present in
//      the resident center index) go to the hit arena, all hits are counted
//      (the q_occ limit of collect_anchors uses |query hits|).
//
// Deque overflow.  RingMinQueue (src/seed/minimizer.cpp:35-97) has capacity
// win and pushes before it expires old entries, so when w+1 consecutive
// valid k-mers have strictly increasing hashes the push lands on the front
// slot and the queue keeps that corrupted state for a while.  The tile pass
// detects the first such position (the only way the queue can be full) and
// queues the whole query for seed_exact_kernel, which replays the reference's
// ring buffer sequentially (one warp per query, the ring walk on one lane)
// and overwrites the tile pass's output for that query.
#include <type_traits>

#include "hg_batch.cuh"

namespace hg {

constexpr int kSeedThreads = 256;
constexpr int kSeedPer = 8;
constexpr int kSeedTile = kSeedThreads * kSeedPer;  // k-mer positions per tile
constexpr int kMaxWin = 255;
constexpr int kMaxK = 31;
constexpr int kCodeBuf = kSeedTile + 512;
constexpr int kHashBuf = kSeedTile + kMaxWin + 1;

struct SeedOut {
    int mode;        // 0: matched hits (pos, entry); 1: every hit as MinimizerHit words
    uint64_t* hx;    // mode 1: x = hash56 << 8 | span
    uint64_t* hy;    // mode 1: y = strand << 63 | rid << 32 | pos
};

// Fast path for a query without exception bytes at window 10 and k <= 24
// (the align-to-center defaults).  Thread t of a tile owns k-mer starts
// P0 = tile + 8t .. P0+7:
//   * the 2-bit forward codes come from one 64-bit packed word: bit-reversed
//     and pair-swapped it holds base P0 in its top two bits, so the k-mer at
//     P0+i is (X << 2i) >> (64 - 2k);
//   * window minimum in registers over 64-bit keys (hash << 8 | 254 - idx):
//     key order is hash order with ties to the later position, so "latest
//     equal hash wins" is a plain minimum; pairs -> quads -> octets, and a
//     window of 10 is an octet plus a pair (the 16 hashes before P0 come
//     from shared memory);
//   * the deque-overflow test (10 strict increases ending at a position) is
//     a run of ten ones in the increase bitmask.
constexpr int kFastWin = 10;
constexpr int kFastMaxK = 24;

__device__ __forceinline__ uint64_t umin64(uint64_t a, uint64_t b) { return a < b ? a : b; }

__device__ __forceinline__ bool seed_fast_eligible(const IndexDev& ix, int len, int64_t e0, int64_t e1)
{
    return e0 == e1 && ix.non_canonical && ix.w == kFastWin && ix.k > 0 && ix.k <= kFastMaxK &&
           len - ix.k + 1 >= kFastWin;
}

constexpr int kSeedFastWarps = 8;
constexpr int kSeedFastChunk = 32 * kSeedPer;  // k-mer starts per warp step

// One warp per query (no block barriers); each warp's shared buffer holds
// the hashes of its current chunk after the 16 that precede it.
__global__ void __launch_bounds__(kSeedFastWarps * 32, 3) seed_fast_kernel(IndexDev ix, BatchDev b)
{
    // the hashes of a warp's chunk after the 16 before it; element idx lives at
    // idx + idx / 8 (one pad word per 8) so that lane l's 8 consecutive
    // elements start 72 bytes after lane l-1's: no bank conflicts
    __shared__ uint64_t hbuf[kSeedFastWarps][(16 + kSeedFastChunk) * 9 / 8];
    __shared__ uint64_t ebuf[kSeedFastWarps][kSeedFastChunk];
    __shared__ uint32_t pbuf[kSeedFastWarps][kSeedFastChunk];
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    uint64_t* hsb = hbuf[threadIdx.x >> 5];
    auto H = [hsb](int idx) -> uint64_t& { return hsb[idx + (idx >> 3)]; };
    uint32_t* ps = pbuf[threadIdx.x >> 5];
    uint64_t* es = ebuf[threadIdx.x >> 5];
    const int k = ix.k;
    const int lsh = 64 - 2 * k;
    for (;;) {
        int qi = 0;
        if (lane == 0) qi = (int)atomicAdd(&b.queues2[0], 1u);
        qi = __shfl_sync(FULL, qi, 0);
        if (qi >= b.n) break;
        const int q = b.order ? b.order[qi] : qi;
        const int len = b.qlen[q];
        if (!seed_fast_eligible(ix, len, b.exc_off[q], b.exc_off[q + 1])) continue;
        const uint8_t* pk = b.packed + b.poff[q];
        const int nk = len - k + 1;
        const int64_t hb = b.hoff[q];
        if (lane < 16) H(lane) = kNoHash;  // positions before 0
        int total_hits = 0, total_matched = 0;
        bool ovf_any = false;
        // EDGE: a chunk touching position 0 or the query end (hashes past either
        // end are kNoHash); interior chunks skip those tests
        auto chunk = [&](auto edge_tag, const int t0) {
            constexpr bool EDGE = decltype(edge_tag)::value;
            const int P0 = t0 + lane * kSeedPer;
            uint64_t h[kSeedPer];
            if (!EDGE || P0 < nk) {
                const uint32_t wb = ((uint32_t)P0 >> 2) & ~7u;
                const uint64_t* w = reinterpret_cast<const uint64_t*>(pk + wb);
                const uint64_t w0 = w[0], w1 = w[1];
                const uint32_t sh = 2u * ((uint32_t)P0 - wb * 4u);
                const uint64_t lo = sh ? (w0 >> sh) | (w1 << (64u - sh)) : w0;
                uint64_t x = __brevll(lo);
                x = ((x >> 1) & 0x5555555555555555ULL) | ((x & 0x5555555555555555ULL) << 1);
#pragma unroll
                for (int i = 0; i < kSeedPer; ++i)
                    h[i] = (!EDGE || P0 + i < nk) ? splitmix64((x << (2 * i)) >> lsh) >> 8 : kNoHash;
            } else {
#pragma unroll
                for (int i = 0; i < kSeedPer; ++i) h[i] = kNoHash;
            }
#pragma unroll
            for (int i = 0; i < kSeedPer; ++i) H(16 + lane * kSeedPer + i) = h[i];
            __syncwarp();
            // the hashes of P0-16 .. P0+7 are A(i) = H(lane * kSeedPer + i), i < 24
            auto A = [&](int i) -> uint64_t { return H(lane * kSeedPer + i); };
            // window minimum on 32-bit keys: the top 26 bits of the 56-bit hash
            // above a 5-bit index, once with ties to the later index (A, the
            // reference's "latest equal wins") and once to the earlier (B).
            // Where the two disagree, two k-mers of the window share the 26-bit
            // prefix (or the window has no k-mer) and the exact 64-bit minimum
            // over keys hash << 8 | (254 - idx) decides.  Valid prefixes are
            // < 2^31, so kNoHash (key 0xffffffff) loses to every k-mer.
            uint32_t tp[24], kA[24], kB[24];  // tp = 0xffffffff exactly for kNoHash
#pragma unroll
            for (int i = 6; i < 24; ++i) {
                tp[i] = (uint32_t)((i < 16 ? A(i) : h[i - 16]) >> 25);
                const bool nh = EDGE && tp[i] == ~0u;
                kA[i] = nh ? ~0u : (tp[i] & ~31u) | (uint32_t)(31 - i);
                kB[i] = nh ? ~0u : (tp[i] & ~31u) | (uint32_t)i;
            }
            uint32_t PA[24], QA[24], OA[24], PB[24], QB[24], OB[24];
#pragma unroll
            for (int i = 7; i < 24; ++i) PA[i] = min(kA[i - 1], kA[i]), PB[i] = min(kB[i - 1], kB[i]);
#pragma unroll
            for (int i = 9; i < 24; ++i) QA[i] = min(PA[i], PA[i - 2]), QB[i] = min(PB[i], PB[i - 2]);
#pragma unroll
            for (int i = 13; i < 24; ++i) OA[i] = min(QA[i], QA[i - 4]), OB[i] = min(QB[i], QB[i - 4]);
            int mi[kSeedPer + 1];  // minimizer of P0-1 .. P0+7 as an index into A (position P0 - 16 + index)
#pragma unroll
            for (int e = 15; e < 24; ++e) {
                const uint32_t mA = min(OA[e], PA[e - 8]), mB = min(OB[e], PB[e - 8]);
                int idx = 31 - (int)(mA & 31u);
                if (idx != (int)(mB & 31u)) {
                    uint64_t best = ~0ull;
#pragma unroll
                    for (int j = e - 9; j <= e; ++j)
                        best = umin64(best, (EDGE && A(j) == kNoHash) ? ~0ull : (A(j) << 8) | (uint64_t)(254 - j));
                    idx = 254 - (int)(best & 0xffu);
                }
                mi[e - 15] = idx;
            }
            // deque overflow: 10 strict increases ending at P0 + i (P0 + i - 10 >= 0,
            // P0 + i < nk); equal prefixes compare the whole hashes
            uint32_t inc = 0, tie = 0;
#pragma unroll
            for (int i = 7; i < 24; ++i) {
                const bool ok = !EDGE || (tp[i - 1] != ~0u && tp[i] != ~0u);
                inc |= (ok && tp[i - 1] < tp[i]) ? (1u << i) : 0u;
                tie |= (ok && tp[i - 1] == tp[i]) ? (1u << i) : 0u;
            }
            if (tie) {
#pragma unroll
                for (int i = 7; i < 24; ++i)
                    if ((tie >> i & 1u) && A(i - 1) < A(i)) inc |= 1u << i;
            }
            const uint32_t r2 = inc & (inc >> 1), r4 = r2 & (r2 >> 2), r8 = r4 & (r4 >> 4), r10 = r8 & (r2 >> 8);
            const uint32_t ovf = (r10 >> 7) & 0xffu;  // run of ten starting at bit 7+i ends at bit 16+i
            // emission; the chunk's emitted minimizers (hash read back from the
            // warp's buffer) are compacted in position order, then probed in the
            // index densely, one per lane
            uint32_t emask = 0;
#pragma unroll
            for (int i = 0; i < kSeedPer; ++i) {
                const int p = P0 + i;
                if (((ovf >> i) & 1u) && (!EDGE || (p - kFastWin >= 0 && p < nk))) ovf_any = true;
                if (EDGE && (p >= nk || p < kFastWin - 1)) continue;
                if ((!EDGE || p > kFastWin - 1) && mi[i + 1] == mi[i]) continue;
                emask |= 1u << i;
            }
            const int n_emit = __popc(emask);
            const int eincl = warp_incl_sum(n_emit);
            const int n_chunk = __shfl_sync(FULL, eincl, 31);
            int e = eincl - n_emit;
#pragma unroll
            for (int i = 0; i < kSeedPer; ++i) {
                if (emask >> i & 1u) {
                    es[e] = H(lane * kSeedPer + mi[i + 1]);
                    ps[e] = (uint32_t)(P0 - 16 + mi[i + 1]);
                    ++e;
                }
            }
            __syncwarp();
            if (lane < 16) H(lane) = H(kSeedFastChunk + lane);  // carry the last 16 hashes
            __syncwarp();
            for (int e0 = 0; e0 < n_chunk; e0 += 32) {
                const int ei = e0 + lane;
                const uint32_t ent = ei < n_chunk ? index_find(ix, es[ei]) : kEmptyKey;
                const bool hit = ent != kEmptyKey;
                const unsigned hm = __ballot_sync(FULL, hit);
                if (hit) {
                    const int o = total_matched + __popc(hm & ((1u << lane) - 1u));
                    b.hit_pos[hb + o] = ps[ei];
                    b.hit_ent[hb + o] = ent;
                }
                total_matched += __popc(hm);
            }
            __syncwarp();
            total_hits += n_chunk;
        };
        for (int t0 = 0; t0 < nk; t0 += kSeedFastChunk) {
            if (t0 > 0 && t0 + kSeedFastChunk <= nk) chunk(std::false_type{}, t0);
            else chunk(std::true_type{}, t0);
        }
        const bool ovf_q = __any_sync(FULL, ovf_any);
        if (lane == 0) {
            b.n_hits[q] = total_hits;
            b.n_matched[q] = total_matched;
            if (ovf_q) b.exact_list[atomicAdd(b.n_exact, 1u)] = (uint32_t)q;
        }
        __syncwarp();
    }
}

__global__ void __launch_bounds__(kSeedThreads) seed_kernel(IndexDev ix, BatchDev b, SeedOut so)
{
    __shared__ __align__(16) uint8_t codes[kCodeBuf];
    __shared__ uint64_t hsh[kHashBuf];
    __shared__ uint8_t strand[kHashBuf];
    __shared__ int32_t mpos[kSeedTile + 1];
    __shared__ int16_t pre[kHashBuf], suf[kHashBuf];  // block prefix / suffix arg-min (relative to hs)
    __shared__ int scan_s[33];
    __shared__ int s_q, s_ovf;

    const int k = ix.k;
    const uint64_t kmask = (1ULL << (2 * k)) - 1ULL;
    const int kshift = 2 * (k - 1);
    const int tid = threadIdx.x;

    for (;;) {
        if (tid == 0) s_q = (int)atomicAdd(&b.queues[0], 1u), s_ovf = 0;
        __syncthreads();
        const int qi = s_q;
        __syncthreads();
        if (qi >= b.n) break;
        const int q = b.order ? b.order[qi] : qi;
        const int len = b.qlen[q];
        const uint8_t* pk = b.packed + b.poff[q];
        const int64_t e0 = b.exc_off[q], e1 = b.exc_off[q + 1];
        if (so.mode == 0 && seed_fast_eligible(ix, len, e0, e1)) continue;  // seed_fast_kernel's query
        int total_hits = 0, total_matched = 0;
        if (len >= k && k > 0 && k <= kMaxK && ix.w > 0 && ix.w <= kMaxWin) {
            const int nk = len - k + 1;
            const int win = ix.w < nk ? ix.w : nk;
            for (int p0 = 0; p0 < nk; p0 += kSeedTile) {
                const int pend = min(p0 + kSeedTile, nk);
                const int hs = max(p0 - win, 0);           // first hashed position
                const int bstart = hs & ~63;              // 64 bases = one uint4
                const int bend = pend + k - 1;            // one past the last base needed
                const int nvec = (bend - bstart + 63) >> 6;
                // 1. packed bases -> nt4 codes (codes[i] = base bstart + i)
                const uint4* src = reinterpret_cast<const uint4*>(pk + (bstart >> 2));
                for (int v = tid; v < nvec; v += kSeedThreads) {
                    const uint4 word = src[v];
                    const uint32_t wv[4] = {word.x, word.y, word.z, word.w};
                    uint32_t* dst = reinterpret_cast<uint32_t*>(codes + v * 64);
#pragma unroll
                    for (int wi = 0; wi < 4; ++wi) {
#pragma unroll
                        for (int bq = 0; bq < 4; ++bq) {
                            const uint32_t byte = (wv[wi] >> (8 * bq)) & 0xffu;
                            // 4 bases of this byte -> 4 code bytes
                            const uint32_t c4 = (byte & 3u) | ((byte >> 2) & 3u) << 8 | ((byte >> 4) & 3u) << 16 |
                                                ((byte >> 6) & 3u) << 24;
                            dst[wi * 4 + bq] = c4;
                        }
                    }
                }
                __syncthreads();
                // exception bytes overlay (U counts as T for minimizers, N/other invalid)
                for (int64_t e = e0 + tid; e < e1; e += kSeedThreads) {
                    const int s = b.exc[e * 3], l = b.exc[e * 3 + 1];
                    const uint8_t c = nt4_of((uint8_t)b.exc[e * 3 + 2]);
                    const int lo = max(s, bstart), hi = min(s + l, bend);
                    for (int i = lo; i < hi; ++i) codes[i - bstart] = c;
                }
                __syncthreads();
                // 2. hashes for positions [hs, pend)
                for (int base = hs + tid * kSeedPer; base < pend; base += kSeedThreads * kSeedPer) {
                    uint64_t fwd = 0, rev = 0;
                    int last_bad = -1;
                    for (int i = 0; i < k - 1; ++i) {
                        const int pos = base + i;
                        const uint32_t c = codes[pos - bstart];
                        if (c >= 4) last_bad = pos;
                        fwd = ((fwd << 2) | (c & 3u)) & kmask;
                        rev = (rev >> 2) | ((uint64_t)(3u ^ (c & 3u)) << kshift);
                    }
                    const int top = min(base + kSeedPer, pend);
                    for (int p = base; p < top; ++p) {
                        const int pos = p + k - 1;
                        const uint32_t c = codes[pos - bstart];
                        if (c >= 4) last_bad = pos;
                        fwd = ((fwd << 2) | (c & 3u)) & kmask;
                        rev = (rev >> 2) | ((uint64_t)(3u ^ (c & 3u)) << kshift);
                        const bool ok = last_bad < p;
                        const uint64_t code = ix.non_canonical ? fwd : (fwd < rev ? fwd : rev);
                        hsh[p - hs] = ok ? (splitmix64(code) >> 8) : kNoHash;
                        strand[p - hs] = ix.non_canonical ? 1 : (fwd <= rev);
                    }
                }
                __syncthreads();
                // 3. window minimum m(p) for p in [p0-1, pend)
                const int mlo = p0 - 1;
                if (win <= k) {
                    // Between two N-free runs lie >= k invalid k-mers, so a window of
                    // win <= k positions only holds valid k-mers of p's own run and an
                    // invalid k-mer can stand for +infinity (kNoHash > every hash).
                    // Arg-min over [p-win+1, p] from block prefix/suffix minima over
                    // blocks of win positions (ties: the later position).
                    const int b0 = hs / win, b1 = (pend - 1) / win;
                    for (int bb = b0 + tid; bb <= b1; bb += kSeedThreads) {
                        const int lo = max(bb * win, hs), hi = min(bb * win + win, pend);
                        int best = lo;
                        uint64_t bh = hsh[lo - hs];
                        pre[lo - hs] = (int16_t)(lo - hs);
                        for (int x = lo + 1; x < hi; ++x) {
                            const uint64_t h = hsh[x - hs];
                            if (h <= bh) bh = h, best = x;
                            pre[x - hs] = (int16_t)(best - hs);
                        }
                        best = hi - 1;
                        bh = hsh[best - hs];
                        suf[best - hs] = (int16_t)(best - hs);
                        for (int x = hi - 2; x >= lo; --x) {
                            const uint64_t h = hsh[x - hs];
                            if (h < bh) bh = h, best = x;
                            suf[x - hs] = (int16_t)(best - hs);
                        }
                    }
                    __syncthreads();
                    for (int p = max(mlo, 0) + tid; p < pend; p += kSeedThreads) {
                        int best = -1;
                        const uint64_t hp = hsh[p - hs];
                        if (hp != kNoHash) {
                            const int a = max(p - win + 1, 0);
                            const int rp = hs + pre[p - hs];
                            if (a / win == p / win || a < hs) {
                                best = rp;
                            } else {
                                const int ls = hs + suf[a - hs];
                                best = hsh[ls - hs] < hsh[rp - hs] ? ls : rp;
                            }
                            // the queue is full before the push at p when hashes strictly
                            // increase over [p-win, p]; walk back over the increases
                            if (p >= p0 && p - win >= 0) {
                                int x = p;
                                while (x > p - win && hsh[x - 1 - hs] != kNoHash && hsh[x - 1 - hs] < hsh[x - hs]) --x;
                                if (x == p - win) s_ovf = 1;
                            }
                        }
                        mpos[p - mlo] = best;
                    }
                } else {
                    for (int p = max(mlo, 0) + tid; p < pend; p += kSeedThreads) {
                        int best = -1;
                        const uint64_t hp = hsh[p - hs];
                        if (hp != kNoHash) {
                            best = p;
                            uint64_t bh = hp, nxt = hp;
                            bool inc = true;
                            const int lo = max(p - win + 1, 0);
                            for (int qq = p - 1; qq >= lo; --qq) {
                                const uint64_t hq = hsh[qq - hs];
                                if (hq == kNoHash) {
                                    inc = false;
                                    break;
                                }
                                if (hq < bh) bh = hq, best = qq;
                                inc = inc && hq < nxt;
                                nxt = hq;
                            }
                            // full queue before the push at p: hashes strictly increase on [p-win, p]
                            if (p >= p0 && inc && p - win >= 0) {
                                const uint64_t hq = hsh[p - win - hs];
                                if (hq != kNoHash && hq < nxt) s_ovf = 1;
                            }
                        }
                        mpos[p - mlo] = best;
                    }
                }
                __syncthreads();
                // 4. emission + compaction in position order
                const int my0 = p0 + tid * kSeedPer;
                const int my1 = min(my0 + kSeedPer, pend);
                int n_emit = 0, n_match = 0;
                uint32_t ent[kSeedPer];
                uint32_t emitmask = 0;
                for (int p = my0; p < my1; ++p) {
                    const int i = p - my0;
                    ent[i] = kEmptyKey;
                    const int m = mpos[p - mlo];
                    if (m < 0 || p + 1 < win) continue;
                    const bool prev_elig = p >= 1 && (p - 1) + 1 >= win && mpos[p - 1 - mlo] >= 0;
                    if (prev_elig && mpos[p - 1 - mlo] == m) continue;
                    emitmask |= 1u << i;
                    ++n_emit;
                    if (so.mode == 0) {
                        ent[i] = index_find(ix, hsh[m - hs]);
                        if (ent[i] != kEmptyKey) ++n_match;
                    }
                }
                int tot_emit, tot_match;
                const int ex_emit = block_excl_sum(n_emit, scan_s, &tot_emit);
                const int ex_match = so.mode == 0 ? block_excl_sum(n_match, scan_s, &tot_match) : 0;
                if (so.mode == 0) {
                    int o = total_matched + ex_match;
                    const int64_t hb = b.hoff[q];
                    for (int p = my0; p < my1; ++p) {
                        const int i = p - my0;
                        if ((emitmask >> i & 1u) && ent[i] != kEmptyKey) {
                            b.hit_pos[hb + o] = (uint32_t)mpos[p - mlo];
                            b.hit_ent[hb + o] = ent[i];
                            ++o;
                        }
                    }
                    total_matched += tot_match;
                } else {
                    int o = total_hits + ex_emit;
                    const int64_t hb = b.hoff[q];
                    for (int p = my0; p < my1; ++p) {
                        const int i = p - my0;
                        if (emitmask >> i & 1u) {
                            const int m = mpos[p - mlo];
                            so.hx[hb + o] = (hsh[m - hs] << 8) | (uint64_t)(uint8_t)k;
                            so.hy[hb + o] = ((uint64_t)(strand[p - hs] ? 0x80000000u : 0u) << 32) | (uint64_t)(uint32_t)m;
                            ++o;
                        }
                    }
                }
                total_hits += tot_emit;
                __syncthreads();
            }
        }
        __syncthreads();
        if (tid == 0) {
            b.n_hits[q] = total_hits;
            b.n_matched[q] = total_matched;
            if (s_ovf) b.exact_list[atomicAdd(b.n_exact, 1u)] = (uint32_t)q;
        }
    }
}

// Replay of extractMinimizer (src/seed/minimizer.cpp:103-177) for the
// queries whose window deque overflows, with the reference's RingMinQueue
// (src/seed/minimizer.cpp:35-97).  The ring leaves the ideal monotone-deque
// behaviour only when a push finds it full: at a k-mer that ends win + 1
// consecutive strictly increasing hashes of one N-free run.  Before that,
// and again once its logical contents equal the ideal deque's, what it emits
// follows from the hashes alone.  One warp per query, 32 bases per step, in
// one of two modes:
//  * ideal: each lane takes one k-mer: the window minimum over a hash
//    history in shared memory (ties to the later position), an emission when
//    it differs from the previous k-mer's, and whether the k-mer leaving the
//    window is popped at the front.  Front pops are the only moves of the
//    ring's head slot, which is all the ring state this mode keeps.
//  * exact: from the first push that finds the ring full, lane 0 runs the
//    ring with the reference's indexing (RingMinQueue::idx subtracts the
//    capacity once; entries past the capacity live in spare slots, i.e.
//    behave as plain memory, the reference writing past its vector there).
//    Entering it rebuilds the ring: the win live entries are the last win
//    k-mers, in consecutive slots from the head.  After each step the warp
//    compares the ring's logical contents with the ideal deque (the suffix
//    minima of the window); when they are equal the ring behaves ideally
//    until the next overflow, and the warp returns to the ideal mode.
// Emissions of both modes queue in shared memory in position order and are
// looked up in the center index and written 32 at a time; each step's
// packed bytes are loaded one step ahead.
constexpr int kExactWarps = 4;
constexpr int kExactBlocks = 64;

// Hash history slots (a power of two holding a window plus a step), from
// the ring size 2 w + 16.
__host__ __device__ __forceinline__ int exact_hist_slots(int ring_slots)
{
    const int w = (ring_slots - 16) / 2;
    int s = 64;
    while (s < w + 64) s <<= 1;
    return s;
}

__host__ __device__ __forceinline__ size_t exact_warp_bytes(int ring_slots)
{
    return ((size_t)exact_hist_slots(ring_slots) * 8 + (size_t)ring_slots * 12 + 64 * 16 + 15) & ~(size_t)15;
}

__global__ void __launch_bounds__(kExactWarps * 32) seed_exact_kernel(IndexDev ix, BatchDev b, SeedOut so)
{
    extern __shared__ uint64_t ex_smem[];
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    const int RS = b.ring_slots;
    const uint32_t HM = (uint32_t)exact_hist_slots(RS) - 1u;
    uint64_t* hist = ex_smem + wl * (exact_warp_bytes(RS) / 8);  // hash of k-mer p at p & HM
    uint64_t* eh = hist + HM + 1;                                 // emission queue: hash
    uint64_t* rh = eh + 64;                                       // ring: hash
    uint32_t* ep = reinterpret_cast<uint32_t*>(rh + RS);          // emission queue: position
    uint32_t* es = ep + 64;                                       // emission queue: strand bit
    uint32_t* rp = es + 64;                                       // ring: position
    const unsigned le = lane == 31 ? FULL : (2u << lane) - 1u;   // lanes <= this one
    const unsigned lt = (1u << lane) - 1u;                        // lanes < this one
    const unsigned total = *b.n_exact;
    const uint32_t k = (uint32_t)ix.k;
    const uint64_t kmask = (1ULL << (2 * k)) - 1ULL;
    const uint32_t last_slot = (uint32_t)RS - 1;
    for (unsigned wi = blockIdx.x * kExactWarps + wl; wi < total; wi += gridDim.x * kExactWarps) {
        const int q = (int)b.exact_list[wi];
        const uint32_t n = (uint32_t)b.qlen[q];
        const uint8_t* pk = b.packed + b.poff[q];
        int64_t ecur = b.exc_off[q];
        const int64_t e1 = b.exc_off[q + 1];
        const int64_t hb = b.hoff[q];
        const uint32_t nk = n - k + 1;
        const uint32_t win = (uint32_t)ix.w < nk ? (uint32_t)ix.w : nk;
        for (int t = lane; t < RS; t += 32) rh[t] = 0, rp[t] = 0;
        uint64_t prev = 0, last_h = 0;
        uint32_t run_base = 0, runlen = 0, m_prev = 0;        // carried from the previous step
        uint32_t head = 0, size = 0, valid = 0, last_p = 0;   // ring state (head in both modes)
        bool exact = false, has_last = false;
        int n_hits = 0, n_match = 0;
        int nq = 0;  // queued emissions (<= 63)
        // the first cnt (<= 32) queued emissions: looked up and written in
        // order; the rest move to the front of the queue
        auto flush = [&](int cnt) {
            const bool act = lane < cnt;
            const uint64_t ch = act ? eh[lane] : 0;
            const uint32_t cp = act ? ep[lane] : 0, cs = act ? es[lane] : 0;
            if (so.mode == 0) {
                const uint32_t ent = act ? index_find(ix, ch) : kEmptyKey;
                const bool hit = act && ent != kEmptyKey;
                const unsigned mm = __ballot_sync(FULL, hit);
                if (hit) {
                    const int r = n_match + __popc(mm & lt);
                    b.hit_pos[hb + r] = cp;
                    b.hit_ent[hb + r] = ent;
                }
                n_match += __popc(mm);
            } else if (act) {
                so.hx[hb + n_hits + lane] = (ch << 8) | (uint64_t)(uint8_t)k;
                so.hy[hb + n_hits + lane] = ((uint64_t)(cs ? 0x80000000u : 0u) << 32) | (uint64_t)cp;
            }
            n_hits += cnt;
            const int rest = nq - cnt;
            const bool mv = lane < rest;
            const uint64_t mh = mv ? eh[cnt + lane] : 0;
            const uint32_t mp = mv ? ep[cnt + lane] : 0, ms = mv ? es[cnt + lane] : 0;
            __syncwarp();
            if (mv) eh[lane] = mh, ep[lane] = mp, es[lane] = ms;
            __syncwarp();
            nq = rest;
        };
        uint32_t pk_next = lane < (int)n ? pk[lane >> 2] : 0u;  // the packed byte of this lane's base, a step ahead
        __syncwarp();
        for (uint32_t i0 = 0; i0 < n; i0 += 32) {
            const uint32_t i = i0 + (uint32_t)lane;
            const bool inq = i < n;
            const uint32_t pkb = pk_next;
            pk_next = i + 32 < n ? pk[(i + 32) >> 2] : 0u;
            uint32_t c = 0;
            if (inq) {
                c = (pkb >> ((i & 3u) * 2u)) & 3u;
                for (int64_t ee = ecur; ee < e1 && (uint32_t)b.exc[ee * 3] <= i; ++ee)
                    if (i < (uint32_t)(b.exc[ee * 3] + b.exc[ee * 3 + 1])) c = nt4_of((uint8_t)b.exc[ee * 3 + 2]);
            }
            while (ecur < e1 && (uint32_t)(b.exc[ecur * 3] + b.exc[ecur * 3 + 1]) <= i0 + 32u) ++ecur;
            const unsigned badm = __ballot_sync(FULL, inq && c >= 4);
            // codes of positions i0 .. i, newest in the low bits
            uint64_t x = (uint64_t)(c & 3u);
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint64_t y = __shfl_up_sync(FULL, x, d);
                if (lane >= d) x |= y << (2 * d);
            }
            const uint64_t fwd = (lane == 31 ? x : (prev << (2 * (lane + 1))) | x) & kmask;
            prev = __shfl_sync(FULL, x, 31);
            uint64_t code = fwd;
            bool strand = true;
            if (!ix.non_canonical) {  // reverse complement: 2-bit groups reversed, complemented
                uint64_t r = __brevll(fwd);
                r = ((r >> 1) & 0x5555555555555555ULL) | ((r & 0x5555555555555555ULL) << 1);
                r = (r >> (64 - 2 * k)) ^ kmask;
                strand = fwd <= r;
                code = fwd < r ? fwd : r;
            }
            const unsigned strm = __ballot_sync(FULL, strand);
            // first base of each lane's N-free run; the k-mer ending here is valid when k bases of it precede
            const unsigned bl = badm & le;
            const uint32_t rb = bl ? i0 + (uint32_t)(32 - __clz(bl)) : run_base;
            const bool kv = inq && c < 4 && i + 1 >= rb + k;
            const uint32_t pos = i + 1 - k;
            const uint64_t h = splitmix64(code) >> 8;
            if (kv) hist[pos & HM] = h;
            run_base = __shfl_sync(FULL, rb, 31);
            __syncwarp();
            // length of the run of strict hash increases ending at each k-mer
            const bool inc = kv && pos > rb && hist[(pos - 1) & HM] < h;
            const unsigned z = ~__ballot_sync(FULL, inc) & le;
            const uint32_t rl = z ? (uint32_t)lane - (31u - (uint32_t)__clz(z)) : runlen + (uint32_t)lane + 1u;
            runlen = __shfl_sync(FULL, rl, 31);
            uint32_t start = 0;
            if (!exact) {
                const unsigned ovm = __ballot_sync(FULL, kv && rl >= win);  // the push finds the ring full
                const int L = ovm ? __ffs(ovm) - 1 : 32;
                const bool act = lane < L && kv && pos + 1 >= win;
                uint64_t hm = ~0ULL;
                uint32_t m = 0;
                bool fp = false;
                if (act) {
                    const uint32_t lo = max(rb, pos + 1 - win);
                    for (uint32_t j = lo; j <= pos; ++j) {
                        const uint64_t y = hist[j & HM];
                        if (y <= hm) hm = y, m = j;
                    }
                    fp = pos >= rb + win && hist[(pos - win) & HM] < hm;  // k-mer pos - win leaves at the front
                }
                uint32_t mp = __shfl_up_sync(FULL, m, 1);
                if (lane == 0) mp = m_prev;
                const bool em = act && (!(pos > rb && pos >= win) || m != mp);
                m_prev = __shfl_sync(FULL, m, 31);
                unsigned fpm = __ballot_sync(FULL, fp);
                const unsigned bm = badm & (L >= 32 ? FULL : (1u << L) - 1u);
                if (bm) {  // an N cleared the ring: count the front pops after the last one
                    const int bn = 31 - __clz(bm);
                    head = 0;
                    fpm &= bn == 31 ? 0u : ~((2u << bn) - 1u);
                }
                head = (head + (uint32_t)__popc(fpm)) % win;
                const unsigned emm = __ballot_sync(FULL, em);
                if (em) {
                    const int r = nq + __popc(emm & lt);
                    eh[r] = hm, ep[r] = m, es[r] = strand ? 1u : 0u;
                }
                nq += __popc(emm);
                if (L < 32) {  // rebuild the full ring before the push of k-mer P
                    const uint32_t P = i0 + (uint32_t)L + 1 - k;
                    for (uint32_t t = (uint32_t)lane; t < win; t += 32) {
                        uint32_t s = head + t;
                        if (s >= win) s -= win;
                        rh[s] = hist[(P - win + t) & HM];
                        rp[s] = P - win + t;
                    }
                    size = win, valid = k, has_last = true;
                    last_h = hist[(P - win) & HM], last_p = P - win;
                    exact = true, start = (uint32_t)L;
                    __syncwarp();
                }
            }
            if (exact) {
                int ne = 0;
                if (lane == 0) {
                    const uint32_t lim = min(32u, n - i0);
                    for (uint32_t l = start; l < lim; ++l) {
                        if (badm >> l & 1u) {
                            valid = 0, head = size = 0, has_last = false;
                            continue;
                        }
                        if (valid < k) ++valid;
                        if (valid < k) continue;
                        const uint32_t p = i0 + l + 1 - k;
                        const uint64_t hh = hist[p & HM];
                        while (size) {
                            uint32_t bi = head + size - 1;
                            if (bi >= win) bi -= win;
                            if (rh[min(bi, last_slot)] >= hh) --size;
                            else break;
                        }
                        {
                            uint32_t bi = head + size;
                            if (bi >= win) bi -= win;
                            bi = min(bi, last_slot);
                            rh[bi] = hh, rp[bi] = p;
                            ++size;
                        }
                        if (p + 1 < win) continue;
                        const uint32_t ws = p + 1 - win;
                        while (size && rp[head] < ws) head = head + 1 >= win ? head + 1 - win : head + 1, --size;
                        if (size) {
                            const uint64_t ch = rh[head];
                            const uint32_t cp = rp[head];
                            if (!has_last || ch != last_h || cp != last_p) {
                                eh[nq + ne] = ch, ep[nq + ne] = cp, es[nq + ne] = strm >> l & 1u;
                                ++ne;
                                last_h = ch, last_p = cp, has_last = true;
                            }
                        }
                    }
                }
                ne = __shfl_sync(FULL, ne, 0);
                head = __shfl_sync(FULL, head, 0);
                size = __shfl_sync(FULL, size, 0);
                valid = __shfl_sync(FULL, valid, 0);
                has_last = __shfl_sync(FULL, (int)has_last, 0) != 0;
                last_h = __shfl_sync(FULL, last_h, 0);
                last_p = __shfl_sync(FULL, last_p, 0);
                __syncwarp();
                nq += ne;
                // back to the ideal mode once the ring holds the ideal deque of the step's last k-mer
                if (i0 + 32 < n && __shfl_sync(FULL, (int)(kv && pos + 1 >= win), 31)) {
                    const uint32_t hp = i0 + 32 - k;
                    uint32_t tot = 0;
                    uint64_t cmin = ~0ULL;  // minimum hash after the current group's k-mers
                    for (int pass = 0; pass < 2; ++pass) {
                        uint32_t before = 0;
                        bool bad = false;
                        cmin = ~0ULL;
                        for (uint32_t g = 0; g < win; g += 32) {
                            const uint32_t t = g + (uint32_t)lane;  // k-mer hp - t
                            const bool in = t < win && hp >= run_base + t;
                            const uint64_t y = in ? hist[(hp - t) & HM] : ~0ULL;
                            uint64_t pm = y;
#pragma unroll
                            for (int d = 1; d < 32; d <<= 1) {
                                const uint64_t o = __shfl_up_sync(FULL, pm, d);
                                if (lane >= d && o < pm) pm = o;
                            }
                            uint64_t ex = __shfl_up_sync(FULL, pm, 1);
                            if (lane == 0) ex = ~0ULL;
                            if (cmin < ex) ex = cmin;
                            const bool f = in && y < ex;  // a suffix minimum: in the ideal deque
                            const unsigned fm = __ballot_sync(FULL, f);
                            if (pass == 1 && f) {
                                const uint32_t r = tot - (before + (uint32_t)__popc(fm & le));  // deque index
                                uint32_t s = head + r;
                                if (s >= win) s -= win;
                                if (rp[min(s, last_slot)] != hp - t) bad = true;
                            }
                            before += (uint32_t)__popc(fm);
                            const uint64_t gm = __shfl_sync(FULL, pm, 31);
                            if (gm < cmin) cmin = gm;
                        }
                        if (pass == 0) {
                            tot = before;
                            if (tot != size) break;
                        } else if (!__any_sync(FULL, bad)) {
                            exact = false;
                            m_prev = last_p;
                        }
                    }
                }
            }
            __syncwarp();
            if (nq >= 32) flush(32);
        }
        while (nq > 0) flush(nq < 32 ? nq : 32);
        if (lane == 0) {
            b.n_hits[q] = n_hits;
            b.n_matched[q] = n_match;
        }
    }
}
}  // namespace hg

extern "C" cudaError_t hg_launch_seed(const hg::IndexDev* ix, const hg::BatchDev* b, int mode, uint64_t* hx,
                                      uint64_t* hy, int grid, cudaStream_t st)
{
    hg::SeedOut so{mode, hx, hy};
    hg::seed_kernel<<<grid, hg::kSeedThreads, 0, st>>>(*ix, *b, so);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (mode == 0) {
        hg::seed_fast_kernel<<<grid, hg::kSeedFastWarps * 32, 0, st>>>(*ix, *b);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    hg::seed_exact_kernel<<<hg::kExactBlocks, hg::kExactWarps * 32,
                            hg::kExactWarps * hg::exact_warp_bytes(b->ring_slots), st>>>(*ix, *b, so);
    return cudaGetLastError();
}
