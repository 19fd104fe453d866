// hg_sketch.cu - multi-reference mode on the device: MinHash sketches of a
// query batch and the best reference of every query.
//
// mash::sketchFromSequence (src/mash/mash.cpp:32-117) keeps, with a max-heap
// and a seen-set, the sketch_size smallest DISTINCT hashes of a sequence's
// valid k-mers; each hash is getHash2bit (src/mash/hash.cpp), XXH3-64 with a
// seed over the 8 big-endian bytes of the 2-bit k-mer code.  The selection
// loop of RefAligner::alignOneQueryToRef (src/align/ref_aligner.cpp:232-241)
// then takes the first reference of largest mash::jaccard (|a & b| /
// min(|a|, |b|), src/mash/mash.cpp:120-164).
//
// One CTA owns one query at a time (persistent grid, atomic queue) and keeps
// the sketch in shared memory:
//   * tiles of kSketchTile k-mer starts; a query without exception bytes
//     (forward codes, k <= 29) takes each thread's four codes from one
//     64-bit window of the 2-bit pack, any other query decodes the tile with
//     the exception runs overlaid (nt4: N and other bytes invalid, lowercase
//     and U valid) and rolls the forward / reverse codes;
//   * a hash is a candidate when it is at most the admission limit: while
//     fewer than sketch_size distinct hashes are kept, a first limit sized
//     for about 1.25 x sketch_size candidates over the query (uniform hashes);
//     once sketch_size are kept, anything below the largest kept one;
//   * when the candidates could overflow the buffer, and at the end, kept +
//     candidates are bucket-sorted (1,024 buckets by leading bits; each
//     bucket sorted by one thread; a bitonic sort when a bucket is large),
//     de-duplicated and cut to sketch_size;
//   * a query that ends with fewer than sketch_size distinct hashes under the
//     first limit (short, repetitive or N-rich queries) is swept again with no
//     limit, so the result is exact for every input;
//   * the sketch is matched against the references: with at most 64
//     references, one probe per kept hash in a resident table hash -> mask of
//     the references whose sketch holds it, and per-reference counts by warp
//     ballots; otherwise a binary search per kept hash in each reference
//     sketch.  The first reference of strictly largest jaccard wins.
#include <cuda_runtime.h>

#include "hg_common.cuh"

namespace hg {

constexpr int kSketchThreads = 512;
constexpr int kSketchPer = 4;
constexpr int kSketchTile = kSketchThreads * kSketchPer;  // k-mer starts per tile
constexpr int kSketchLB = 10;                              // log2 of the flush buckets
constexpr int kSketchBuckets = 1 << kSketchLB;
constexpr int kSketchBucketMax = 48;  // larger buckets: bitonic sort instead
constexpr int kSketchFastMaxK = 29;   // four starts' k-mers inside one 32-base window

// getHash2bit: XXH3-64 of the 8 big-endian bytes of `code` (xxHash 0.8.3, its
// 4..8-byte input branch).  The seed's low word is byte-swapped into its high
// word; the input is read as two little-endian 32-bit words, the first on top;
// it is xored with (secret[8..15] ^ secret[16..23]) - seed, the two secret
// words being little-endian reads of XXH3's default secret; the rrmxmx
// finaliser mixes in the input length 8.
__device__ __forceinline__ uint64_t hash2bit(uint64_t code, uint64_t seed_mixed)
{
    const uint32_t w_hi = __byte_perm((uint32_t)(code >> 32), 0, 0x0123);
    const uint32_t w_lo = __byte_perm((uint32_t)code, 0, 0x0123);
    uint64_t h = (((uint64_t)w_hi << 32) | w_lo) ^ (0xc73ab174c5ecd5a2ULL - seed_mixed);
    h ^= ((h << 49) | (h >> 15)) ^ ((h << 24) | (h >> 40));
    h *= 0x9FB21C651E98DF25ULL;
    h ^= (h >> 35) + 8;
    h *= 0x9FB21C651E98DF25ULL;
    return h ^ (h >> 28);
}

struct SketchArgs {
    const uint8_t* packed;
    const int64_t* poff;
    const int32_t* qlen;
    const int32_t* exc;      // runs {start, len, byte}
    const int64_t* exc_off;  // n + 1
    int n;
    int k, s;                // k-mer size, sketch size
    int noncanonical;
    uint64_t seed_mixed;     // seed ^ (bswap32(seed) << 32)
    int cap;                 // entries of each of the two shared regions: s + kSketchTile
    uint64_t* out;           // optional: n x out_stride hashes
    int64_t out_stride;
    int32_t* out_n;          // optional: sketch sizes
    const uint64_t* ref_h;   // optional: reference sketches, concatenated
    const int64_t* ref_off;  // n_refs + 1
    int n_refs;
    const ulonglong2* ref_tab;  // with <= 64 references: hash -> mask of references (y = 0: empty)
    uint32_t ref_tab_mask;
    int32_t* best;           // with ref_h: best reference per query
    double* best_j;          // with ref_h: its jaccard
    unsigned* queue;
};

__device__ __forceinline__ int next_pow2(int v)
{
    int p = 2;
    while (p < v) p <<= 1;
    return p;
}

__device__ __forceinline__ uint64_t block_or64(uint64_t v, uint64_t* red)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v |= __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[wid] = v;
    __syncthreads();
    uint64_t r = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r |= red[i];
    __syncthreads();
    return r;
}

// Sort buf[0, total) ascending, de-duplicate, keep the smallest `s` at
// buf[0, kept).  buf[cap, 2 cap) is the sorted copy.
__device__ int sketch_flush(uint64_t* buf, int total, int s, int cap, int* scratch, uint32_t* hist,
                            uint64_t* red)
{
    const int tid = threadIdx.x, nt = blockDim.x;
    uint64_t* srt = buf + cap;
    // buckets by the leading kSketchLB bits below the highest set bit of all values
    uint64_t any = 0;
    for (int i = tid; i < total; i += nt) any |= buf[i];
    any = block_or64(any, red);
    const int sh = any ? __clzll((long long)any) : 63;
    auto bucket = [&](uint64_t h) { return (uint32_t)((h << sh) >> (64 - kSketchLB)); };
    for (int j = tid; j < kSketchBuckets; j += nt) hist[j] = 0;
    __syncthreads();
    for (int i = tid; i < total; i += nt) atomicAdd(&hist[bucket(buf[i])], 1u);
    __syncthreads();
    // exclusive offsets, kSketchBuckets / nt consecutive buckets per thread
    constexpr int kPerT = kSketchBuckets / kSketchThreads;
    uint32_t c[kPerT], sum = 0, big = 0;
#pragma unroll
    for (int q = 0; q < kPerT; ++q) c[q] = hist[tid * kPerT + q], sum += c[q], big = max(big, c[q]);
    int tot = 0;
    uint32_t o = (uint32_t)block_excl_sum((int)sum, scratch, &tot);
    const unsigned any_big = __syncthreads_or(big > (uint32_t)kSketchBucketMax);
#pragma unroll
    for (int q = 0; q < kPerT; ++q) hist[tid * kPerT + q] = o, o += c[q];
    __syncthreads();
    if (!any_big) {
        for (int i = tid; i < total; i += nt) srt[atomicAdd(&hist[bucket(buf[i])], 1u)] = buf[i];
        __syncthreads();
        // hist[j] is now the end of bucket j; one thread sorts each bucket
        for (int j = tid; j < kSketchBuckets; j += nt) {
            const int e = (int)hist[j], b = j ? (int)hist[j - 1] : 0;
            for (int x = b + 1; x < e; ++x) {
                const uint64_t v = srt[x];
                int y = x - 1;
                while (y >= b && srt[y] > v) srt[y + 1] = srt[y], --y;
                srt[y + 1] = v;
            }
        }
        __syncthreads();
    } else {  // skewed values: bitonic sort over both regions, then the sorted copy
        const int P = next_pow2(total);
        for (int i = total + tid; i < P; i += nt) buf[i] = ~0ull;
        __syncthreads();
        for (int size = 2; size <= P; size <<= 1) {
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                for (int i = tid; i < (P >> 1); i += nt) {
                    const int lo = 2 * i - (i & (stride - 1)), hi = lo + stride;
                    const uint64_t x = buf[lo], y = buf[hi];
                    const bool up = (lo & size) == 0;
                    if ((x > y) == up) buf[lo] = y, buf[hi] = x;
                }
                __syncthreads();
            }
        }
        // the sorted values sit in buf[0, total), disjoint from srt (total <= cap)
        for (int i = tid; i < total; i += nt) srt[i] = buf[i];
        __syncthreads();
    }
    // first occurrences, in order, into buf[0, min(distinct, s))
    const int per = (total + nt - 1) / nt;
    const int i0 = min(tid * per, total), i1 = min(i0 + per, total);
    int u = 0;
    for (int i = i0; i < i1; ++i) u += (i == 0 || srt[i] != srt[i - 1]);
    int n_unique = 0;
    int w = block_excl_sum(u, scratch, &n_unique);
    for (int i = i0; i < i1 && w < s; ++i)
        if (i == 0 || srt[i] != srt[i - 1]) buf[w++] = srt[i];
    __syncthreads();
    return min(n_unique, s);
}

__global__ void __launch_bounds__(kSketchThreads, 3) sketch_kernel(SketchArgs a)
{
    extern __shared__ uint64_t buf[];  // 2 x cap hashes
    __shared__ uint8_t codes[kSketchTile + 32];
    __shared__ uint32_t hist[kSketchBuckets];
    __shared__ uint64_t red[kSketchThreads / 32];
    __shared__ int scratch[33];
    __shared__ int s_q, s_cnt;
    __shared__ unsigned s_warp_base[kSketchThreads / 32];
    __shared__ unsigned refcnt[64];
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, wid = tid >> 5;
    const int k = a.k, s = a.s;
    const uint64_t mask = (1ull << ((2 * k) & 63)) - 1ull;  // shift count mod 64, as the host CPU: 0 at k = 32
    const int shift = 2 * (k - 1);
    const int lsh = 64 - 2 * k;
    for (;;) {
        if (tid == 0) s_q = (int)atomicAdd(a.queue, 1u);
        __syncthreads();
        const int q = s_q;
        __syncthreads();
        if (q >= a.n) break;
        const int len = a.qlen[q];
        const uint8_t* pk = a.packed + a.poff[q];
        const int64_t e0 = a.exc_off[q], e1 = a.exc_off[q + 1];
        const bool fast = e0 == e1 && a.noncanonical && k <= kSketchFastMaxK;
        int kept = 0;
        if (k > 0 && k <= 32 && s > 0 && len >= k) {
            const int nk = len - k + 1;
            // first admission limit: about 1.25 s + 64 uniform hashes at or below it
            uint64_t lim0 = ~0ull;
            const double frac = (1.25 * (double)s + 64.0) / (double)nk;
            if (frac < 1.0) lim0 = (uint64_t)ldexp(frac, 64);
            for (int sweep = 0; sweep < 2; ++sweep) {
                bool open = true;    // an admission limit exists
                uint64_t lim = lim0;  // admit h <= lim
                kept = 0;
                if (tid == 0) s_cnt = 0;
                __syncthreads();
                for (int t0 = 0; t0 < nk; t0 += kSketchTile) {
                    const int p0 = t0 + tid * kSketchPer;
                    uint64_t hv[kSketchPer];
                    bool ok[kSketchPer];
#pragma unroll
                    for (int i = 0; i < kSketchPer; ++i) ok[i] = false;
                    if (fast) {
                        // bases p0 .. p0+31 from one 64-bit window: bit-reversed and
                        // pair-swapped, base p0 sits in the top two bits, so the
                        // forward code of the k-mer at p0+i is (x << 2i) >> (64 - 2k)
                        if (p0 < nk && open) {
                            const uint32_t wb = ((uint32_t)p0 >> 2) & ~7u;
                            const uint64_t* wp = reinterpret_cast<const uint64_t*>(pk + wb);
                            const uint64_t w0 = wp[0], w1 = wp[1];
                            const uint32_t sb = 2u * ((uint32_t)p0 - wb * 4u);
                            const uint64_t lo = sb ? (w0 >> sb) | (w1 << (64u - sb)) : w0;
                            uint64_t x = __brevll(lo);
                            x = ((x >> 1) & 0x5555555555555555ULL) | ((x & 0x5555555555555555ULL) << 1);
#pragma unroll
                            for (int i = 0; i < kSketchPer; ++i) {
                                if (p0 + i < nk) {
                                    hv[i] = hash2bit((x << (2 * i)) >> lsh, a.seed_mixed);
                                    ok[i] = hv[i] <= lim;
                                }
                            }
                        }
                    } else {
                        __syncthreads();  // the previous tile's codes are read
                        const int span = min(kSketchTile + k - 1, len - t0);
                        for (int i = tid; i < span; i += nt)
                            codes[i] = (uint8_t)packed_code(pk, (uint32_t)(t0 + i));
                        __syncthreads();
                        for (int64_t e = e0; e < e1; ++e) {
                            const int st = a.exc[3 * e], rl = a.exc[3 * e + 1];
                            const uint8_t c = nt4_of((uint8_t)a.exc[3 * e + 2]);
                            const int lo = max(st, t0), hi = min(st + rl, t0 + span);
                            for (int p = lo + tid; p < hi; p += nt) codes[p - t0] = c;
                        }
                        __syncthreads();
                        // this thread's starts p0 .. p0+3; the window covers codes[j - k + 1 .. j]
                        if (p0 < nk && open) {
                            uint64_t fwd = 0, rev = 0;
                            int last_bad = -1;
                            const int jn = min(k - 1 + kSketchPer, len - p0);
                            for (int j = 0; j < jn; ++j) {
                                const uint32_t c = codes[p0 - t0 + j];
                                if (c >= 4) last_bad = j;
                                fwd = ((fwd << 2) | (c & 3u)) & mask;
                                rev = (rev >> 2) | ((uint64_t)(3u ^ (c & 3u)) << shift);
                                const int i = j - (k - 1);
                                if (i >= 0 && p0 + i < nk && last_bad < i) {
                                    const uint64_t code = a.noncanonical ? fwd : (fwd < rev ? fwd : rev);
                                    const uint64_t h = hash2bit(code, a.seed_mixed);
#pragma unroll
                                    for (int t = 0; t < kSketchPer; ++t)
                                        if (t == i) hv[t] = h, ok[t] = h <= lim;
                                }
                            }
                        }
                    }
                    // warp-aggregated appends after the kept region
#pragma unroll
                    for (int i = 0; i < kSketchPer; ++i) {
                        const unsigned m = __ballot_sync(0xffffffffu, ok[i]);
                        if (lane == 0 && m) s_warp_base[wid] = (unsigned)atomicAdd(&s_cnt, __popc(m));
                        __syncwarp();
                        if (ok[i]) buf[kept + s_warp_base[wid] + __popc(m & ((1u << lane) - 1u))] = hv[i];
                        __syncwarp();
                    }
                    __syncthreads();
                    const int cnt = s_cnt;
                    const bool last_tile = t0 + kSketchTile >= nk;
                    if (kept + cnt + kSketchTile > a.cap || (last_tile && cnt > 0)) {
                        kept = sketch_flush(buf, kept + cnt, s, a.cap, scratch, hist, red);
                        if (tid == 0) s_cnt = 0;
                        if (kept == s) {
                            open = buf[s - 1] != 0;
                            lim = buf[s - 1] - 1;  // strictly below the largest kept hash
                        }
                    }
                    __syncthreads();
                }
                if (kept >= s || lim0 == ~0ull) break;
                lim0 = ~0ull;  // too few distinct hashes under the first limit: sweep again without it
            }
        }
        if (a.out) {
            for (int i = tid; i < kept; i += nt) a.out[(int64_t)q * a.out_stride + i] = buf[i];
            if (tid == 0) a.out_n[q] = kept;
        }
        if (a.ref_h) {
            double best = -1.0;
            int best_r = 0;
            auto consider = [&](int r, int inter) {
                const int nr = (int)(a.ref_off[r + 1] - a.ref_off[r]);
                double j;
                if (kept == 0 && nr == 0) j = 1.0;
                else if (kept == 0 || nr == 0) j = 0.0;
                else j = (double)inter / (double)min(kept, nr);
                if (j > best) best = j, best_r = r;
            };
            if (a.ref_tab) {  // one probe per kept hash, counts per reference by ballots
                for (int r = tid; r < 64; r += nt) refcnt[r] = 0;
                __syncthreads();
                for (int base = wid * 32; base < kept; base += nt) {
                    const int i = base + lane;
                    uint64_t m = 0;
                    if (i < kept) {
                        const uint64_t x = buf[i];
                        for (uint32_t sl = (uint32_t)x & a.ref_tab_mask;; sl = (sl + 1) & a.ref_tab_mask) {
                            const ulonglong2 e = a.ref_tab[sl];
                            if (e.y == 0) break;
                            if (e.x == x) {
                                m = e.y;
                                break;
                            }
                        }
                    }
                    uint64_t wm = m;
                    for (int o = 16; o > 0; o >>= 1) wm |= __shfl_xor_sync(0xffffffffu, wm, o);
                    while (wm) {
                        const int r = __ffsll((long long)wm) - 1;
                        wm &= wm - 1;
                        const unsigned c = __popc(__ballot_sync(0xffffffffu, (m >> r) & 1ull));
                        if (lane == 0) atomicAdd(&refcnt[r], c);
                    }
                }
                __syncthreads();
                for (int r = 0; r < a.n_refs; ++r) consider(r, (int)refcnt[r]);
            } else {
                for (int r = 0; r < a.n_refs; ++r) {
                    const uint64_t* rh = a.ref_h + a.ref_off[r];
                    const int nr = (int)(a.ref_off[r + 1] - a.ref_off[r]);
                    int hit = 0;
                    for (int i = tid; i < kept && nr > 0; i += nt) {
                        const uint64_t x = buf[i];
                        int lo = 0, hi = nr;  // first element >= x
                        while (lo < hi) {
                            const int mid = (lo + hi) >> 1;
                            if (rh[mid] < x) lo = mid + 1;
                            else hi = mid;
                        }
                        hit += lo < nr && rh[lo] == x;
                    }
                    int inter = 0;
                    block_excl_sum(hit, scratch, &inter);
                    consider(r, inter);
                }
            }
            if (tid == 0) a.best[q] = best_r, a.best_j[q] = best;
        }
        __syncthreads();
    }
}

}  // namespace hg

// Shared-memory bytes and region size of a sketch launch; 0 when sketch_size
// is above what one CTA holds.
extern "C" size_t hg_sketch_smem(int sketch_size, int* cap)
{
    if (sketch_size <= 0) sketch_size = 1;
    const int c = sketch_size + hg::kSketchTile;
    const size_t bytes = (size_t)2 * c * 8;
    if (bytes > 200 * 1024) return 0;
    if (cap) *cap = c;
    return bytes;
}

extern "C" cudaError_t hg_launch_sketch(const uint8_t* packed, const int64_t* poff, const int32_t* qlen,
                                        const int32_t* exc, const int64_t* exc_off, int n, int k, int s,
                                        int noncanonical, int seed, uint64_t* out, int64_t out_stride,
                                        int32_t* out_n, const uint64_t* ref_h, const int64_t* ref_off,
                                        int n_refs, const ulonglong2* ref_tab, uint32_t ref_tab_mask,
                                        int32_t* best, double* best_j, unsigned* queue, int sms, cudaStream_t st)
{
    hg::SketchArgs a;
    a.packed = packed, a.poff = poff, a.qlen = qlen, a.exc = exc, a.exc_off = exc_off, a.n = n;
    a.k = k, a.s = s, a.noncanonical = noncanonical;
    const uint32_t s32 = (uint32_t)seed;
    a.seed_mixed = (uint64_t)s32 ^ ((uint64_t)__builtin_bswap32(s32) << 32);
    const size_t smem = hg_sketch_smem(s, &a.cap);
    if (!smem) return cudaErrorInvalidValue;
    a.out = out, a.out_stride = out_stride, a.out_n = out_n;
    a.ref_h = ref_h, a.ref_off = ref_off, a.n_refs = n_refs, a.best = best, a.best_j = best_j;
    a.ref_tab = n_refs <= 64 ? ref_tab : nullptr, a.ref_tab_mask = ref_tab_mask;
    a.queue = queue;
    cudaError_t e = cudaFuncSetAttribute(hg::sketch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, hg::sketch_kernel, hg::kSketchThreads, smem);
    if (e != cudaSuccess) return e;
    const int grid = std::max(1, std::min(n, sms * std::max(per_sm, 1)));
    e = cudaMemsetAsync(queue, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    if (n == 0) return cudaSuccess;
    hg::sketch_kernel<<<grid, hg::kSketchThreads, smem, st>>>(a);
    return cudaGetLastError();
}
