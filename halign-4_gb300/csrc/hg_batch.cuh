// hg_batch.cuh - device-side views of the resident center index and of one
// batch of queries, passed by value to every stage kernel.
#pragma once

#include "hg_common.cuh"

namespace hg {

// Center index, built once per center and kept in HBM (the reference rebuilds
// it on every collect_anchors call, src/seed/minimizer.cpp:238-265).
struct IndexDev {
    int L;                     // center length
    int k, w;                  // minimizer k-mer size and window
    int non_canonical;         // 1 on the align-to-center path (src/align/ref_aligner.cpp:83)
    const uint8_t* center;     // DNA5 codes of the center the DP aligns to
    const uint8_t* center2;    // the same center 2-bit packed (base i at bits 2(i&3) of byte i>>2), 64 B slack
    int center_plain;          // 1 when every center code is A/C/G/T (center2 is exact)
    const ulonglong2* tab;     // open-addressing table, one 16-byte slot per probe:
                               // {key = hash56 (kNoHash = empty), entry id of the key}
    uint32_t tab_mask;
    uint32_t n_ent;            // distinct center minimizer hashes
    const uint2* ent_meta;     // x: the center position if the entry occurs once, else its start in cpos;
                               // y: occurrence count | 1 << 31 if count > the occurrence threshold
    const uint32_t* cpos;      // center positions grouped by hash, ascending within a hash
    const uint32_t* cspan;     // matching spans (always k for a single center)
    double q_occ_frac;
    uint64_t sample_every;
    // chain parameters (anchor::ChainParams, include/anchor.h:116-127)
    int max_dist_x, max_dist_y, bw, max_skip, max_iter, min_cnt, min_score;
    float gap_pen, skip_pen;
    int dg_nopen;              // with dd == 0 the chain penalty is 0 for every dg <= dg_nopen (>= k)
    const float* log2tab;      // log2f(i) for i in [0, n_log2)
    int n_log2;
};

// One gap-fill segment of globalAlignMM2 (src/align/align.cpp:221-293).
struct Seg {
    uint32_t rs, qs, rl, ql;  // center start/len, query start/len
    uint32_t slot;            // op slot, relative to the query's CIGAR scratch
    int32_t nops;             // DP result length; -1 = segment did not consume (I/D fallback)
    uint32_t q;               // query index
    uint32_t kind;            // low byte: SegKind; bit 8: left-aligned gaps (first segment)
};

enum SegKind : uint32_t {
    kSegEmpty = 0, kSegIns = 1, kSegDel = 2, kSegDpSmall = 3, kSegDpLarge = 4, kSegGlobal = 5,
    kSegMatch = 6,  // equal lengths, identical A/C/G/T on both sides: the extz2 CIGAR is rl M
    kSegDpThin = 7,  // query side <= 32, long center side: grouped wavefront, ops stored last-first
    kSegDpSquare = 8  // both sides moderate: thread DP, directions in the warp's slot, ops stored last-first
};

// True for the gap-fill kinds that run an extz2 DP (and own a CIGAR slot).
__host__ __device__ __forceinline__ bool seg_is_dp(uint32_t kind)
{
    return kind == kSegDpSmall || kind == kSegDpLarge || kind == kSegGlobal || kind == kSegDpThin ||
           kind == kSegDpSquare;
}
constexpr uint32_t kSegLeft = 1u << 8;

// Small-DP tier: one thread per segment, direction nibbles in shared memory,
// one to four 32-bit words per row of the longer side.  Two shape ranges:
// small (shorter side <= 16, rows x words <= 64) and medium (shorter side
// 17..32, rows x words <= 160); both are far inside the band
// globalAlignKSW2 gives them (w >= 200 or unbounded), so the band never binds.
constexpr int kSmallMaxInner = 16;
constexpr int kSmallDirWords = 64;   // words of 8 nibbles per thread, small range
constexpr int kMedMaxInner = 32;
constexpr int kMedDirWords = 160;    // words per thread, medium range

__host__ __device__ __forceinline__ bool small_tier_fits(uint32_t rl, uint32_t ql)
{
    const uint32_t inner = rl < ql ? rl : ql, outer = rl < ql ? ql : rl;
    return inner >= 1 && inner <= (uint32_t)kSmallMaxInner && outer * ((inner + 7) / 8) <= (uint32_t)kSmallDirWords;
}

__host__ __device__ __forceinline__ bool medium_tier_fits(uint32_t rl, uint32_t ql)
{
    const uint32_t inner = rl < ql ? rl : ql, outer = rl < ql ? ql : rl;
    return inner > (uint32_t)kSmallMaxInner && inner <= (uint32_t)kMedMaxInner &&
           outer * ((inner + 7) / 8) <= (uint32_t)kMedDirWords;
}

// Sort key of a small-tier segment: warps then run identical loop bounds.
// Both ranges keep the longer side <= 64 (rows x words bound), so the key is
// [0,6) outer-1, [6,10) inner-1 (small) or inner-17 (medium), 10 orientation,
// 11 left-aligned, 12 medium range (sorts after every small shape).
constexpr uint32_t kShapeBins = 1u << 13;
constexpr uint32_t kNoShape = 0xffffffffu;  // key of an unused small-list entry (a hole)
constexpr uint32_t kSmallBlock = 64;        // small-list entries a chain warp reserves at a time
constexpr uint32_t kShapeMedium = 1u << 12;
__device__ __forceinline__ uint32_t shape_key(const Seg& g)
{
    const uint32_t inner = g.rl < g.ql ? g.rl : g.ql, outer = g.rl < g.ql ? g.ql : g.rl;
    const uint32_t tinner = g.rl <= g.ql ? 1u : 0u;
    const uint32_t left = (g.kind & kSegLeft) ? 1u : 0u;
    const uint32_t med = inner > (uint32_t)kSmallMaxInner ? 1u : 0u;
    const uint32_t icode = med ? inner - 17u : inner - 1u;
    return (outer - 1) | icode << 6 | tinner << 10 | left << 11 | med << 12;
}

// Thin tier: the query side 1..32 bases against a longer center side beyond
// the small and medium bounds, with a band that never binds (as for the
// wavefront tiers).  Several such segments share a warp, one lane per query
// column: a group of W = ql lanes (W = 32 above 16) runs one segment's
// anti-diagonal wavefront (floor(32 / W) groups per warp), so a step costs
// one cell per lane however short the query side is.  Direction nibbles go to
// the warp's own scratch region (16 bytes per step), which bounds the steps
// (rl + ql - 1) of a thin segment.
constexpr int kThinMaxInner = 32;
constexpr int kThinMaxSteps = 32768;
constexpr size_t kThinWarpBytes = (size_t)kThinMaxSteps * 16;
constexpr int kThinKeyClassShift = 7;  // key bits above it: the query length - 1 (the group width)
constexpr int kThinBins = kThinMaxInner << kThinKeyClassShift;

// Sort key of a thin segment: query length first (a warp takes segments of
// one length), then longest first by quarter-octave class of the center
// side, then gap mode.
__host__ __device__ __forceinline__ uint32_t thin_key(uint32_t rl, uint32_t ql, bool left)
{
    uint32_t lg = 0;
    for (uint32_t t = rl; t > 1; t >>= 1) ++lg;  // floor(log2(rl)), rl >= 33
    const uint32_t frac = lg >= 2 ? (rl >> (lg - 2)) & 3u : 0u;
    uint32_t cls = lg >= 5 ? (lg - 5) * 4 + frac : 0u;
    cls = cls > 63 ? 63 : cls;
    return (ql - 1) << kThinKeyClassShift | (63u - cls) << 1 | (left ? 0u : 1u);
}

// Wavefront tiers: segments the band never binds (auto_band < 0 or >= both
// lengths) whose shorter side is at most kWaveWarpMaxInner run one warp per
// segment; wider ones up to kWaveMaxInner run one 16-warp CTA per segment.
constexpr int kWaveWarpMaxInner = 256;   // 32 lanes x 8 columns
constexpr int kWaveMaxInner = 4096;      // 16 warps x 32 lanes x 8 columns
constexpr int kWaveBins = 256;           // sort bins of the one-warp list

__host__ __device__ __forceinline__ bool wave_eligible(uint32_t rl, uint32_t ql)
{
    const uint32_t inner = rl < ql ? rl : ql, outer = rl < ql ? ql : rl;
    if (inner == 0 || inner > (uint32_t)kWaveMaxInner) return false;
    // auto_band: -1 when (outer - inner) / outer > 0.5, which for lengths
    // below 2^31 is exactly 2 (outer - inner) > outer; otherwise w >= 200
    if (2 * (outer - inner) > outer || outer <= 200) return true;
    const int w = auto_band((int)rl, (int)ql);
    return w >= (int)outer;
}

__host__ __device__ __forceinline__ bool thin_tier_fits(uint32_t rl, uint32_t ql)
{
    if (ql < 1 || ql > (uint32_t)kThinMaxInner || rl <= ql) return false;
    if (small_tier_fits(rl, ql) || medium_tier_fits(rl, ql) || !wave_eligible(rl, ql)) return false;
    return (int64_t)rl + ql - 1 <= kThinMaxSteps;
}

// Square tier: a segment the band never binds with the shorter side <= 128
// that no tier above takes, whose directions (4 bits per cell, rows of
// ceil(inner / 8) words) fit the warp's scratch slot for 32 segments: rows x
// words <= kSquareRowWords.  One thread per segment, so its latency grows
// with the cells: above kSquareMaxCells the one-warp wavefront keeps it.
constexpr int kSquareMaxInner = 128;
constexpr int kSquareRowWords = 2048;  // 32 lanes x 2048 words x 4 B = one 256 KB slot
constexpr int kSquareMaxCells = 12288;
// default cell limit (launch knob 7): a lower limit moves the largest square
// segments to the wavefront tier, shortening the tier's per-sub-batch tail
// (measured equal device time on mito 100k and 5% faster host-buffer calls,
// which run the batch as six parts)
constexpr int kSquareDefaultCells = 3072;
constexpr int kSquareBins = 2048;      // sort bins of the square list

__host__ __device__ __forceinline__ bool square_tier_fits(uint32_t rl, uint32_t ql)
{
    const uint32_t inner = rl < ql ? rl : ql, outer = rl < ql ? ql : rl;
    if (inner < 1 || inner > (uint32_t)kSquareMaxInner || !wave_eligible(rl, ql)) return false;
    if ((uint64_t)rl * ql > (uint64_t)kSquareMaxCells) return false;
    return outer * ((inner + 7) / 8) <= (uint32_t)kSquareRowWords;
}

// Sort key of a square segment: rows x words class first (longest first), then
// orientation and gap mode, so a warp's 32 segments have similar loop bounds.
__host__ __device__ __forceinline__ uint32_t square_key(uint32_t rl, uint32_t ql, bool left)
{
    const uint32_t inner = rl < ql ? rl : ql, outer = rl < ql ? ql : rl;
    uint32_t cost = outer * ((inner + 3) / 4);  // state words touched per segment, <= 2 kSquareRowWords
    cost = cost > 4095 ? 4095 : cost;
    return (511u - (cost >> 3)) << 2 | (rl <= ql ? 1u : 0u) << 1 | (left ? 0u : 1u);
}

// Columns per lane of the one-warp wavefront: the smallest power of two with
// 32 x P >= inner.
__host__ __device__ __forceinline__ int wave_warp_cols(int inner)
{
    return inner <= 32 ? 1 : inner <= 64 ? 2 : inner <= 128 ? 4 : 8;
}

// Columns per lane of the CTA wavefront: 16 warps x 32 lanes x P >= inner.
__host__ __device__ __forceinline__ int wave_cta_cols(int inner)
{
    return inner <= 512 ? 1 : inner <= 1024 ? 2 : inner <= 2048 ? 4 : 8;
}

// Sort key of a one-warp wavefront segment: longest first by power-of-two
// class of rl + ql (the step count), so long segments do not start last;
// within a class widest first, then orientation and gap mode, so the warps
// of an SM run the same code together.
__host__ __device__ __forceinline__ uint32_t wave_key(uint32_t rl, uint32_t ql, bool left)
{
    const int inner = (int)(rl < ql ? rl : ql);
    const int P = wave_warp_cols(inner);
    const uint32_t pidx = P == 1 ? 0u : P == 2 ? 1u : P == 4 ? 2u : 3u;
    uint32_t cls = 0;
    for (uint32_t t = (rl + ql) >> 1; t && cls < 15; t >>= 1) ++cls;
    return (15u - cls) << 4 | (3u - pidx) << 2 | (rl <= ql ? 1u : 0u) << 1 | (left ? 0u : 1u);
}

// Small-tier work record, written in shape-sorted order by the sort pass so
// the DP reads it sequentially: absolute base position of the segment's
// query start in the packed stream, absolute op-word offset of its CIGAR
// slot, center start, shape and flags.
struct SmallRec {
    uint64_t qpos;      // poff[q] * 4 + qs
    uint32_t sid;       // segment id (the DP writes seg[sid].nops)
    uint32_t out;       // coff[q] + slot
    uint32_t rs;        // center start
    uint32_t shape;     // rl | ql << 8 | left << 16 | fast << 17 (fast: no query exception, plain center)
    uint32_t q;         // query index (exception lookups off the fast path)
    uint32_t pad;
};
constexpr uint32_t kRecLeft = 1u << 16, kRecFast = 1u << 17;

struct BatchDev {
    int n;                       // queries in the batch
    const uint8_t* packed;       // 2-bit packed bases
    const int64_t* poff;         // per-query byte offset (16-byte aligned)
    const int32_t* qlen;
    const int32_t* exc;          // exception runs: start, len, byte
    const int64_t* exc_off;      // per-query run range [exc_off[q], exc_off[q+1])
    const int32_t* order;        // processing order (longest first)
    // K1 seed
    const int64_t* hoff;         // per-query base into the hit arrays (capacity qlen-k+1)
    uint32_t* hit_pos;
    uint32_t* hit_ent;
    int32_t* n_hits;             // all minimizers of the query
    int32_t* n_matched;          // minimizers whose hash occurs in the center
    uint32_t* exact_list;        // queries whose window deque overflows (re-run sequentially)
    unsigned int* n_exact;
    int ring_slots;              // ring entries of the sequential re-run (2 w + 16)
    // K2 anchors (dynamic arena)
    uint32_t* a_ref;
    uint32_t* a_qry;
    int32_t* a_f;
    int32_t* a_p;
    int32_t* a_t;
    unsigned long long* a_tmp;   // 2 words per anchor: sort scratch
    int64_t acap;
    unsigned long long* a_cursor;
    int64_t* a_base;
    int32_t* a_n;
    uint32_t* ent_cnt;           // per-CTA query-side counters when n_ent is large
    // K3 chain + segments (dynamic arena)
    Seg* seg;
    int64_t scap;
    unsigned long long* s_cursor;
    int64_t* s_base;
    int32_t* s_n;
    int32_t* n_chain;
    int32_t* chain_meta;         // per query: best chain end (-1: none), first anchor whose speculated
                                 // predecessor was wrong (the anchor count if none); p is stored from there on
    int32_t thin_max_inner;      // tier boundaries (launch knobs): longest query side of the thin tier,
    int32_t square_max_cells;    // most cells of the square tier
    uint32_t* work_small;        // global segment ids per DP tier
    uint32_t* work_large;
    uint32_t* work_sorted;       // small tier sorted by shape_key (unused when work_rec is set)
    SmallRec* work_rec;          // small tier records in shape-sorted order
    uint32_t* work_key;          // shape_key of each work_small entry (written with it)
    uint32_t* shape_hist;        // kShapeBins counters, then kShapeBins cursors
    unsigned int* n_small;
    unsigned int* n_large;
    uint32_t* work_wave;         // one-warp wavefront tier, in chain order
    uint32_t* work_wave_key;     // its wave_key per entry
    uint32_t* work_wave_sorted;  // sorted by wave_key
    uint32_t* wave_hist;         // kWaveBins counters, then kWaveBins cursors
    uint32_t* work_wide;         // CTA wavefront tier
    unsigned int* n_wave;
    unsigned int* n_wide;
    uint32_t* work_thin;         // thin tier: segment ids, keys, sorted ids
    uint32_t* work_thin_key;
    uint32_t* work_thin_sorted;
    uint32_t* thin_hist;         // kThinBins counters, then kThinBins cursors
    unsigned int* n_thin;
    unsigned int* thin_q;        // kThinMaxInner queue heads of the thin tier, one per query length
    uint32_t* work_sq;           // square tier: segment ids, keys, sorted ids
    uint32_t* work_sq_key;
    uint32_t* work_sq_sorted;
    uint32_t* sq_hist;           // kSquareBins counters, then kSquareBins cursors
    unsigned int* n_sq;
    int64_t wcap;
    // K6 DP scratch: one reusable slot per large-tier warp, plus a bump arena
    // for segments whose scratch exceeds a slot
    uint8_t* dp_slots;
    uint8_t* thin_scratch;       // kThinWarpBytes per warp of the thin tier
    int thin_nwarps;
    int64_t dp_slot_bytes;
    int dp_nslots;
    uint8_t* dp_arena;
    int64_t dp_cap;
    unsigned long long* dp_cursor;
    // CIGARs
    const int64_t* coff;         // per-query base of the op scratch (capacity qlen + L + 4)
    uint32_t* cig_seg;           // per-segment ops, at coff[q] + seg.slot
    uint32_t* cig;               // merged CIGAR per query, at coff[q]
    int32_t* n_cig;
    uint8_t* has_ins;
    // rows + counters
    uint8_t* rows;               // n x L
    uint32_t* counts;            // L x 7 (A C G T U N -)
    uint32_t* ins;               // L + 1 insertion events
    uint32_t* status;            // per query
    unsigned int* queues;        // work-queue heads, one per stage
    unsigned int* queues2;       // [0] seed fast-path queue; [1] start of the medium small-tier records; [2] square queue;
                                 // [3] small-tier records (the small list without its holes)
    unsigned long long* cells;   // extz2 band cells computed: sum over DP calls of sum_r (en0 - st0 + 1)
    unsigned long long* match_cells;  // the part of `cells` in match segments (emitted without a DP)
    int small_pair;              // small tier: two records per thread in int16x2 halves (else int32, one)
    uint32_t* run_flags;         // OR of every query status since the last reset
};

// Hash-table probe; returns the entry id or kEmptyKey.
__device__ __forceinline__ uint32_t index_find(const IndexDev& ix, uint64_t h)
{
    uint32_t s = (uint32_t)h & ix.tab_mask;
    for (;;) {
        const ulonglong2 e = ix.tab[s];
        const uint64_t kk = e.x;
        if (kk == h) return (uint32_t)e.y;
        if (kk == kNoHash) return kEmptyKey;
        s = (s + 1) & ix.tab_mask;
    }
}

}  // namespace hg
