// hg_runtime.cu - host runtime behind the C ABI (include/halign_gb300.h).
//
// * hg_index: the resident center index.  The center's minimizers come from
//   the same seed kernel the queries use; the host groups them by hash,
//   derives the -f/-U occurrence threshold (anchor::compute_ref_occ_threshold,
//   src/seed/anchor.cpp:73-117) and uploads an open-addressing hash table.
//   The DP center is the consensus of the single center record
//   (pickConsensusChar, src/consensus/consensus.cpp:18-35: A/C/G/T/U keep
//   their letter, every other byte becomes 'A'), as RefAligner aligns queries
//   to consensus_seq while seeding from the raw record.
// * hg_ctx: one stream plus the sub-batch arenas in HBM.  A sub-batch runs as
//   one captured CUDA graph (control reset + 8 stage kernels); graphs are
//   cached per (batch view, size) and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <set>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/halign_gb300.h"
#include "hg_batch.cuh"
#include "hg_internal.h"

extern "C" {
cudaError_t hg_launch_seed(const hg::IndexDev*, const hg::BatchDev*, int, uint64_t*, uint64_t*, int, cudaStream_t);
cudaError_t hg_launch_anchor(const hg::IndexDev*, const hg::BatchDev*, int, cudaStream_t);
cudaError_t hg_launch_chain(const hg::IndexDev*, const hg::BatchDev*, int, cudaStream_t);
cudaError_t hg_launch_dp_small(const hg::IndexDev*, const hg::BatchDev*, int, cudaStream_t);
cudaError_t hg_launch_dp_large(const hg::IndexDev*, const hg::BatchDev*, int, cudaStream_t);
cudaError_t hg_launch_dp_wave(const hg::IndexDev*, const hg::BatchDev*, int, cudaStream_t);
cudaError_t hg_launch_dp_thin(const hg::IndexDev*, const hg::BatchDev*, int, cudaStream_t);
cudaError_t hg_launch_dp_wide(const hg::IndexDev*, const hg::BatchDev*, int, cudaStream_t);
cudaError_t hg_prepare_dp_kernels(void);
cudaError_t hg_launch_stitch(const hg::IndexDev*, const hg::BatchDev*, int, cudaStream_t);
cudaError_t hg_launch_rows(const hg::IndexDev*, const hg::BatchDev*, int64_t, int, cudaStream_t);
cudaError_t hg_launch_count(const uint8_t*, int64_t, int, int, uint32_t*, cudaStream_t);
cudaError_t hg_launch_status_or(const uint32_t*, int, uint32_t*, const unsigned long long*, const int32_t*,
                                unsigned long long*, cudaStream_t);
size_t hg_ksw_scratch_bytes(int, int, int, int);
cudaError_t hg_prepare_kernels(void);
cudaError_t hg_launch_ascii_pack(const uint8_t*, const int64_t*, int, const int64_t*, uint8_t*, int32_t*, int64_t*,
                                 int32_t*, int64_t, int32_t*, int, cudaStream_t);
cudaError_t hg_launch_ksw_single(int, const uint8_t*, int, const uint8_t*, int, const int8_t*, int, int, int, int,
                                 int, int, uint8_t*, uint32_t*, int, void*, cudaStream_t);
}

thread_local std::string g_err;

int hg::set_error(int code, const std::string& msg)
{
    g_err = msg;
    return code;
}

namespace {

using hg::DevBuf;

int fail(int code, const std::string& msg) { return hg::set_error(code, msg); }

int cuda_fail(cudaError_t e, const char* where) { return hg::cuda_error(e, where); }

uint8_t consensus_letter(uint8_t c)
{  // pickConsensusChar over one record's k_base_map category
    switch (c) {
    case 'A': case 'a': return 'A';
    case 'C': case 'c': return 'C';
    case 'G': case 'g': return 'G';
    case 'T': case 't': return 'T';
    case 'U': case 'u': return 'U';
    default: return 'A';
    }
}

int sm_count(int dev)
{
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

}  // namespace

struct hg_index {
    int device = 0;
    int k = 15, w = 10;
    hg_params_t prm{};
    std::string center_raw;
    int L = 0;
    uint64_t occ_thr = 0;
    int64_t n_hits = 0;
    DevBuf<uint8_t> center, center2;
    DevBuf<ulonglong2> tab;
    DevBuf<uint2> ent_meta;
    DevBuf<uint32_t> cpos, cspan;
    DevBuf<float> log2tab;
    hg::IndexDev dev{};
    hg_ctx_t* single = nullptr;  // lazily created context for single-query calls
    std::mutex single_mu;
};

struct SubPlan {
    int64_t first, n;      // queries [first, first+n)
    int64_t bases, bytes, excs;
};

struct GraphKey {
    hg::BatchDev b;
    bool operator<(const GraphKey& o) const { return std::memcmp(&b, &o.b, sizeof(b)) < 0; }
};

struct hg_ctx {
    hg_index_t* ix = nullptr;
    cudaStream_t st = nullptr;
    cudaStream_t st2 = nullptr;                            // side stream of the CTA wavefront tier
    cudaStream_t st3 = nullptr;                            // side stream of the one-warp wavefront and exact tiers
    // CTAs per SM of the seed, anchor, chain, dp_small, stitch and rows launches (hg_ctx_set_launch)
    int32_t launch[HG_LAUNCH_KNOBS] = {6, 6, 12, 12, 8, 6, hg::kThinMaxInner, hg::kSquareDefaultCells, 0, 2, 10};
    // second compute lane: a context of the same capacity on its own streams
    // that runs every other sub-batch of a multi-sub-batch run (knob 9 = 2)
    hg_ctx* peer = nullptr;
    cudaEvent_t lane_ev = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr, join3_ev = nullptr;
    int sms = 1;
    int64_t max_n = 0, max_bases = 0, exc_cap = 0;
    int64_t row_stride = 0;
    // inputs (one sub-batch)
    DevBuf<uint8_t> packed;
    DevBuf<int64_t> poff, exc_off, hoff, coff;
    DevBuf<int32_t> qlen, exc, order;
    // stage arenas
    DevBuf<uint32_t> hit_pos, hit_ent;
    DevBuf<int32_t> n_hits, n_matched;
    DevBuf<uint32_t> exact_list;
    int64_t acap = 0;
    DevBuf<uint32_t> a_ref, a_qry;
    DevBuf<int32_t> a_f, a_p, a_t, a_n;
    DevBuf<unsigned long long> a_tmp;
    DevBuf<int64_t> a_base;
    DevBuf<uint32_t> ent_cnt;
    int64_t scap = 0;
    DevBuf<hg::Seg> seg;
    DevBuf<int64_t> s_base;
    DevBuf<int32_t> s_n, n_chain, chain_meta;
    DevBuf<uint32_t> work_small, work_large, work_sorted, work_key, shape_hist;
    DevBuf<uint32_t> work_wave, work_wave_key, work_wave_sorted, wave_hist, work_wide;
    DevBuf<uint32_t> work_thin, work_thin_key, work_thin_sorted;  // thin_hist lives in wave_hist
    DevBuf<uint32_t> work_sq, work_sq_key, work_sq_sorted;        // and so does sq_hist
    DevBuf<hg::SmallRec> work_rec;
    int64_t dp_cap = 0;
    DevBuf<uint8_t> dp_arena;
    int64_t dp_slot_bytes = 0;
    int dp_nslots = 0;
    DevBuf<uint8_t> dp_slots;
    DevBuf<uint8_t> thin_scratch;  // direction nibbles of the thin tier, one region per warp
    int thin_nwarps = 0;
    DevBuf<uint32_t> run_flags;
    int64_t cig_cap = 0;
    DevBuf<uint32_t> cig_seg, cig;
    DevBuf<int32_t> n_cig;
    DevBuf<uint8_t> has_ins;
    DevBuf<uint8_t> rows, rows2;                         // rows2: second buffer while rows of the previous sub-batch copy out
    cudaStream_t cst = nullptr;                          // copy stream for row read-back
    cudaEvent_t rows_ev[4] = {nullptr, nullptr, nullptr, nullptr}, comp_ev = nullptr;  // one per row buffer
    DevBuf<uint32_t> counts, ins, status;
    // control block: queues[8], cursors (a, s, dp), n_small, n_large
    DevBuf<unsigned long long> control;
    DevBuf<unsigned long long> cells;  // accumulated DP cells (GCUPS numerator)
    DevBuf<unsigned long long> work;   // accumulated anchors, segment records, DP segments
    // compaction
    DevBuf<int64_t> cig_off;
    DevBuf<uint32_t> cig_compact;
    // pipelined host-buffer path (hg_align_batch over several sub-batches):
    // the second input set and compaction buffer (slot 0 uses the ones above),
    // pinned per-slot copies of the offsets, status and insertion flags, and
    // the events between the input stream, the compute stream and the copy stream
    struct PipeSlot {
        DevBuf<uint8_t> packed;
        DevBuf<int64_t> poff, exc_off, hoff, coff;
        DevBuf<int32_t> qlen, exc, order;
        DevBuf<uint32_t> compact;
        // ASCII input (hg_align_ascii): the sub-batch's bytes and offsets,
        // run counts, the exception-capacity flag and its pinned copy
        DevBuf<uint8_t> ascii;
        DevBuf<int64_t> aoff;
        DevBuf<int32_t> nrun, excflag;
        int32_t* h_excflag = nullptr;
        // pinned staging of the small per-query input arrays (offsets,
        // order, lengths): uploads from it run asynchronously and touch no
        // fresh pageable pages
        int64_t* h_in64 = nullptr;  // 5 (max_n + 1): poff, exc_off, hoff, coff, ASCII offsets
        int32_t* h_in32 = nullptr;  // 2 max_n: order, lengths
        int64_t* h_off = nullptr;
        uint32_t* h_status = nullptr;
        uint8_t* h_ins = nullptr;
        cudaEvent_t in_ready = nullptr, in_free = nullptr, off_ev = nullptr, done = nullptr, cfree = nullptr;
    } pipe[4];  // slot 0's device inputs are the context's own
    cudaStream_t ist = nullptr;
    int pipe_slots = 0;  // slots set up
    // staged full batch (device-resident form)
    std::vector<SubPlan> staged_plan;
    std::vector<int32_t> staged_qlen;
    DevBuf<uint8_t> s_packed;
    DevBuf<int64_t> s_poff, s_exc_off, s_hoff, s_coff;
    DevBuf<int32_t> s_qlen, s_exc, s_order;
    bool staged = false;
    // staged outputs for fetch
    DevBuf<int32_t> s_n_cig;
    DevBuf<uint8_t> s_has_ins, s_rows;
    DevBuf<uint32_t> s_status, s_cig;
    DevBuf<int64_t> s_cigoff_dev;
    int64_t s_cig_cap = 0;
    std::map<GraphKey, cudaGraphExec_t> graphs;
    std::set<GraphKey> graph_seen;  // sub-batch shapes launched once without a graph
    // host arrays of the pipelined host-buffer path, per input slot, kept
    // across calls so a call does not allocate (and fault in) fresh pages
    std::vector<int32_t> pl_order[4], pl_qlen;
    std::vector<int64_t> pl_hoff[4], pl_coff[4], pl_spoff[4];
    // asynchronous form: pinned staging + completion event
    uint8_t* h_packed = nullptr;
    int64_t* h_i64 = nullptr;      // poff, exc_off, hoff, coff, cig_off (5 x (max_n + 1))
    int32_t* h_i32 = nullptr;      // qlen, order, exc (2 x max_n + exc_cap x 3)
    uint8_t* h_has_ins = nullptr;
    uint32_t* h_status = nullptr;
    // the batch's compacted CIGARs, written by the device straight into
    // mapped pinned memory at the end of the batch (up to h_cig_cap ops), so
    // a collect needs no device work when they fit
    uint32_t* h_cig = nullptr;
    uint32_t* h_cig_dev = nullptr;
    int64_t h_cig_cap = 0;
    cudaEvent_t done_ev = nullptr;     // blocking-sync: a waiting host thread sleeps instead of spinning
    cudaEvent_t collected_ev = nullptr;
    int64_t async_n = -1;
    bool async_ascii = false;   // the batch in flight is packed on the device (its capacity flag is read back)
    bool async_exc_over = false;  // the last hg_collect failed on that flag
    bool timing = false;
    cudaEvent_t ev[10] = {};
    cudaEvent_t run_ev[2] = {};
    bool run_recorded = false;
    float last_total_ms = 0, last_stage_ms[8] = {};
    int64_t last_launches = 0, last_cells = 0;
    int lanes_used = 1;  // lanes of the last staged run
};

extern "C" const char* hg_last_error(void) { return g_err.c_str(); }

extern "C" int hg_device_count(void)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

extern "C" int hg_set_device(int ordinal)
{
    const int n = hg_device_count();
    if (ordinal < 0 || ordinal >= n) return fail(HG_ERR_ARG, "hg_set_device: ordinal out of range");
    const cudaError_t e = cudaSetDevice(ordinal);
    if (e != cudaSuccess) return cuda_fail(e, "hg_set_device");
    return HG_OK;
}

extern "C" void hg_default_params(hg_params_t* p)
{
    p->f_top_frac = 2e-4;
    p->u_floor = 10;
    p->u_ceil = 1000000;
    p->q_occ_frac = 0.01;
    p->sample_every_bp = 500;
    p->max_dist_x = 5000;
    p->max_dist_y = 5000;
    p->bw = 500;
    p->max_skip = 25;
    p->max_iter = 5000;
    p->min_cnt = 3;
    p->min_score = 40;
    p->gap_penalty = 0.01f;
    p->skip_penalty = 0.01f;
}

// ------------------------------------------------------------------ packing

namespace {
struct PackLut {
    uint8_t code[256];
    PackLut()
    {
        for (int i = 0; i < 256; ++i) code[i] = 0xff;
        code['A'] = 0, code['C'] = 1, code['G'] = 2, code['T'] = 3;
    }
};
const PackLut kPackLut;
}  // namespace

namespace {

// Eight ASCII bytes -> 16 bits of 2-bit codes (base j at bits 2j) when all
// eight are A/C/G/T: ((c >> 1) ^ (c >> 2)) & 3 maps A C G T to 0 1 2 3, and
// rebuilding the bytes from the codes (0x41 + 2 b0 + 6 b1 + 11 b0 b1)
// confirms the input.  Returns false (out untouched) otherwise.
inline bool pack8(const unsigned char* s, uint32_t* out16)
{
    uint64_t w;
    std::memcpy(&w, s, 8);
    const uint64_t c = ((w >> 1) ^ (w >> 2)) & 0x0303030303030303ULL;
    const uint64_t b0 = c & 0x0101010101010101ULL, b1 = (c >> 1) & 0x0101010101010101ULL;
    const uint64_t e = 0x4141414141414141ULL + 2 * b0 + 6 * b1 + 11 * (b0 & b1);
    if (e != w) return false;
    uint64_t x = c;
    x = (x | (x >> 6)) & 0x000F000F000F000FULL;
    x = (x | (x >> 12)) & 0x000000FF000000FFULL;
    x = (x | (x >> 24)) & 0xFFFFULL;
    *out16 = (uint32_t)x;
    return true;
}

// Pack one query into `out` (nullptr: only detect exceptions).  Returns
// whether any byte is not A/C/G/T (such bytes pack as 0).
bool pack_one(const unsigned char* s, int64_t len, uint8_t* out)
{
    const uint8_t* lut = kPackLut.code;
    bool any_exc = false;
    int64_t j = 0;
    for (; j + 8 <= len; j += 8) {
        uint32_t v;
        if (pack8(s + j, &v)) {
            if (out) out[j >> 2] = (uint8_t)v, out[(j >> 2) + 1] = (uint8_t)(v >> 8);
            continue;
        }
        any_exc = true;
        if (!out) continue;
        for (int64_t t = j; t < j + 8; t += 4) {
            const uint32_t c0 = lut[s[t]], c1 = lut[s[t + 1]], c2 = lut[s[t + 2]], c3 = lut[s[t + 3]];
            const uint32_t m0 = c0 < 4 ? c0 : 0, m1 = c1 < 4 ? c1 : 0, m2 = c2 < 4 ? c2 : 0, m3 = c3 < 4 ? c3 : 0;
            out[t >> 2] = (uint8_t)(m0 | m1 << 2 | m2 << 4 | m3 << 6);
        }
    }
    for (; j < len; j += 4) {
        uint32_t byte = 0;
        for (int64_t t = j; t < len && t < j + 4; ++t) {
            const uint32_t c = lut[s[t]];
            if (c > 3) any_exc = true;
            else byte |= c << ((t - j) * 2);
        }
        if (out) out[j >> 2] = (uint8_t)byte;
    }
    return any_exc;
}

}  // namespace

namespace {

// Exception runs (maximal runs of one non-A/C/G/T byte) of one query; writes
// them to `exc` when it is given.  Returns the number of runs.
int64_t exc_runs(const unsigned char* s, int64_t len, int32_t* exc)
{
    const uint8_t* lut = kPackLut.code;
    int64_t ne = 0, run_start = -1;
    unsigned char run_byte = 0;
    for (int64_t t = 0; t <= len; ++t) {
        const bool isx = t < len && lut[s[t]] > 3;
        if (run_start >= 0 && (!isx || s[t] != run_byte)) {
            if (exc) exc[ne * 3] = (int32_t)run_start, exc[ne * 3 + 1] = (int32_t)(t - run_start),
                     exc[ne * 3 + 2] = run_byte;
            ++ne;
            run_start = -1;
        }
        if (isx && run_start < 0) run_start = t, run_byte = s[t];
    }
    return ne;
}

}  // namespace

// Queries are packed independently (OpenMP over queries).  Padded byte
// offsets follow from the lengths alone.  With `packed` given, one pass packs
// the bases and counts the exception runs of the queries that hold any; a
// second pass over only those queries writes the runs.  With packed == NULL a
// pass only counts (sizes for a caller that allocates everything up front).
extern "C" int hg_pack(const char* seqs, const int64_t* offsets, int64_t n, uint8_t* packed, int64_t packed_cap,
                       int64_t* poff, int32_t* exc, int64_t exc_cap, int64_t* exc_off, int64_t* packed_bytes,
                       int64_t* n_exc)
{
    if (n < 0 || !offsets) return fail(HG_ERR_ARG, "hg_pack: bad arguments");
    for (int64_t i = 0; i < n; ++i) {
        const int64_t len = offsets[i + 1] - offsets[i];
        if (len < 0 || len > INT32_MAX) return fail(HG_ERR_ARG, "hg_pack: bad query length");
    }
    const unsigned char* base = reinterpret_cast<const unsigned char*>(seqs);
    std::vector<int64_t> qoff((size_t)n);
    int64_t pb = 0;
    for (int64_t i = 0; i < n; ++i) {
        qoff[(size_t)i] = pb;
        pb += (((offsets[i + 1] - offsets[i]) + 3) / 4 + 15) / 16 * 16;
    }
    if (packed_bytes) *packed_bytes = pb;
    if (packed && pb > packed_cap) return fail(HG_ERR_CAPACITY, "hg_pack: packed buffer too small");
    std::vector<int64_t> nrun((size_t)n);
    const bool par = n >= 64;
#pragma omp parallel for schedule(dynamic, 16) if (par)
    for (int64_t i = 0; i < n; ++i) {
        const unsigned char* s = base + offsets[i];
        const int64_t len = offsets[i + 1] - offsets[i];
        uint8_t* out = packed ? packed + qoff[(size_t)i] : nullptr;
        // 4 bases per byte; an exception byte packs as 0 and is listed as a run
        const bool any_exc = pack_one(s, len, out);
        if (out) {
            poff[i] = qoff[(size_t)i];
            const int64_t used = (len + 3) / 4, nbytes = (used + 15) / 16 * 16;
            std::memset(out + used, 0, (size_t)(nbytes - used));
        }
        nrun[(size_t)i] = any_exc ? exc_runs(s, len, nullptr) : 0;
    }
    std::vector<int64_t> eo((size_t)n + 1);
    int64_t ne = 0;
    for (int64_t i = 0; i < n; ++i) eo[(size_t)i] = ne, ne += nrun[(size_t)i];
    eo[(size_t)n] = ne;
    if (n_exc) *n_exc = ne;
    if (exc_off)
        for (int64_t i = 0; i <= n; ++i) exc_off[i] = eo[(size_t)i];
    if (!packed) return HG_OK;
    if (ne > exc_cap || (ne > 0 && !exc)) return fail(HG_ERR_CAPACITY, "hg_pack: exception buffer too small");
    if (ne == 0) return HG_OK;
#pragma omp parallel for schedule(dynamic, 16) if (par)
    for (int64_t i = 0; i < n; ++i)
        if (nrun[(size_t)i]) exc_runs(base + offsets[i], offsets[i + 1] - offsets[i], exc + 3 * eo[(size_t)i]);
    return HG_OK;
}

// ------------------------------------------------------------------- index

namespace {

}  // namespace

uint64_t hg::occ_threshold(std::vector<uint64_t> occs, const hg_params_t& p)
{  // compute_ref_occ_threshold (src/seed/anchor.cpp:73-117)
    uint64_t f_cut;
    if (occs.empty() || p.f_top_frac <= 0.0) f_cut = UINT64_MAX;
    else if (p.f_top_frac >= 1.0) f_cut = 1;
    else {
        const uint64_t n_skip = (uint64_t)std::floor(p.f_top_frac * (double)occs.size());
        if (n_skip == 0) f_cut = UINT64_MAX;
        else {
            std::nth_element(occs.begin(), occs.begin() + (n_skip - 1), occs.end(), std::greater<uint64_t>());
            f_cut = occs[n_skip - 1];
        }
    }
    const uint64_t capped = std::min(p.u_ceil, f_cut);
    return std::max(p.u_floor, capped);
}

extern "C" uint64_t hg_occ_threshold(const uint64_t* occs, int64_t n, const hg_params_t* params,
                                     uint64_t* cutoff_top_frac)
{
    hg_params_t p;
    if (params) p = *params;
    else hg_default_params(&p);
    std::vector<uint64_t> v(occs, occs + (n > 0 ? n : 0));
    if (cutoff_top_frac) {
        hg_params_t q = p;  // the -f cutoff alone: no -U bounds
        q.u_floor = 0, q.u_ceil = UINT64_MAX;
        *cutoff_top_frac = hg::occ_threshold(v, q);
    }
    return hg::occ_threshold(std::move(v), p);
}

std::vector<float> hg::log2_table(int n)
{
    std::vector<float> lg((size_t)n);
    for (int i = 0; i < n; ++i) lg[i] = i >= 1 ? (float)std::log2((double)i) : 0.0f;
    return lg;
}

extern "C" int hg_index_create(const char* center, int64_t len, int k, int w, const hg_params_t* params,
                               hg_index_t** out)
{
    return hg::index_create(center, len, k, w, params, true, out);
}

int hg::index_create(const char* center, int64_t len, int k, int w, const hg_params_t* params, bool dp_consensus,
                     hg_index_t** out)
{
    if (!out || !center || len <= 0 || len > INT32_MAX) return fail(HG_ERR_ARG, "hg_index_create: bad arguments");
    if (k <= 0 || k > 31 || w <= 0 || w >= 256) return fail(HG_ERR_ARG, "hg_index_create: need 0<k<=31, 0<w<256");
    if (hg_device_count() <= 0) return fail(HG_ERR_CUDA, "hg_index_create: no CUDA device");
    auto* ix = new hg_index();
    cudaGetDevice(&ix->device);
    ix->k = k, ix->w = w;
    if (params) ix->prm = *params;
    else hg_default_params(&ix->prm);
    ix->center_raw.assign(center, (size_t)len);
    ix->L = (int)len;
    std::vector<uint64_t> xs, ys;
    int r = hg::run_extract(k, w, 1, center, len, xs, ys);
    if (r) {
        delete ix;
        return r;
    }
    ix->n_hits = (int64_t)xs.size();
    // group by (hash, rid, pos, strand) = (hash, pos) for one forward center
    std::vector<uint32_t> idx(xs.size());
    std::iota(idx.begin(), idx.end(), 0u);
    std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) {
        const uint64_t ha = xs[a] >> 8, hb = xs[b] >> 8;
        if (ha != hb) return ha < hb;
        return (uint32_t)ys[a] < (uint32_t)ys[b];
    });
    std::vector<uint32_t> cpos(idx.size()), cspan(idx.size()), est, ecnt;
    std::vector<uint64_t> ekey, occs;
    for (size_t i = 0; i < idx.size(); ++i) {
        cpos[i] = (uint32_t)ys[idx[i]];
        cspan[i] = (uint32_t)(xs[idx[i]] & 0xff);
        const uint64_t h = xs[idx[i]] >> 8;
        if (i == 0 || h != ekey.back()) {
            ekey.push_back(h);
            est.push_back((uint32_t)i);
            ecnt.push_back(0);
        }
        ecnt.back()++;
    }
    for (auto c : ecnt) occs.push_back(c);
    ix->occ_thr = hg::occ_threshold(occs, ix->prm);
    std::vector<uint8_t> over(ekey.size());
    for (size_t e = 0; e < ekey.size(); ++e) over[e] = ecnt[e] > ix->occ_thr ? 1 : 0;
    uint32_t tsize = 16;
    while (tsize < 2 * ekey.size() + 16) tsize <<= 1;
    std::vector<uint64_t> tkey(tsize, hg::kNoHash);
    std::vector<uint32_t> tval(tsize, 0);
    for (size_t e = 0; e < ekey.size(); ++e) {
        uint32_t s = (uint32_t)ekey[e] & (tsize - 1);
        while (tkey[s] != hg::kNoHash) s = (s + 1) & (tsize - 1);
        tkey[s] = ekey[e], tval[s] = (uint32_t)e;
    }
    std::vector<ulonglong2> tab(tsize);
    for (uint32_t i = 0; i < tsize; ++i) tab[i].x = tkey[i], tab[i].y = tval[i];
    // DP center in DNA5 codes: the consensus of the single record (one
    // center), or the record itself (one reference of several)
    std::vector<uint8_t> cdp((size_t)len);
    for (int64_t i = 0; i < len; ++i)
        cdp[i] = hg::dna5_of(dp_consensus ? consensus_letter((uint8_t)center[i]) : (uint8_t)center[i]);
    // 2-bit copy for the small DP tier's register loads (64 bytes of slack: it reads 24 bytes at a time)
    std::vector<uint8_t> c2((size_t)(len + 3) / 4 + 64, 0);
    int cplain = 1;
    for (int64_t i = 0; i < len; ++i) {
        if (cdp[i] > 3) cplain = 0;
        c2[(size_t)i >> 2] |= (uint8_t)((cdp[i] & 3u) << (2 * (i & 3)));
    }
    // log2f table for the chain penalty (arguments 2 .. bw+1)
    const int nlog = std::max(ix->prm.bw + 2, 513);
    const std::vector<float> lg = hg::log2_table(nlog);
    // per entry: its center position when it occurs once (the common case),
    // else its start in cpos; the occurrence count with the over-threshold bit
    std::vector<uint2> meta(ekey.size());
    for (size_t e = 0; e < ekey.size(); ++e) {
        meta[e].x = ecnt[e] == 1 ? cpos[est[e]] : est[e];
        meta[e].y = ecnt[e] | (over[e] ? 0x80000000u : 0u);
    }
    auto up = [&](auto& buf, const auto& v) -> cudaError_t {
        cudaError_t e = buf.alloc(std::max<size_t>(v.size(), 1));
        if (e != cudaSuccess) return e;
        return v.empty() ? cudaSuccess
                         : cudaMemcpy(buf.p, v.data(), sizeof(v[0]) * v.size(), cudaMemcpyHostToDevice);
    };
    cudaError_t e = cudaSuccess;
    if ((e = up(ix->center, cdp)) || (e = up(ix->center2, c2)) || (e = up(ix->tab, tab)) ||
        (e = up(ix->ent_meta, meta)) ||
        (e = up(ix->cpos, cpos)) || (e = up(ix->cspan, cspan)) || (e = up(ix->log2tab, lg))) {
        delete ix;
        return cuda_fail(e, "hg_index_create: upload");
    }
    hg::IndexDev& d = ix->dev;
    d.L = (int)len, d.k = k, d.w = w, d.non_canonical = 1;
    d.center = ix->center.p, d.center2 = ix->center2.p, d.center_plain = cplain;
    d.tab = ix->tab.p, d.tab_mask = tsize - 1;
    d.n_ent = (uint32_t)ekey.size();
    d.ent_meta = ix->ent_meta.p;
    d.cpos = ix->cpos.p, d.cspan = ix->cspan.p;
    d.q_occ_frac = ix->prm.q_occ_frac, d.sample_every = ix->prm.sample_every_bp;
    d.max_dist_x = ix->prm.max_dist_x, d.max_dist_y = ix->prm.max_dist_y, d.bw = ix->prm.bw;
    d.max_skip = ix->prm.max_skip, d.max_iter = ix->prm.max_iter, d.min_cnt = ix->prm.min_cnt;
    d.min_score = ix->prm.min_score, d.gap_pen = ix->prm.gap_penalty, d.skip_pen = ix->prm.skip_penalty;
    d.log2tab = ix->log2tab.p, d.n_log2 = nlog;
    // largest dg whose penalty (dd = 0) truncates to 0, evaluated as the kernel
    // does: separate round-to-nearest products and sums
    {
        int z = k;
        for (int dg = k + 1; dg <= (1 << 20); ++dg) {
            volatile float a = ix->prm.gap_penalty * 0.0f;
            volatile float c = ix->prm.skip_penalty * (float)dg;
            volatile float lin = a + c;
            volatile float h = 0.5f * 0.0f;
            volatile float t = lin + h;
            if ((int)t != 0) break;
            z = dg;
        }
        d.dg_nopen = z;
    }
    *out = ix;
    return HG_OK;
}

extern "C" void hg_index_destroy(hg_index_t* ix)
{
    if (!ix) return;
    cudaSetDevice(ix->device);
    if (ix->single) hg_ctx_destroy(ix->single);
    ix->center.free(), ix->tab.free(), ix->ent_meta.free();
    ix->cpos.free(), ix->cspan.free(), ix->log2tab.free(), ix->center2.free();
    delete ix;
}

int64_t hg::index_length(const hg_index_t* ix) { return ix ? ix->L : 0; }

extern "C" int hg_index_device(const hg_index_t* ix, int* ordinal, char* pci_bus_id, int len)
{
    if (!ix) return fail(HG_ERR_ARG, "hg_index_device: null index");
    if (ordinal) *ordinal = ix->device;
    if (pci_bus_id && len > 0) {
        const cudaError_t e = cudaDeviceGetPCIBusId(pci_bus_id, len, ix->device);
        if (e != cudaSuccess) return cuda_fail(e, "hg_index_device");
    }
    return HG_OK;
}

extern "C" int hg_index_info(const hg_index_t* ix, int64_t* n_distinct, int64_t* n_hits, uint64_t* occ_threshold)
{
    if (!ix) return fail(HG_ERR_ARG, "hg_index_info: null index");
    if (n_distinct) *n_distinct = ix->dev.n_ent;
    if (n_hits) *n_hits = ix->n_hits;
    if (occ_threshold) *occ_threshold = ix->occ_thr;
    return HG_OK;
}

// ----------------------------------------------------------------- context

namespace {

constexpr int kControlWords = 32;
// control words: queues[8] | a_cursor | s_cursor | dp_cursor | n_small | n_large | n_exact | n_wave | n_wide |
// queues2[4] | n_thin | n_sq | thin_q[32]
// sort counters of the one-warp wavefront list, then of the thin list (counters and cursors each)
constexpr size_t kSortHistWords = 2 * (size_t)hg::kWaveBins + 2 * (size_t)hg::kThinBins + 2 * (size_t)hg::kSquareBins;
constexpr int kLargeBlocksPerSm = 4;  // dp_large grid = SMs x 4 CTAs x 4 warps
constexpr int kWaveBlocksPerSm = 4;
constexpr int kThinWarpsPerSm = 16;   // dp_wave grid = SMs x 4 CTAs x 4 warps (one checkpoint slot per warp)
// kernel launches per sub-batch: seed 3, anchor, chain, dp_small 5, thin 2, square + dp_wave 4,
// dp_wide, dp_large, stitch, rows, count, status (the per-query plain form has no status pass)
constexpr int kLaunchesBatch = 23;
constexpr size_t kMaxGraphs = 64;  // cached sub-batch graphs (and first-seen shapes) per context
constexpr int kLaunchesPlain = 22;

__global__ void compact_offsets_kernel(const int32_t* n_cig, int n, int64_t* off)
{
    // single CTA exclusive scan over n entries
    __shared__ int64_t part[1024];
    const int tid = threadIdx.x;
    const int per = (n + 1023) / 1024;
    const int i0 = min(tid * per, n), i1 = min(i0 + per, n);
    int64_t s = 0;
    for (int i = i0; i < i1; ++i) s += n_cig[i];
    part[tid] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const int64_t v = tid >= o ? part[tid - o] : 0;
        __syncthreads();
        part[tid] += v;
        __syncthreads();
    }
    int64_t run = part[tid] - s;
    for (int i = i0; i < i1; ++i) {
        off[i] = run;
        run += n_cig[i];
    }
    if (tid == 1023) off[n] = part[1023];
}

__global__ void compact_copy_kernel(const uint32_t* cig, const int64_t* coff, const int32_t* n_cig,
                                    const int64_t* off, int n, uint32_t* out, int64_t out_cap, int64_t out_base)
{
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int q = w; q < n; q += nw) {
        const int64_t o = off[q] - out_base;
        const int m = n_cig[q];
        for (int i = lane; i < m; i += 32)
            if (o + i >= 0 && o + i < out_cap) out[o + i] = cig[coff[q] + i];
    }
}

size_t padded_bytes(int64_t len) { return (size_t)(((len + 3) / 4 + 15) / 16 * 16); }

}  // namespace

extern "C" int hg_ctx_create(hg_index_t* ix, int64_t max_queries, int64_t max_bases, hg_ctx_t** out)
{
    if (!ix || !out || max_queries <= 0 || max_bases <= 0) return fail(HG_ERR_ARG, "hg_ctx_create: bad arguments");
    auto* c = new hg_ctx();
    c->ix = ix;
    cudaSetDevice(ix->device);
    cudaError_t pe = hg_prepare_kernels();
    if (pe == cudaSuccess) pe = hg_prepare_dp_kernels();
    if (pe != cudaSuccess) {
        delete c;
        return cuda_fail(pe, "hg_ctx_create: kernel attributes");
    }
    c->sms = sm_count(ix->device);
    c->max_n = max_queries, c->max_bases = max_bases;
    c->exc_cap = max_bases / 16 + 4096;
    const int64_t L = ix->L;
    c->row_stride = (L + 15) / 16 * 16;
    c->acap = max_bases / 4 + 65536;
    c->scap = max_bases / 2 + 4 * max_queries + 65536;
    c->dp_cap = std::max<int64_t>((int64_t)1 << 30, max_bases);
    c->dp_slot_bytes = (int64_t)256 << 10;
    c->dp_nslots = c->sms * kLargeBlocksPerSm * 4 + c->sms;  // warp slots, then one per CTA-tier CTA
    // thin tier: 16 warps per SM, fewer for a small context (a warp takes 2+ segments at a time)
    c->thin_nwarps = (int)std::min<int64_t>((int64_t)c->sms * kThinWarpsPerSm, (max_queries + 3) / 4 * 4);
    c->cig_cap = max_bases + max_queries * (L + 4);
    if (c->cig_cap >= ((int64_t)1 << 32)) {  // SmallRec holds 32-bit op offsets
        delete c;
        return fail(HG_ERR_ARG, "hg_ctx_create: max_bases + max_queries * (center length + 4) must stay below 2^32");
    }
    const int64_t n_ent = ix->dev.n_ent;
    const int grid_anchor = c->sms * 6;  // the anchor kernel's largest grid
    cudaError_t e = cudaSuccess;
    if ((e = cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking)) ||
        (e = cudaStreamCreateWithFlags(&c->st2, cudaStreamNonBlocking)) ||
        (e = cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming)) ||
        (e = cudaEventCreateWithFlags(&c->join_ev, cudaEventDisableTiming)) ||
        (e = cudaStreamCreateWithFlags(&c->st3, cudaStreamNonBlocking)) ||
        (e = cudaEventCreateWithFlags(&c->join3_ev, cudaEventDisableTiming)) ||
        (e = cudaStreamCreateWithFlags(&c->cst, cudaStreamNonBlocking)) ||
        (e = cudaEventCreateWithFlags(&c->rows_ev[0], cudaEventDisableTiming)) ||
        (e = cudaEventCreateWithFlags(&c->rows_ev[1], cudaEventDisableTiming)) ||
        (e = cudaEventCreateWithFlags(&c->rows_ev[2], cudaEventDisableTiming)) ||
        (e = cudaEventCreateWithFlags(&c->rows_ev[3], cudaEventDisableTiming)) ||
        (e = cudaEventCreateWithFlags(&c->comp_ev, cudaEventDisableTiming)) ||
        (e = c->packed.alloc(max_bases / 4 + 16 * max_queries + 64)) || (e = c->poff.alloc(max_queries)) ||
        (e = c->exc_off.alloc(max_queries + 1)) || (e = c->hoff.alloc(max_queries)) ||
        (e = c->coff.alloc(max_queries)) || (e = c->qlen.alloc(max_queries)) ||
        (e = c->exc.alloc(c->exc_cap * 3)) || (e = c->order.alloc(max_queries)) ||
        (e = c->hit_pos.alloc(max_bases)) || (e = c->hit_ent.alloc(max_bases)) ||
        (e = c->n_hits.alloc(max_queries)) || (e = c->n_matched.alloc(max_queries)) ||
        (e = c->exact_list.alloc(max_queries)) ||
        (e = c->a_ref.alloc(c->acap)) || (e = c->a_qry.alloc(c->acap)) || (e = c->a_f.alloc(c->acap)) ||
        (e = c->a_p.alloc(c->acap)) || (e = c->a_t.alloc(c->acap)) || (e = c->a_tmp.alloc(2 * c->acap)) ||
        (e = c->a_base.alloc(max_queries)) || (e = c->a_n.alloc(max_queries)) ||
        (e = c->ent_cnt.alloc(n_ent > 8192 ? (size_t)grid_anchor * n_ent : 1)) || (e = c->seg.alloc(c->scap)) ||
        (e = c->s_base.alloc(max_queries)) || (e = c->s_n.alloc(max_queries)) ||
        (e = c->n_chain.alloc(max_queries)) || (e = c->chain_meta.alloc(2 * max_queries)) || (e = c->work_small.alloc(c->scap)) ||
        (e = c->work_large.alloc(c->scap)) || (e = c->dp_arena.alloc(c->dp_cap)) ||
        (e = c->work_sorted.alloc(c->scap)) || (e = c->work_key.alloc(c->scap)) ||
        (e = c->shape_hist.alloc(2 * (size_t)hg::kShapeBins)) ||
        (e = c->work_wave.alloc(c->scap)) || (e = c->work_wave_key.alloc(c->scap)) ||
        (e = c->work_wave_sorted.alloc(c->scap)) || (e = c->wave_hist.alloc(kSortHistWords)) ||
        (e = c->work_thin.alloc(c->scap)) || (e = c->work_thin_key.alloc(c->scap)) ||
        (e = c->work_thin_sorted.alloc(c->scap)) || (e = c->work_sq.alloc(c->scap)) ||
        (e = c->work_sq_key.alloc(c->scap)) || (e = c->work_sq_sorted.alloc(c->scap)) ||
        (e = c->work_wide.alloc(c->scap)) || (e = c->work_rec.alloc(c->scap)) ||
        (e = c->dp_slots.alloc((size_t)c->dp_nslots * c->dp_slot_bytes)) ||
        (e = c->thin_scratch.alloc((size_t)c->thin_nwarps * hg::kThinWarpBytes)) || (e = c->run_flags.alloc(1)) ||
        (e = c->cig_seg.alloc(c->cig_cap)) || (e = c->cig.alloc(c->cig_cap)) ||
        (e = c->n_cig.alloc(max_queries)) || (e = c->has_ins.alloc(max_queries)) ||
        (e = c->rows.alloc((size_t)max_queries * c->row_stride)) || (e = c->counts.alloc(L * 7)) ||
        (e = c->ins.alloc(L + 1)) || (e = c->status.alloc(max_queries)) || (e = c->control.alloc(kControlWords)) || (e = c->cells.alloc(2)) || (e = c->work.alloc(4)) ||
        (e = c->cig_off.alloc(max_queries + 1)) || (e = c->cig_compact.alloc(max_bases / 4 + 1024))) {
        hg_ctx_destroy(c);
        return cuda_fail(e, "hg_ctx_create: device allocation");
    }
    if (n_ent > 8192 && (e = cudaMemset(c->ent_cnt.p, 0, sizeof(uint32_t) * (size_t)grid_anchor * n_ent))) {
        hg_ctx_destroy(c);
        return cuda_fail(e, "hg_ctx_create: memset");
    }
    cudaMemset(c->counts.p, 0, sizeof(uint32_t) * L * 7);
    cudaMemset(c->cells.p, 0, 2 * sizeof(unsigned long long));
    cudaMemset(c->work.p, 0, 4 * sizeof(unsigned long long));
    cudaMemset(c->ins.p, 0, sizeof(uint32_t) * (L + 1));
    for (auto& ev : c->ev) cudaEventCreate(&ev);
    for (auto& ev : c->run_ev) cudaEventCreate(&ev);
    *out = c;
    return HG_OK;
}

// Launch shape of the sub-batch stages (CTAs per SM); bounds keep every
// per-CTA scratch slice in range.  Cached graphs are dropped.
extern "C" int hg_ctx_set_launch(hg_ctx_t* c, const int32_t* ctas_per_sm, int n)
{
    static const int32_t lo[HG_LAUNCH_KNOBS] = {1, 1, 1, 1, 1, 1, 0, 0, 0, 1, 0};
    static const int32_t hi[HG_LAUNCH_KNOBS] = {32, 6, 64, 32, 32, 32, hg::kThinMaxInner, hg::kSquareMaxCells, 1, 2, 24};
    if (!c || !ctas_per_sm || n < 0 || n > HG_LAUNCH_KNOBS) return fail(HG_ERR_ARG, "hg_ctx_set_launch: bad arguments");
    for (int i = 0; i < n; ++i)
        if (ctas_per_sm[i] < lo[i] || ctas_per_sm[i] > hi[i])
            return fail(HG_ERR_ARG, "hg_ctx_set_launch: knob " + std::to_string(i) + " out of range");
    cudaStreamSynchronize(c->st);
    for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second);
    c->graphs.clear();
    for (int i = 0; i < n; ++i) c->launch[i] = ctas_per_sm[i];
    if (c->peer) {
        const int r = hg_ctx_set_launch(c->peer, ctas_per_sm, n);
        c->peer->launch[9] = 1;  // the second lane never opens a third
        return r;
    }
    return HG_OK;
}

extern "C" int hg_ctx_get_launch(const hg_ctx_t* c, int32_t* ctas_per_sm, int n)
{
    if (!c || !ctas_per_sm || n < 0 || n > HG_LAUNCH_KNOBS) return fail(HG_ERR_ARG, "hg_ctx_get_launch: bad arguments");
    for (int i = 0; i < n; ++i) ctas_per_sm[i] = c->launch[i];
    return HG_OK;
}

extern "C" void hg_ctx_destroy(hg_ctx_t* c)
{
    if (!c) return;
    cudaSetDevice(c->ix->device);
    if (c->peer) hg_ctx_destroy(c->peer), c->peer = nullptr;
    if (c->lane_ev) cudaEventDestroy(c->lane_ev);
    if (c->st) cudaStreamSynchronize(c->st);
    for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second);
    if (c->h_packed) cudaFreeHost(c->h_packed);
    if (c->h_cig) cudaFreeHost(c->h_cig);
    if (c->h_i64) cudaFreeHost(c->h_i64);
    if (c->h_i32) cudaFreeHost(c->h_i32);
    if (c->h_has_ins) cudaFreeHost(c->h_has_ins);
    if (c->h_status) cudaFreeHost(c->h_status);
    if (c->done_ev) cudaEventDestroy(c->done_ev);
    if (c->collected_ev) cudaEventDestroy(c->collected_ev);
    if (c->ist) cudaStreamSynchronize(c->ist), cudaStreamDestroy(c->ist);
    for (auto& ps : c->pipe) {
        if (ps.h_off) cudaFreeHost(ps.h_off);
        if (ps.h_status) cudaFreeHost(ps.h_status);
        if (ps.h_ins) cudaFreeHost(ps.h_ins);
        if (ps.h_excflag) cudaFreeHost(ps.h_excflag);
        if (ps.h_in64) cudaFreeHost(ps.h_in64);
        if (ps.h_in32) cudaFreeHost(ps.h_in32);
        for (cudaEvent_t e : {ps.in_ready, ps.in_free, ps.off_ev, ps.done, ps.cfree})
            if (e) cudaEventDestroy(e);
    }
    for (auto& ev : c->ev)
        if (ev) cudaEventDestroy(ev);
    for (auto& ev : c->run_ev)
        if (ev) cudaEventDestroy(ev);
    if (c->fork_ev) cudaEventDestroy(c->fork_ev);
    if (c->cst) cudaStreamSynchronize(c->cst), cudaStreamDestroy(c->cst);
    for (auto& ev : c->rows_ev)
        if (ev) cudaEventDestroy(ev);
    if (c->comp_ev) cudaEventDestroy(c->comp_ev);
    if (c->join_ev) cudaEventDestroy(c->join_ev);
    if (c->join3_ev) cudaEventDestroy(c->join3_ev);
    if (c->st3) cudaStreamDestroy(c->st3);
    if (c->st2) cudaStreamDestroy(c->st2);
    if (c->st) cudaStreamDestroy(c->st);
    delete c;  // DevBuf members are freed below via explicit frees
}

namespace {

// Plan sub-batches bounded by the context capacities.
std::vector<SubPlan> plan(hg_ctx_t* c, const int64_t* poff, const int32_t* qlen, const int64_t* exc_off, int64_t n)
{
    std::vector<SubPlan> out;
    int64_t i = 0;
    while (i < n) {
        SubPlan p{i, 0, 0, 0, 0};
        while (i < n) {
            const int64_t b = qlen[i], by = (int64_t)padded_bytes(qlen[i]);
            const int64_t ex = exc_off ? exc_off[i + 1] - exc_off[i] : 0;  // ASCII input: checked on the device
            if (p.n > 0 && (p.n + 1 > c->max_n || p.bases + b > c->max_bases ||
                            p.bytes + by > (int64_t)c->packed.n || p.excs + ex > c->exc_cap))
                break;
            p.n++, p.bases += b, p.bytes += by, p.excs += ex, ++i;
        }
        out.push_back(p);
    }
    (void)poff;
    return out;
}

// Host-buffer calls: the first sub-batch's inputs upload before anything
// computes, and the last sub-batches' outputs (the rows above all) copy out
// after everything has.  With s = launch knob 10 (0 = off) and at least
// 32 MB to move, the edges are re-cut into small parts: the first two
// sub-batches' queries into parts of s, s, 50 - s and 50 - s percent of
// their bases, the last two into 50 - s, 50 - s, s and s percent (with
// three sub-batches or fewer, all queries into s, s, 50 - 2s, 50 - 2s, s
// and s percent).  The two lanes then start after a small upload each, and
// the large parts' outputs copy out while the small last parts compute.  A
// cut that would exceed the context's capacity keeps the sub-batches.
std::vector<SubPlan> edge_split(hg_ctx_t* c, const std::vector<SubPlan>& plans, const int32_t* qlen,
                                const int64_t* exc_off, bool rows, bool ascii)
{
    const size_t K = plans.size();
    const int64_t s = c->launch[10];
    if (K == 0 || s <= 0) return plans;
    const int64_t n = plans[K - 1].first + plans[K - 1].n - plans[0].first;
    int64_t bases = 0;
    for (const SubPlan& p : plans) bases += p.bases;
    const int64_t moved = (rows ? n * c->row_stride : 0) + (ascii ? bases : bases / 4);
    if (n < 16 || moved < (32LL << 20)) return plans;
    bool ok = true;
    // queries [f, e) cut at the given cumulative percentages of their bases
    auto recut = [&](int64_t f, int64_t e, std::initializer_list<int64_t> pct, std::vector<SubPlan>& out) {
        int64_t B = 0;
        for (int64_t i = f; i < e; ++i) B += qlen[i];
        int64_t i = f, acc = 0, cum = 0;
        const size_t np = pct.size();
        size_t part = 0;
        for (int64_t p_pct : pct) {
            cum += p_pct;
            const int64_t lim = B * cum / 100;
            const bool last = ++part == np;
            SubPlan p{i, 0, 0, 0, 0};
            while (i < e && (p.n == 0 || last || acc + qlen[i] <= lim)) {
                const int64_t by = (int64_t)padded_bytes(qlen[i]), ex = exc_off ? exc_off[i + 1] - exc_off[i] : 0;
                p.n++, p.bases += qlen[i], p.bytes += by, p.excs += ex, acc += qlen[i], ++i;
            }
            if (!p.n) continue;
            if (p.n > c->max_n || p.bases > c->max_bases || p.bytes > (int64_t)c->packed.n || p.excs > c->exc_cap)
                ok = false;
            out.push_back(p);
        }
    };
    std::vector<SubPlan> out;
    auto end_of = [&](size_t k) { return plans[k].first + plans[k].n; };
    if (K <= 3) {
        recut(plans[0].first, end_of(K - 1), {s, s, 50 - 2 * s, 50 - 2 * s, s, s}, out);
    } else {
        recut(plans[0].first, end_of(1), {s, s, 50 - s, 50 - s}, out);
        out.insert(out.end(), plans.begin() + 2, plans.end() - 2);
        recut(plans[K - 2].first, end_of(K - 1), {50 - s, 50 - s, s, s}, out);
    }
    return ok ? out : plans;
}

hg::BatchDev batch_view(hg_ctx_t* c, int n, const uint8_t* packed, const int64_t* poff, const int32_t* qlen,
                        const int32_t* exc, const int64_t* exc_off, const int32_t* order, const int64_t* hoff,
                        const int64_t* coff)
{
    hg::BatchDev b;
    std::memset(&b, 0, sizeof(b));  // graph cache keys compare the raw bytes
    b.n = n;
    b.packed = packed, b.poff = poff, b.qlen = qlen, b.exc = exc, b.exc_off = exc_off, b.order = order;
    b.hoff = hoff, b.hit_pos = c->hit_pos.p, b.hit_ent = c->hit_ent.p, b.n_hits = c->n_hits.p,
    b.n_matched = c->n_matched.p;
    b.exact_list = c->exact_list.p;
    b.ring_slots = 2 * c->ix->w + 16;
    b.a_ref = c->a_ref.p, b.a_qry = c->a_qry.p, b.a_f = c->a_f.p, b.a_p = c->a_p.p, b.a_t = c->a_t.p,
    b.a_tmp = c->a_tmp.p;
    b.acap = c->acap;
    unsigned long long* ctl = c->control.p;
    b.queues = reinterpret_cast<unsigned int*>(ctl);  // 8 x uint32 in words 0..3
    b.queues2 = reinterpret_cast<unsigned int*>(ctl + 12);  // 4 x uint32 in words 12..13
    b.a_cursor = ctl + 4, b.s_cursor = ctl + 5, b.dp_cursor = ctl + 6;
    b.n_small = reinterpret_cast<unsigned int*>(ctl + 7);
    b.n_large = reinterpret_cast<unsigned int*>(ctl + 8);
    b.n_exact = reinterpret_cast<unsigned int*>(ctl + 9);
    b.cells = c->cells.p;
    b.match_cells = c->cells.p + 1;
    b.a_base = c->a_base.p, b.a_n = c->a_n.p, b.ent_cnt = c->ent_cnt.p;
    b.seg = c->seg.p, b.scap = c->scap, b.s_base = c->s_base.p, b.s_n = c->s_n.p, b.n_chain = c->n_chain.p;
    b.chain_meta = c->chain_meta.p;
    b.thin_max_inner = c->launch[6], b.square_max_cells = c->launch[7];
    b.small_pair = c->launch[8];
    b.work_small = c->work_small.p, b.work_large = c->work_large.p, b.wcap = c->scap;
    b.work_sorted = c->work_sorted.p, b.work_key = c->work_key.p, b.shape_hist = c->shape_hist.p;
    b.work_wave = c->work_wave.p, b.work_wave_key = c->work_wave_key.p, b.work_wave_sorted = c->work_wave_sorted.p;
    b.wave_hist = c->wave_hist.p, b.work_wide = c->work_wide.p, b.work_rec = c->work_rec.p;
    b.n_wave = reinterpret_cast<unsigned int*>(ctl + 10);
    b.n_wide = reinterpret_cast<unsigned int*>(ctl + 11);
    b.n_thin = reinterpret_cast<unsigned int*>(ctl + 14);
    b.thin_q = reinterpret_cast<unsigned int*>(ctl + 16);  // 32 x uint32 in words 16..31
    b.work_thin = c->work_thin.p, b.work_thin_key = c->work_thin_key.p, b.work_thin_sorted = c->work_thin_sorted.p;
    b.thin_hist = c->wave_hist.p + 2 * hg::kWaveBins;
    b.work_sq = c->work_sq.p, b.work_sq_key = c->work_sq_key.p, b.work_sq_sorted = c->work_sq_sorted.p;
    b.sq_hist = c->wave_hist.p + 2 * hg::kWaveBins + 2 * hg::kThinBins;
    b.n_sq = reinterpret_cast<unsigned int*>(ctl + 15);
    b.dp_arena = c->dp_arena.p, b.dp_cap = c->dp_cap;
    b.dp_slots = c->dp_slots.p, b.dp_slot_bytes = c->dp_slot_bytes, b.dp_nslots = c->dp_nslots;
    b.thin_scratch = c->thin_scratch.p, b.thin_nwarps = c->thin_nwarps;
    b.run_flags = c->run_flags.p;
    b.coff = coff, b.cig_seg = c->cig_seg.p, b.cig = c->cig.p, b.n_cig = c->n_cig.p, b.has_ins = c->has_ins.p;
    b.rows = c->rows.p, b.counts = c->counts.p, b.ins = c->ins.p, b.status = c->status.p;
    return b;
}

const char* kStageNames[8] = {"seed", "anchor", "chain", "dp_small", "dp_large", "stitch", "rows", "count"};

// Enqueue the stage sequence of one sub-batch.
int enqueue_stages(hg_ctx_t* c, const hg::BatchDev& b, bool timed)
{
    const hg::IndexDev& ix = c->ix->dev;
    const int S = c->sms;
    cudaStream_t st = c->st;
    HG_CUDA(cudaMemsetAsync(c->control.p, 0, sizeof(unsigned long long) * kControlWords, st));
    HG_CUDA(cudaMemsetAsync(c->status.p, 0, sizeof(uint32_t) * (size_t)b.n, st));
    HG_CUDA(cudaMemsetAsync(c->shape_hist.p, 0, sizeof(uint32_t) * hg::kShapeBins, st));
    HG_CUDA(cudaMemsetAsync(c->wave_hist.p, 0, sizeof(uint32_t) * kSortHistWords, st));
    const int n = b.n;
    auto mark = [&](int i) -> cudaError_t { return timed ? cudaEventRecord(c->ev[i], st) : cudaSuccess; };
    HG_CUDA(mark(0));
    const int32_t* K = c->launch;
    HG_CUDA(hg_launch_seed(&ix, &b, 0, nullptr, nullptr, std::min(n, S * K[0]), st));
    HG_CUDA(mark(1));
    HG_CUDA(hg_launch_anchor(&ix, &b, std::min(n, S * K[1]), st));
    HG_CUDA(mark(2));
    HG_CUDA(hg_launch_chain(&ix, &b, std::max(1, std::min((n + 3) / 4, S * K[2])), st));
    HG_CUDA(mark(3));
    // the DP tiers are independent work lists with disjoint scratch: the CTA
    // wavefront tier runs on st2, the one-warp wavefront and exact tiers on
    // st3, the small and thin tiers on st (their tails overlap)
    HG_CUDA(cudaEventRecord(c->fork_ev, st));
    HG_CUDA(cudaStreamWaitEvent(c->st2, c->fork_ev, 0));
    HG_CUDA(cudaStreamWaitEvent(c->st3, c->fork_ev, 0));
    HG_CUDA(hg_launch_dp_wide(&ix, &b, S, c->st2));
    HG_CUDA(cudaEventRecord(c->join_ev, c->st2));
    HG_CUDA(hg_launch_dp_wave(&ix, &b, S * kWaveBlocksPerSm, c->st3));
    HG_CUDA(hg_launch_dp_large(&ix, &b, S * kLargeBlocksPerSm, c->st3));
    HG_CUDA(cudaEventRecord(c->join3_ev, c->st3));
    HG_CUDA(hg_launch_dp_small(&ix, &b, S * K[3], st));
    HG_CUDA(hg_launch_dp_thin(&ix, &b, S * kWaveBlocksPerSm, st));
    HG_CUDA(mark(4));
    HG_CUDA(cudaStreamWaitEvent(st, c->join_ev, 0));
    HG_CUDA(cudaStreamWaitEvent(st, c->join3_ev, 0));
    HG_CUDA(mark(5));
    HG_CUDA(hg_launch_stitch(&ix, &b, std::max(1, std::min((n + 3) / 4, S * K[4])), st));
    HG_CUDA(mark(6));
    HG_CUDA(hg_launch_rows(&ix, &b, c->row_stride, std::max(1, std::min((n + 7) / 8, S * K[5])), st));
    HG_CUDA(mark(7));
    HG_CUDA(hg_launch_count(b.rows, c->row_stride, n, ix.L, c->counts.p, st));
    HG_CUDA(mark(8));
    HG_CUDA(hg_launch_status_or(c->status.p, n, c->run_flags.p, c->control.p, b.s_n, c->work.p, st));
    (void)kStageNames;
    return HG_OK;
}

// The second compute lane of a multi-sub-batch run (nullptr: one lane).  The
// peer is created on first use with the context's capacity and launch
// knobs; when the device has no room for it the context stays at one lane.
hg_ctx_t* lane_peer(hg_ctx_t* c)
{
    if (c->launch[9] < 2) return nullptr;
    if (!c->peer) {
        hg_ctx_t* p = nullptr;
        const std::string saved = g_err;
        // the second lane must leave room: at least an eighth of the device
        // (and 16 GB) free after it, for the host-buffer path's second input
        // set and the caller's other work
        size_t free_b = 0, total_b = 0;
        bool ok = hg_ctx_create(c->ix, c->max_n, c->max_bases, &p) == HG_OK &&
                  cudaMemGetInfo(&free_b, &total_b) == cudaSuccess &&
                  free_b >= std::max<size_t>(total_b / 8, (size_t)16 << 30);
        if (ok && !c->lane_ev) ok = cudaEventCreateWithFlags(&c->lane_ev, cudaEventDisableTiming) == cudaSuccess;
        if (!ok) {
            if (p) hg_ctx_destroy(p);
            cudaGetLastError();
            g_err = saved;
            c->launch[9] = 1;
            return nullptr;
        }
        std::copy(c->launch, c->launch + HG_LAUNCH_KNOBS, p->launch);
        p->launch[9] = 1;
        c->peer = p;
    }
    return c->peer;
}

int run_sub(hg_ctx_t* c, const hg::BatchDev& b, bool use_graph)
{
    if (c->timing || !use_graph) {
        int r = enqueue_stages(c, b, c->timing);
        if (r) return r;
        if (c->timing) {
            HG_CUDA(cudaEventSynchronize(c->ev[8]));
            float tot = 0;
            for (int i = 0; i < 8; ++i) {
                float ms = 0;
                cudaEventElapsedTime(&ms, c->ev[i], c->ev[i + 1]);
                c->last_stage_ms[i] += ms;
                tot += ms;
            }
            c->last_total_ms += tot;
        }
        c->last_launches += kLaunchesBatch;
        return HG_OK;
    }
    GraphKey key{b};
    auto it = c->graphs.find(key);
    if (it == c->graphs.end()) {
        // a sub-batch shape seen for the first time launches its stages
        // directly (capture + instantiation cost more than one run); its
        // graph is captured when the shape comes again.  Both sets are
        // bounded (a stream of ever-new shapes starts them over).
        if (c->graph_seen.size() >= kMaxGraphs) c->graph_seen.clear();
        if (c->graph_seen.insert(key).second) {
            int r = enqueue_stages(c, b, false);
            if (r) return r;
            c->last_launches += kLaunchesBatch;
            return HG_OK;
        }
        if (c->graphs.size() >= kMaxGraphs) {  // an in-flight graph is freed when it completes
            for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second);
            c->graphs.clear();
        }
        cudaGraph_t g;
        HG_CUDA(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
        int r = enqueue_stages(c, b, false);
        cudaError_t e = cudaStreamEndCapture(c->st, &g);
        if (r) return r;
        if (e != cudaSuccess) return cuda_fail(e, "graph capture");
        cudaGraphExec_t ge;
        e = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_fail(e, "graph instantiate");
        it = c->graphs.emplace(key, ge).first;
    }
    HG_CUDA(cudaGraphLaunch(it->second, c->st));
    c->last_launches += kLaunchesBatch;
    return HG_OK;
}

// Host-side per-query arrays of a sub-batch.
void sub_arrays(hg_ctx_t* c, const int32_t* qlen, int64_t n, std::vector<int32_t>& order, std::vector<int64_t>& hoff,
                std::vector<int64_t>& coff)
{
    const int k = c->ix->k;
    const int64_t L = c->ix->L;
    order.resize(n), hoff.resize(n), coff.resize(n);
    std::iota(order.begin(), order.end(), 0);
    // longest first, ties in input order (std::sort in place: no temporary
    // buffer, so no page faults on the per-call path)
    std::sort(order.begin(), order.end(), [&](int a, int b) { return qlen[a] > qlen[b] || (qlen[a] == qlen[b] && a < b); });
    int64_t h = 0, co = 0;
    for (int64_t i = 0; i < n; ++i) {
        hoff[i] = h;
        h += std::max<int64_t>(qlen[i] - k + 1, 0);
        coff[i] = co;
        co += qlen[i] + L + 4;
    }
}

// Copy back outputs of a finished sub-batch (compacted CIGARs).
int fetch_outputs(hg_ctx_t* c, int n, const int64_t* d_coff, uint32_t* cigar, int64_t cigar_cap, int64_t cig_base, int64_t* cigar_off,
                  uint8_t* has_ins, uint8_t* rows, int64_t row_stride, uint32_t* status, int64_t* total_out,
                  const uint8_t* d_rows)
{
    compact_offsets_kernel<<<1, 1024, 0, c->st>>>(c->n_cig.p, n, c->cig_off.p);
    HG_CUDA(cudaGetLastError());
    std::vector<int64_t> off((size_t)n + 1);
    HG_CUDA(cudaMemcpyAsync(off.data(), c->cig_off.p, 8 * ((size_t)n + 1), cudaMemcpyDeviceToHost, c->st));
    if (status) HG_CUDA(cudaMemcpyAsync(status, c->status.p, 4 * (size_t)n, cudaMemcpyDeviceToHost, c->st));
    if (has_ins) HG_CUDA(cudaMemcpyAsync(has_ins, c->has_ins.p, (size_t)n, cudaMemcpyDeviceToHost, c->st));
    if (rows) {
        // row read-back runs on the copy stream, overlapping the next sub-batch
        const int64_t L = c->ix->L;
        const int slot = (d_rows == c->rows2.p && c->rows2.p) ? 1 : 0;
        HG_CUDA(cudaEventRecord(c->comp_ev, c->st));
        HG_CUDA(cudaStreamWaitEvent(c->cst, c->comp_ev, 0));
        if ((int64_t)row_stride == c->row_stride)
            HG_CUDA(cudaMemcpyAsync(rows, d_rows, (size_t)row_stride * (size_t)n, cudaMemcpyDeviceToHost, c->cst));
        else
            HG_CUDA(cudaMemcpy2DAsync(rows, (size_t)row_stride, d_rows, (size_t)c->row_stride, (size_t)L, (size_t)n,
                                      cudaMemcpyDeviceToHost, c->cst));
        HG_CUDA(cudaEventRecord(c->rows_ev[slot], c->cst));
    }
    HG_CUDA(cudaStreamSynchronize(c->st));
    const int64_t total = off[n];
    if (cig_base + total > cigar_cap) return fail(HG_ERR_CAPACITY, "hg_align_batch: cigar buffer too small");
    // copy in pieces through the compact buffer
    const int64_t piece = (int64_t)c->cig_compact.n;
    for (int64_t done = 0; done < total; done += piece) {
        const int64_t m = std::min(piece, total - done);
        compact_copy_kernel<<<c->sms * 4, 256, 0, c->st>>>(c->cig.p, d_coff, c->n_cig.p, c->cig_off.p, n,
                                                           c->cig_compact.p, m, done);
        HG_CUDA(cudaGetLastError());
        HG_CUDA(cudaMemcpyAsync(cigar + cig_base + done, c->cig_compact.p, 4 * (size_t)m, cudaMemcpyDeviceToHost,
                                c->st));
    }
    HG_CUDA(cudaStreamSynchronize(c->st));
    for (int i = 0; i <= n; ++i) cigar_off[i] = cig_base + off[i];
    *total_out = total;
    return HG_OK;
}

int status_error(const uint32_t* status, int64_t n)
{
    for (int64_t i = 0; i < n; ++i) {
        if (status[i] & HG_ST_ARENA_OVERFLOW)
            return fail(HG_ERR_CAPACITY, "query " + std::to_string(i) + ": device arena overflow (raise the context capacity)");
        if (status[i] & HG_ST_CIGAR_OVERFLOW) return fail(HG_ERR_CIGAR, "query " + std::to_string(i) + ": CIGAR length overflow");
        if (status[i] & (HG_ST_LENGTH_MISMATCH | HG_ST_PARTIAL_CIGAR))
            return fail(HG_ERR_LENGTH_MISMATCH,
                        "Sequence length mismatch: query " + std::to_string(i) + " does not span the center");
    }
    return HG_OK;
}

// Device input set and compaction buffer of pipeline slot 0 or 1.
struct InView {
    uint8_t* packed;
    int64_t *poff, *exc_off, *hoff, *coff;
    int32_t *qlen, *exc, *order;
    uint32_t* compact;
    size_t compact_n;
};

InView in_view(hg_ctx_t* c, int slot)
{
    if (slot == 0)
        return {c->packed.p, c->poff.p, c->exc_off.p, c->hoff.p, c->coff.p, c->qlen.p, c->exc.p, c->order.p,
                c->cig_compact.p, c->cig_compact.n};
    auto& q = c->pipe[slot];
    return {q.packed.p, q.poff.p, q.exc_off.p, q.hoff.p, q.coff.p, q.qlen.p, q.exc.p, q.order.p, q.compact.p, q.compact.n};
}

// Input slots 0 .. want-1 (2 or 4), set up on first use: device inputs
// (slot 0 uses the context's own), pinned read-back staging and events.
// Returns the slots available: 4 only when their memory could be had.
int pipe_setup(hg_ctx_t* c, int want, int* have)
{
    const size_t M = (size_t)c->max_n;
    cudaError_t e;
    if (!c->ist && (e = cudaStreamCreateWithFlags(&c->ist, cudaStreamNonBlocking)))
        return cuda_fail(e, "hg_align_batch: input stream");
    for (int s = c->pipe_slots; s < want; ++s) {
        auto& q = c->pipe[s];
        if (s > 0 && ((e = q.packed.alloc(c->packed.n)) || (e = q.poff.alloc(M)) || (e = q.exc_off.alloc(M + 1)) ||
                      (e = q.hoff.alloc(M)) || (e = q.coff.alloc(M)) || (e = q.qlen.alloc(M)) ||
                      (e = q.exc.alloc(c->exc.n)) || (e = q.order.alloc(M)) || (e = q.compact.alloc(c->cig_compact.n)))) {
            q.packed.free(), q.poff.free(), q.exc_off.free(), q.hoff.free(), q.coff.free(), q.qlen.free();
            q.exc.free(), q.order.free(), q.compact.free();
            cudaGetLastError();
            if (s >= 2) break;  // two slots are enough to run
            return cuda_fail(e, "hg_align_batch: pipeline buffers");
        }
        if ((e = cudaHostAlloc(&q.h_in64, 8 * 5 * (M + 1), cudaHostAllocDefault)) ||
            (e = cudaHostAlloc(&q.h_in32, 4 * 2 * M, cudaHostAllocDefault)) ||
            (e = cudaHostAlloc(&q.h_off, 8 * (M + 1), cudaHostAllocDefault)) ||
            (e = cudaHostAlloc(&q.h_status, 4 * M, cudaHostAllocDefault)) ||
            (e = cudaHostAlloc(&q.h_ins, M, cudaHostAllocDefault)))
            return cuda_fail(e, "hg_align_batch: pinned pipeline staging");
        for (cudaEvent_t* ev : {&q.in_ready, &q.in_free, &q.off_ev, &q.done, &q.cfree})
            if ((e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming))) return cuda_fail(e, "hg_align_batch: events");
        c->pipe_slots = s + 1;
    }
    *have = std::min(want, c->pipe_slots);
    return HG_OK;
}

// Buffers of the ASCII input form, per pipeline slot (allocated on first use).
int ascii_setup(hg_ctx_t* c, int slots)
{
    const size_t M = (size_t)c->max_n;
    for (int s = 0; s < slots; ++s) {
        auto& ps = c->pipe[s];
        if (ps.ascii.p) continue;
        cudaError_t e;
        if ((e = ps.ascii.alloc((size_t)c->max_bases + 16)) || (e = ps.aoff.alloc(M + 1)) || (e = ps.nrun.alloc(M)) ||
            (e = ps.excflag.alloc(1)) || (e = cudaHostAlloc(&ps.h_excflag, 4, cudaHostAllocDefault))) {
            ps.ascii.free();
            return cuda_fail(e, "hg_align_ascii: input buffers");
        }
    }
    return HG_OK;
}

// hg_align_batch over several sub-batches: sub-batch k+1's inputs upload on
// the input stream while k computes; after k the compute stream compacts
// its CIGARs into the slot's buffer (bounded by its size) and copies the
// offsets, status and flags to pinned memory; the host reads the offsets
// before launching k+1 (the uncompacted CIGAR scratch is still intact
// then, so a sub-batch whose CIGARs exceed the buffer is copied in pieces
// instead), and the compacted CIGARs and the rows copy out on the copy
// stream while k+1 computes.
int align_pipelined(hg_ctx_t* c, const std::vector<SubPlan>& plans, const uint8_t* packed, const int64_t* poff,
                    const int32_t* qlen, const int32_t* exc, const int64_t* exc_off, int64_t n, uint32_t* cigar,
                    int64_t cigar_cap, int64_t* cigar_off, uint8_t* has_ins, uint8_t* rows, int64_t row_stride,
                    uint32_t* status, const uint8_t* ascii = nullptr, const int64_t* aoffs = nullptr)
{
    const int K = (int)plans.size();
    // lanes: with two, the odd sub-batches compute on the second lane's
    // arenas and streams; four input slots (two per lane) let a lane's next
    // inputs upload while it computes
    hg_ctx_t* P = K > 1 ? lane_peer(c) : nullptr;
    int NS = 2;
    int r = pipe_setup(c, P && K > 2 ? 4 : 2, &NS);
    if (r) return r;
    if (NS != 4) NS = 2;
    if (ascii && (r = ascii_setup(c, NS))) return r;
    auto slot_of = [&](int k) { return k % NS; };
    if (rows && !c->rows2.p) HG_CUDA(c->rows2.alloc((size_t)c->max_n * c->row_stride));
    // per-slot host arrays kept by the context across calls (grown once)
    std::vector<int32_t>* order = c->pl_order;
    std::vector<int64_t>*hoff = c->pl_hoff, *coff = c->pl_coff, *spoff = c->pl_spoff;
    for (const SubPlan& sp : plans)
        if (sp.n > c->max_n || sp.bases > c->max_bases)
            return fail(HG_ERR_CAPACITY, "query " + std::to_string(sp.first) + " exceeds the context capacity");
    auto issue_inputs = [&](int k) -> int {
        const SubPlan& sp = plans[(size_t)k];
        const int slot = slot_of(k);
        const InView V = in_view(c, slot);
        const int64_t f = sp.first, m = sp.n;
        sub_arrays(c, qlen + f, m, order[slot], hoff[slot], coff[slot]);
        spoff[slot].resize((size_t)m);
        int64_t pb = 0;
        for (int64_t i = 0; i < m; ++i) spoff[slot][i] = pb, pb += (int64_t)padded_bytes(qlen[f + i]);
        cudaStream_t is = c->ist;
        auto& PS = c->pipe[slot];
        // the slot's staging is rewritten only after its last upload has run
        HG_CUDA(cudaEventSynchronize(PS.in_ready));
        const size_t M1 = (size_t)c->max_n + 1;
        int64_t *s_poff = PS.h_in64, *s_eoff = PS.h_in64 + M1, *s_hoff = PS.h_in64 + 2 * M1,
                *s_coff = PS.h_in64 + 3 * M1, *s_aoff = PS.h_in64 + 4 * M1;
        int32_t *s_order = PS.h_in32, *s_qlen = PS.h_in32 + (M1 - 1);
        std::memcpy(s_poff, spoff[slot].data(), 8 * (size_t)m);
        std::memcpy(s_hoff, hoff[slot].data(), 8 * (size_t)m);
        std::memcpy(s_coff, coff[slot].data(), 8 * (size_t)m);
        std::memcpy(s_order, order[slot].data(), 4 * (size_t)m);
        std::memcpy(s_qlen, qlen + f, 4 * (size_t)m);
        HG_CUDA(cudaStreamWaitEvent(is, PS.in_free, 0));  // sub-batch k-NS is done with the slot
        if (ascii) {  // the bytes as they are; the compute stream packs them
            std::memcpy(s_aoff, aoffs + f, 8 * ((size_t)m + 1));
            HG_CUDA(cudaMemcpyAsync(PS.ascii.p, ascii + aoffs[f], (size_t)(aoffs[f + m] - aoffs[f]),
                                    cudaMemcpyHostToDevice, is));
            HG_CUDA(cudaMemcpyAsync(PS.aoff.p, s_aoff, 8 * ((size_t)m + 1), cudaMemcpyHostToDevice, is));
        } else {
            for (int64_t i = 0; i <= m; ++i) s_eoff[i] = exc_off[f + i] - exc_off[f];
            bool contiguous = true;
            for (int64_t i = 1; i < m && contiguous; ++i) contiguous = poff[f + i] == poff[f] + spoff[slot][i];
            if (contiguous) {
                HG_CUDA(cudaMemcpyAsync(V.packed, packed + poff[f], (size_t)pb, cudaMemcpyHostToDevice, is));
            } else {
                for (int64_t i = 0; i < m; ++i)
                    HG_CUDA(cudaMemcpyAsync(V.packed + spoff[slot][i], packed + poff[f + i],
                                            padded_bytes(qlen[f + i]), cudaMemcpyHostToDevice, is));
            }
            const int64_t ne = s_eoff[m];
            if (ne) HG_CUDA(cudaMemcpyAsync(V.exc, exc + 3 * exc_off[f], 12 * (size_t)ne, cudaMemcpyHostToDevice, is));
            HG_CUDA(cudaMemcpyAsync(V.exc_off, s_eoff, 8 * ((size_t)m + 1), cudaMemcpyHostToDevice, is));
        }
        HG_CUDA(cudaMemcpyAsync(V.poff, s_poff, 8 * (size_t)m, cudaMemcpyHostToDevice, is));
        HG_CUDA(cudaMemcpyAsync(V.qlen, s_qlen, 4 * (size_t)m, cudaMemcpyHostToDevice, is));
        HG_CUDA(cudaMemcpyAsync(V.order, s_order, 4 * (size_t)m, cudaMemcpyHostToDevice, is));
        HG_CUDA(cudaMemcpyAsync(V.hoff, s_hoff, 8 * (size_t)m, cudaMemcpyHostToDevice, is));
        HG_CUDA(cudaMemcpyAsync(V.coff, s_coff, 8 * (size_t)m, cudaMemcpyHostToDevice, is));
        HG_CUDA(cudaEventRecord(PS.in_ready, is));
        return HG_OK;
    };
    auto lane_of = [&](int k) -> hg_ctx_t* { return (P && (k & 1)) ? P : c; };
    // row buffers: with two lanes each lane alternates between two of them
    // when it runs more than one sub-batch, so no sub-batch waits for the
    // read-back of the one before it on its lane
    bool rows4 = false;
    if (rows && P && K > 2) {
        if (!P->rows2.p && P->rows2.alloc((size_t)P->max_n * P->row_stride) != cudaSuccess) {
            P->rows2.p = nullptr, P->rows2.n = 0;
            cudaGetLastError();
        }
        rows4 = P->rows2.p != nullptr;
    }
    auto rbuf_of = [&](int k) -> int { return P ? ((k & 1) | (rows4 ? (k & 2) : 0)) : (k & 1); };
    auto rows_of = [&](int k) -> uint8_t* {
        const int r = rbuf_of(k);
        if (!P) return r ? c->rows2.p : c->rows.p;
        hg_ctx_t* L = (r & 1) ? P : c;
        return (r & 2) ? L->rows2.p : L->rows.p;
    };
    auto enqueue_compute = [&](int k) -> int {
        const SubPlan& sp = plans[(size_t)k];
        const int slot = slot_of(k);
        auto& PS = c->pipe[slot];
        const InView V = in_view(c, slot);
        hg_ctx_t* L = lane_of(k);
        const int64_t m = sp.n;
        uint8_t* rbuf = rows_of(k);
        cudaStream_t st = L->st;
        HG_CUDA(cudaStreamWaitEvent(st, PS.in_ready, 0));
        if (rows) HG_CUDA(cudaStreamWaitEvent(st, c->rows_ev[rbuf_of(k)], 0));  // its last read-back is done
        if (ascii)
            HG_CUDA(hg_launch_ascii_pack(PS.ascii.p, PS.aoff.p, (int)m, V.poff, V.packed, PS.nrun.p, V.exc_off, V.exc,
                                         c->exc_cap, PS.excflag.p, c->sms, st));
        hg::BatchDev b = batch_view(L, (int)m, V.packed, V.poff, V.qlen, V.exc, V.exc_off, V.order, V.hoff, V.coff);
        if (rbuf) b.rows = rbuf;
        int rr = run_sub(L, b, true);
        if (rr) return rr;
        compact_offsets_kernel<<<1, 1024, 0, st>>>(L->n_cig.p, (int)m, L->cig_off.p);
        HG_CUDA(cudaGetLastError());
        HG_CUDA(cudaMemcpyAsync(PS.h_off, L->cig_off.p, 8 * ((size_t)m + 1), cudaMemcpyDeviceToHost, st));
        HG_CUDA(cudaMemcpyAsync(PS.h_status, L->status.p, 4 * (size_t)m, cudaMemcpyDeviceToHost, st));
        if (has_ins) HG_CUDA(cudaMemcpyAsync(PS.h_ins, L->has_ins.p, (size_t)m, cudaMemcpyDeviceToHost, st));
        if (ascii) HG_CUDA(cudaMemcpyAsync(PS.h_excflag, PS.excflag.p, 4, cudaMemcpyDeviceToHost, st));
        HG_CUDA(cudaEventRecord(PS.off_ev, st));
        HG_CUDA(cudaStreamWaitEvent(st, PS.cfree, 0));  // the slot's previous CIGARs have copied out
        compact_copy_kernel<<<c->sms * 4, 256, 0, st>>>(L->cig.p, V.coff, L->n_cig.p, L->cig_off.p, (int)m, V.compact,
                                                        (int64_t)V.compact_n, 0);
        HG_CUDA(cudaGetLastError());
        HG_CUDA(cudaEventRecord(PS.in_free, st));
        HG_CUDA(cudaEventRecord(PS.done, st));
        // the rows copy out behind the small read-backs above (copies in one
        // direction share an engine in order, and the offsets gate the next launch)
        if (rows) {
            const int64_t f = sp.first;
            HG_CUDA(cudaStreamWaitEvent(c->cst, PS.done, 0));
            if (row_stride == c->row_stride)
                HG_CUDA(cudaMemcpyAsync(rows + f * row_stride, rbuf, (size_t)row_stride * (size_t)m,
                                        cudaMemcpyDeviceToHost, c->cst));
            else
                HG_CUDA(cudaMemcpy2DAsync(rows + f * row_stride, (size_t)row_stride, rbuf, (size_t)c->row_stride,
                                          (size_t)c->ix->L, (size_t)m, cudaMemcpyDeviceToHost, c->cst));
            HG_CUDA(cudaEventRecord(c->rows_ev[rbuf_of(k)], c->cst));
        }
        return HG_OK;
    };
    int64_t cig_base = 0;
    auto read_back = [&](int k) -> int {
        const SubPlan& sp = plans[(size_t)k];
        const int slot = slot_of(k);
        auto& PS = c->pipe[slot];
        const InView V = in_view(c, slot);
        hg_ctx_t* L = lane_of(k);
        const int64_t f = sp.first, m = sp.n;
        // the offsets decide the copy before the lane's scratch may be overwritten
        HG_CUDA(cudaEventSynchronize(PS.off_ev));
        if (ascii && *PS.h_excflag)
            return fail(HG_ERR_CAPACITY, "hg_align_ascii: the exception runs (bytes other than A/C/G/T) of queries " +
                                             std::to_string(f) + ".. exceed the context's " +
                                             std::to_string(c->exc_cap) + " per sub-batch; pack them with hg_pack");
        const int64_t total = PS.h_off[m];
        if (cig_base + total > cigar_cap) return fail(HG_ERR_CAPACITY, "hg_align_batch: cigar buffer too small");
        if (total <= (int64_t)V.compact_n) {
            HG_CUDA(cudaStreamWaitEvent(c->cst, PS.done, 0));
            if (total)
                HG_CUDA(cudaMemcpyAsync(cigar + cig_base, V.compact, 4 * (size_t)total, cudaMemcpyDeviceToHost, c->cst));
            HG_CUDA(cudaEventRecord(PS.cfree, c->cst));
        } else {  // more CIGAR words than the buffer: copy in pieces now
            HG_CUDA(cudaStreamSynchronize(L->st));
            for (int64_t done = 0; done < total; done += (int64_t)V.compact_n) {
                const int64_t cnt = std::min((int64_t)V.compact_n, total - done);
                compact_copy_kernel<<<c->sms * 4, 256, 0, L->st>>>(L->cig.p, V.coff, L->n_cig.p, L->cig_off.p, (int)m,
                                                                   V.compact, cnt, done);
                HG_CUDA(cudaGetLastError());
                HG_CUDA(cudaMemcpyAsync(cigar + cig_base + done, V.compact, 4 * (size_t)cnt, cudaMemcpyDeviceToHost,
                                        L->st));
            }
            HG_CUDA(cudaStreamSynchronize(L->st));
        }
        for (int64_t i = 0; i <= m; ++i) cigar_off[f + i] = cig_base + PS.h_off[i];
        std::memcpy(status + f, PS.h_status, 4 * (size_t)m);
        if (has_ins) std::memcpy(has_ins + f, PS.h_ins, (size_t)m);
        cig_base += total;
        return HG_OK;
    };
    // an error returns only after the copies already issued into the
    // caller's buffers have finished
    auto drain = [&](int rc) -> int {
        cudaStreamSynchronize(c->ist);
        if (P) cudaStreamSynchronize(P->st);
        cudaStreamSynchronize(c->st);
        cudaStreamSynchronize(c->cst);
        return rc;
    };
    if ((r = issue_inputs(0))) return drain(r);
    if (P) {
        // sub-batch k+1 (the other lane) is enqueued before k's offsets are
        // read; k+2 (this lane, the next slot) has its inputs on the way
        // while k computes and is enqueued once k's offsets are read (the
        // lane's scratch is not reused before that read)
        if ((r = enqueue_compute(0)) || (r = issue_inputs(1)) || (r = enqueue_compute(1))) return drain(r);
        for (int k = 0; k < K; ++k) {
            if (k + 2 < K && NS == 4 && (r = issue_inputs(k + 2))) return drain(r);
            if ((r = read_back(k))) return drain(r);
            if (k + 2 < K) {
                if (NS != 4 && (r = issue_inputs(k + 2))) return drain(r);
                if ((r = enqueue_compute(k + 2))) return drain(r);
            }
        }
    } else {
        for (int k = 0; k < K; ++k) {
            if ((r = enqueue_compute(k))) return drain(r);
            if (k + 1 < K && (r = issue_inputs(k + 1))) return drain(r);  // host work and upload overlap this compute
            if ((r = read_back(k))) return drain(r);
        }
    }
    if (P) HG_CUDA(cudaStreamSynchronize(P->st));
    HG_CUDA(cudaStreamSynchronize(c->cst));
    HG_CUDA(cudaStreamSynchronize(c->st));
    return status_error(status, n);
}

int align_impl(hg_ctx_t* c, const uint8_t* packed, const int64_t* poff, const int32_t* qlen, const int32_t* exc,
               const int64_t* exc_off, int64_t n, uint32_t* cigar, int64_t cigar_cap, int64_t* cigar_off,
               uint8_t* has_ins, uint8_t* rows, int64_t row_stride, uint32_t* status, bool plain)
{
    if (!c || n < 0 || (n && (!packed || !poff || !qlen || !exc_off || !cigar || !cigar_off)))
        return fail(HG_ERR_ARG, "hg_align_batch: bad arguments");
    if (rows && row_stride < c->ix->L) return fail(HG_ERR_ARG, "hg_align_batch: row_stride < center length");
    cudaSetDevice(c->ix->device);
    std::vector<uint32_t> st_local;
    if (!status) st_local.resize((size_t)n), status = st_local.data();
    int64_t cig_base = 0;
    if (n == 0) {
        cigar_off[0] = 0;
        return HG_OK;
    }
    auto plans = plan(c, poff, qlen, exc_off, n);
    if (!plain) plans = edge_split(c, plans, qlen, exc_off, rows != nullptr, false);
    if (!plain && plans.size() > 1)
        return align_pipelined(c, plans, packed, poff, qlen, exc, exc_off, n, cigar, cigar_cap, cigar_off, has_ins,
                               rows, row_stride, status);
    // two row buffers alternate between sub-batches so the read-back of one
    // overlaps the next sub-batch's compute
    if (rows && !plain && plans.size() > 1 && !c->rows2.p)
        HG_CUDA(c->rows2.alloc((size_t)c->max_n * c->row_stride));
    size_t sub_i = 0;
    std::vector<int32_t> order;
    std::vector<int64_t> hoff, coff, spoff, seoff;
    for (const SubPlan& sp : plans) {
        const int64_t f = sp.first;
        if (sp.n > c->max_n || sp.bases > c->max_bases)
            return fail(HG_ERR_CAPACITY, "query " + std::to_string(f) + " exceeds the context capacity");
        sub_arrays(c, qlen + f, sp.n, order, hoff, coff);
        spoff.resize(sp.n), seoff.resize(sp.n + 1);
        int64_t pb = 0;
        for (int64_t i = 0; i < sp.n; ++i) spoff[i] = pb, pb += (int64_t)padded_bytes(qlen[f + i]);
        for (int64_t i = 0; i <= sp.n; ++i) seoff[i] = exc_off[f + i] - exc_off[f];
        // inputs: per-query packed blocks may be scattered in the caller's buffer
        bool contiguous = true;
        for (int64_t i = 1; i < sp.n && contiguous; ++i) contiguous = poff[f + i] == poff[f] + spoff[i];
        if (contiguous) {
            HG_CUDA(cudaMemcpyAsync(c->packed.p, packed + poff[f], (size_t)pb, cudaMemcpyHostToDevice, c->st));
        } else {
            for (int64_t i = 0; i < sp.n; ++i)
                HG_CUDA(cudaMemcpyAsync(c->packed.p + spoff[i], packed + poff[f + i], padded_bytes(qlen[f + i]),
                                        cudaMemcpyHostToDevice, c->st));
        }
        const int64_t ne = seoff[sp.n];
        if (ne) HG_CUDA(cudaMemcpyAsync(c->exc.p, exc + 3 * exc_off[f], 12 * (size_t)ne, cudaMemcpyHostToDevice, c->st));
        HG_CUDA(cudaMemcpyAsync(c->poff.p, spoff.data(), 8 * (size_t)sp.n, cudaMemcpyHostToDevice, c->st));
        HG_CUDA(cudaMemcpyAsync(c->qlen.p, qlen + f, 4 * (size_t)sp.n, cudaMemcpyHostToDevice, c->st));
        HG_CUDA(cudaMemcpyAsync(c->exc_off.p, seoff.data(), 8 * ((size_t)sp.n + 1), cudaMemcpyHostToDevice, c->st));
        HG_CUDA(cudaMemcpyAsync(c->order.p, order.data(), 4 * (size_t)sp.n, cudaMemcpyHostToDevice, c->st));
        HG_CUDA(cudaMemcpyAsync(c->hoff.p, hoff.data(), 8 * (size_t)sp.n, cudaMemcpyHostToDevice, c->st));
        HG_CUDA(cudaMemcpyAsync(c->coff.p, coff.data(), 8 * (size_t)sp.n, cudaMemcpyHostToDevice, c->st));
        const int rslot = (c->rows2.p && (sub_i & 1)) ? 1 : 0;
        uint8_t* rbuf = rslot ? c->rows2.p : c->rows.p;
        HG_CUDA(cudaStreamWaitEvent(c->st, c->rows_ev[rslot], 0));  // its last read-back is done
        if (!plain) {
            hg::BatchDev b = batch_view(c, (int)sp.n, c->packed.p, c->poff.p, c->qlen.p, c->exc.p,
                                        c->exc_off.p, c->order.p, c->hoff.p, c->coff.p);
            b.rows = rbuf;
            int r = run_sub(c, b, true);
            if (r) return r;
        } else {
            // one launch sequence per query: a one-query view of the same buffers
            for (int64_t i = 0; i < sp.n; ++i) {
                hg::BatchDev b = batch_view(c, 1, c->packed.p, c->poff.p + i, c->qlen.p + i, c->exc.p,
                                            c->exc_off.p + i, nullptr, c->hoff.p + i, c->coff.p + i);
                // per-query outputs land at index 0 of the view: shift the output arrays
                b.n_hits = c->n_hits.p + i, b.n_matched = c->n_matched.p + i, b.a_base = c->a_base.p + i,
                b.a_n = c->a_n.p + i, b.s_base = c->s_base.p + i, b.s_n = c->s_n.p + i, b.n_chain = c->n_chain.p + i;
                b.chain_meta = c->chain_meta.p + 2 * i;
                b.n_cig = c->n_cig.p + i, b.has_ins = c->has_ins.p + i, b.status = c->status.p + i;
                b.rows = c->rows.p + i * c->row_stride;
                if (i == 0) HG_CUDA(cudaMemsetAsync(c->status.p, 0, 4 * (size_t)sp.n, c->st));
                // status must survive the per-launch reset: enqueue without the batch memset
                HG_CUDA(cudaMemsetAsync(c->control.p, 0, sizeof(unsigned long long) * kControlWords, c->st));
                HG_CUDA(cudaMemsetAsync(c->shape_hist.p, 0, sizeof(uint32_t) * hg::kShapeBins, c->st));
                HG_CUDA(cudaMemsetAsync(c->wave_hist.p, 0, sizeof(uint32_t) * kSortHistWords, c->st));
                const hg::IndexDev& ix = c->ix->dev;
                HG_CUDA(hg_launch_seed(&ix, &b, 0, nullptr, nullptr, 1, c->st));
                HG_CUDA(hg_launch_anchor(&ix, &b, 1, c->st));
                HG_CUDA(hg_launch_chain(&ix, &b, 1, c->st));
                HG_CUDA(hg_launch_dp_small(&ix, &b, c->sms, c->st));
                HG_CUDA(hg_launch_dp_thin(&ix, &b, c->sms, c->st));
                HG_CUDA(hg_launch_dp_wave(&ix, &b, c->sms, c->st));
                HG_CUDA(hg_launch_dp_wide(&ix, &b, c->sms, c->st));
                HG_CUDA(hg_launch_dp_large(&ix, &b, c->sms, c->st));
                HG_CUDA(hg_launch_stitch(&ix, &b, 1, c->st));
                HG_CUDA(hg_launch_rows(&ix, &b, c->row_stride, 1, c->st));
                HG_CUDA(hg_launch_count(b.rows, c->row_stride, 1, ix.L, c->counts.p, c->st));
                c->last_launches += kLaunchesPlain;
            }
        }
        int64_t total = 0;
        int r = fetch_outputs(c, (int)sp.n, c->coff.p, cigar, cigar_cap, cig_base, cigar_off + f,
                              has_ins ? has_ins + f : nullptr, rows ? rows + f * row_stride : nullptr, row_stride,
                              status + f, &total, rbuf);
        if (r) return r;
        cig_base += total;
        ++sub_i;
    }
    HG_CUDA(cudaStreamSynchronize(c->cst));
    return status_error(status, n);
}

}  // namespace

extern "C" int hg_align_batch(hg_ctx_t* ctx, const uint8_t* packed, const int64_t* poff, const int32_t* qlen,
                              const int32_t* exc, const int64_t* exc_off, int64_t n, uint32_t* cigar,
                              int64_t cigar_cap, int64_t* cigar_off, uint8_t* has_ins, uint8_t* rows,
                              int64_t row_stride, uint32_t* status)
{
    return align_impl(ctx, packed, poff, qlen, exc, exc_off, n, cigar, cigar_cap, cigar_off, has_ins, rows,
                      row_stride, status, false);
}

extern "C" int hg_align_plain(hg_ctx_t* ctx, const uint8_t* packed, const int64_t* poff, const int32_t* qlen,
                              const int32_t* exc, const int64_t* exc_off, int64_t n, uint32_t* cigar,
                              int64_t cigar_cap, int64_t* cigar_off, uint8_t* has_ins, uint8_t* rows,
                              int64_t row_stride, uint32_t* status)
{
    return align_impl(ctx, packed, poff, qlen, exc, exc_off, n, cigar, cigar_cap, cigar_off, has_ins, rows,
                      row_stride, status, true);
}

extern "C" int hg_align_ascii(hg_ctx_t* c, const char* seqs, const int64_t* offsets, int64_t n, uint32_t* cigar,
                              int64_t cigar_cap, int64_t* cigar_off, uint8_t* has_ins, uint8_t* rows,
                              int64_t row_stride, uint32_t* status)
{
    if (!c || n < 0 || (n && (!seqs || !offsets || !cigar || !cigar_off)))
        return fail(HG_ERR_ARG, "hg_align_ascii: bad arguments");
    if (rows && row_stride < c->ix->L) return fail(HG_ERR_ARG, "hg_align_ascii: row_stride < center length");
    if (n == 0) {
        cigar_off[0] = 0;
        return HG_OK;
    }
    std::vector<int32_t>& qlen = c->pl_qlen;  // kept across calls
    qlen.resize((size_t)n);
    for (int64_t i = 0; i < n; ++i) {
        const int64_t len = offsets[i + 1] - offsets[i];
        if (len < 0 || len > INT32_MAX) return fail(HG_ERR_ARG, "hg_align_ascii: bad query length");
        qlen[(size_t)i] = (int32_t)len;
    }
    cudaSetDevice(c->ix->device);
    std::vector<uint32_t> st_local;
    if (!status) st_local.resize((size_t)n), status = st_local.data();
    auto plans = plan(c, nullptr, qlen.data(), nullptr, n);
    plans = edge_split(c, plans, qlen.data(), nullptr, rows != nullptr, true);
    return align_pipelined(c, plans, nullptr, nullptr, qlen.data(), nullptr, nullptr, n, cigar, cigar_cap, cigar_off,
                           has_ins, rows, row_stride, status, reinterpret_cast<const uint8_t*>(seqs), offsets);
}

extern "C" int hg_fetch_chain(hg_ctx_t* c, int64_t query, uint32_t* pos_ref, uint32_t* pos_qry, int32_t* f,
                              int32_t* p, int64_t cap, int64_t* n_anchors, int64_t* chain_end, int64_t* n_chain)
{
    if (!c || !c->staged || !n_anchors || query < 0 || query >= (int64_t)c->staged_qlen.size())
        return fail(HG_ERR_ARG, "hg_fetch_chain: bad arguments or nothing staged");
    if (c->staged_plan.size() != 1)
        return fail(HG_ERR_ARG, "hg_fetch_chain: the staged batch spans several sub-batches");
    cudaSetDevice(c->ix->device);
    HG_CUDA(cudaStreamSynchronize(c->st));
    int64_t base = 0;
    int32_t A = 0, nc = 0, meta[2] = {-1, 0};
    HG_CUDA(cudaMemcpy(&base, c->a_base.p + query, 8, cudaMemcpyDeviceToHost));
    HG_CUDA(cudaMemcpy(&A, c->a_n.p + query, 4, cudaMemcpyDeviceToHost));
    HG_CUDA(cudaMemcpy(&nc, c->n_chain.p + query, 4, cudaMemcpyDeviceToHost));
    HG_CUDA(cudaMemcpy(meta, c->chain_meta.p + 2 * query, 8, cudaMemcpyDeviceToHost));
    *n_anchors = A;
    if (chain_end) *chain_end = meta[0];
    if (n_chain) *n_chain = nc;
    if (A > cap || A == 0) return HG_OK;
    std::vector<int32_t> fv((size_t)A), pv((size_t)A);
    if (pos_ref) HG_CUDA(cudaMemcpy(pos_ref, c->a_ref.p + base, 4 * (size_t)A, cudaMemcpyDeviceToHost));
    if (pos_qry) HG_CUDA(cudaMemcpy(pos_qry, c->a_qry.p + base, 4 * (size_t)A, cudaMemcpyDeviceToHost));
    HG_CUDA(cudaMemcpy(fv.data(), c->a_f.p + base, 4 * (size_t)A, cudaMemcpyDeviceToHost));
    HG_CUDA(cudaMemcpy(pv.data(), c->a_p.p + base, 4 * (size_t)A, cudaMemcpyDeviceToHost));
    // below the first wrong speculation the kernel keeps p implicit: the
    // previous anchor when f exceeds the lone-anchor score (the span, k)
    const int32_t k0 = std::min(std::max(meta[1], 0), A);
    for (int32_t i = 0; i < k0; ++i) pv[i] = fv[i] > c->ix->k ? i - 1 : -1;
    if (f) std::copy(fv.begin(), fv.end(), f);
    if (p) std::copy(pv.begin(), pv.end(), p);
    return HG_OK;
}

extern "C" int hg_counters(hg_ctx_t* c, uint32_t* counts7, uint32_t* ins, int reset)
{
    if (!c) return fail(HG_ERR_ARG, "hg_counters: null context");
    cudaSetDevice(c->ix->device);
    const int64_t L = c->ix->L;
    HG_CUDA(cudaStreamSynchronize(c->st));
    if (counts7) HG_CUDA(cudaMemcpy(counts7, c->counts.p, 4 * (size_t)L * 7, cudaMemcpyDeviceToHost));
    if (ins) HG_CUDA(cudaMemcpy(ins, c->ins.p, 4 * (size_t)(L + 1), cudaMemcpyDeviceToHost));
    if (reset) {
        HG_CUDA(cudaMemset(c->counts.p, 0, 4 * (size_t)L * 7));
        HG_CUDA(cudaMemset(c->ins.p, 0, 4 * (size_t)(L + 1)));
    }
    if (c->peer) {  // rows aligned on the second lane (uint32 sums wrap as SiteCount's do)
        std::vector<uint32_t> pc(counts7 ? (size_t)L * 7 : 0), pi(ins ? (size_t)L + 1 : 0);
        int r = hg_counters(c->peer, counts7 ? pc.data() : nullptr, ins ? pi.data() : nullptr, reset);
        if (r) return r;
        for (size_t i = 0; i < pc.size(); ++i) counts7[i] += pc[i];
        for (size_t i = 0; i < pi.size(); ++i) ins[i] += pi[i];
    }
    return HG_OK;
}

// ------------------------------------------------------- device-resident form

extern "C" int hg_stage(hg_ctx_t* c, const uint8_t* packed, const int64_t* poff, const int32_t* qlen,
                        const int32_t* exc, const int64_t* exc_off, int64_t n)
{
    if (!c || n <= 0) return fail(HG_ERR_ARG, "hg_stage: bad arguments");
    cudaSetDevice(c->ix->device);
    c->staged_plan = plan(c, poff, qlen, exc_off, n);
    c->staged_qlen.assign(qlen, qlen + n);
    int64_t pb = 0;
    std::vector<int64_t> spoff(n), seoff(n + 1), hoff(n), coff(n);
    std::vector<int32_t> order(n);
    for (int64_t i = 0; i < n; ++i) spoff[i] = pb, pb += (int64_t)padded_bytes(qlen[i]);
    for (int64_t i = 0; i <= n; ++i) seoff[i] = exc_off[i] - exc_off[0];
    // per sub-batch: local order / hit / cigar offsets, kept in one array
    for (const SubPlan& sp : c->staged_plan) {
        std::vector<int32_t> o;
        std::vector<int64_t> h, co;
        sub_arrays(c, qlen + sp.first, sp.n, o, h, co);
        for (int64_t i = 0; i < sp.n; ++i) order[sp.first + i] = o[i], hoff[sp.first + i] = h[i], coff[sp.first + i] = co[i];
    }
    const int64_t ne = seoff[n];
    cudaError_t e = cudaSuccess;
    // 64 bytes of slack: kernels read packed bases as aligned 24-byte windows
    if ((e = c->s_packed.alloc(pb + 64)) || (e = c->s_poff.alloc(n)) || (e = c->s_exc_off.alloc(n + 1)) ||
        (e = c->s_hoff.alloc(n)) || (e = c->s_coff.alloc(n)) || (e = c->s_qlen.alloc(n)) ||
        (e = c->s_exc.alloc(std::max<int64_t>(ne, 1) * 3)) || (e = c->s_order.alloc(n)))
        return cuda_fail(e, "hg_stage: allocation");
    bool contiguous = true;
    for (int64_t i = 1; i < n && contiguous; ++i) contiguous = poff[i] == poff[0] + spoff[i];
    if (contiguous) HG_CUDA(cudaMemcpy(c->s_packed.p, packed + poff[0], (size_t)pb, cudaMemcpyHostToDevice));
    else
        for (int64_t i = 0; i < n; ++i)
            HG_CUDA(cudaMemcpy(c->s_packed.p + spoff[i], packed + poff[i], padded_bytes(qlen[i]), cudaMemcpyHostToDevice));
    if (ne) HG_CUDA(cudaMemcpy(c->s_exc.p, exc + 3 * exc_off[0], 12 * (size_t)ne, cudaMemcpyHostToDevice));
    HG_CUDA(cudaMemcpy(c->s_poff.p, spoff.data(), 8 * n, cudaMemcpyHostToDevice));
    HG_CUDA(cudaMemcpy(c->s_exc_off.p, seoff.data(), 8 * (n + 1), cudaMemcpyHostToDevice));
    HG_CUDA(cudaMemcpy(c->s_hoff.p, hoff.data(), 8 * n, cudaMemcpyHostToDevice));
    HG_CUDA(cudaMemcpy(c->s_coff.p, coff.data(), 8 * n, cudaMemcpyHostToDevice));
    HG_CUDA(cudaMemcpy(c->s_qlen.p, qlen, 4 * n, cudaMemcpyHostToDevice));
    HG_CUDA(cudaMemcpy(c->s_order.p, order.data(), 4 * n, cudaMemcpyHostToDevice));
    c->staged = true;
    return HG_OK;
}

extern "C" int hg_set_timing(hg_ctx_t* c, int on)
{
    if (!c) return fail(HG_ERR_ARG, "hg_set_timing: null context");
    c->timing = on != 0;
    return HG_OK;
}

extern "C" int hg_run_staged(hg_ctx_t* c)
{
    if (!c || !c->staged) return fail(HG_ERR_ARG, "hg_run_staged: nothing staged");
    cudaSetDevice(c->ix->device);
    c->last_total_ms = 0;
    std::fill(c->last_stage_ms, c->last_stage_ms + 8, 0.0f);
    c->last_launches = 0;
    // every other sub-batch on the second lane (its own arenas and streams),
    // reading the staged inputs; the run's end waits for both lanes
    hg_ctx_t* P = (c->timing || c->staged_plan.size() < 2) ? nullptr : lane_peer(c);
    HG_CUDA(cudaMemsetAsync(c->cells.p, 0, 2 * sizeof(unsigned long long), c->st));
    HG_CUDA(cudaMemsetAsync(c->run_flags.p, 0, sizeof(uint32_t), c->st));
    HG_CUDA(cudaEventRecord(c->run_ev[0], c->st));
    if (P) {
        P->last_launches = 0;
        HG_CUDA(cudaStreamWaitEvent(P->st, c->run_ev[0], 0));
        HG_CUDA(cudaMemsetAsync(P->cells.p, 0, 2 * sizeof(unsigned long long), P->st));
        HG_CUDA(cudaMemsetAsync(P->run_flags.p, 0, sizeof(uint32_t), P->st));
    }
    c->lanes_used = P ? 2 : 1;
    for (size_t k = 0; k < c->staged_plan.size(); ++k) {
        const SubPlan& sp = c->staged_plan[k];
        const int64_t f = sp.first;
        hg_ctx_t* L = (P && (k & 1)) ? P : c;
        // exception offsets of the sub-batch are global: rebase through exc_off view
        const hg::BatchDev b = batch_view(L, (int)sp.n, c->s_packed.p, c->s_poff.p + f, c->s_qlen.p + f, c->s_exc.p,
                                          c->s_exc_off.p + f, c->s_order.p + f, c->s_hoff.p + f, c->s_coff.p + f);
        int r = run_sub(L, b, true);
        if (r) return r;
    }
    if (P) {
        HG_CUDA(cudaEventRecord(c->lane_ev, P->st));
        HG_CUDA(cudaStreamWaitEvent(c->st, c->lane_ev, 0));
        c->last_launches += P->last_launches;
    }
    HG_CUDA(cudaEventRecord(c->run_ev[1], c->st));
    c->run_recorded = true;
    return HG_OK;
}

extern "C" int hg_last_timing(hg_ctx_t* c, float* total_ms, float* stage_ms, int64_t* launches, int64_t* cells)
{
    if (!c) return fail(HG_ERR_ARG, "hg_last_timing: null context");
    cudaSetDevice(c->ix->device);
    HG_CUDA(cudaStreamSynchronize(c->st));
    float tot = c->last_total_ms;
    if (!c->timing && c->run_recorded) HG_CUDA(cudaEventElapsedTime(&tot, c->run_ev[0], c->run_ev[1]));
    if (total_ms) *total_ms = tot;
    if (stage_ms) std::copy(c->last_stage_ms, c->last_stage_ms + 8, stage_ms);
    if (launches) *launches = c->last_launches;
    if (cells) {
        int64_t v = 0;
        int r = hg_last_cells(c, &v, nullptr);
        if (r) return r;
        *cells = v;
    }
    return HG_OK;
}

extern "C" int hg_last_cells(hg_ctx_t* c, int64_t* cells, int64_t* match_cells)
{
    if (!c) return fail(HG_ERR_ARG, "hg_last_cells: null context");
    cudaSetDevice(c->ix->device);
    HG_CUDA(cudaStreamSynchronize(c->st));
    unsigned long long v[2] = {0, 0}, w[2] = {0, 0};
    HG_CUDA(cudaMemcpy(v, c->cells.p, sizeof(v), cudaMemcpyDeviceToHost));
    if (c->peer && c->lanes_used == 2) {  // the second lane's sub-batches
        HG_CUDA(cudaStreamSynchronize(c->peer->st));
        HG_CUDA(cudaMemcpy(w, c->peer->cells.p, sizeof(w), cudaMemcpyDeviceToHost));
    }
    if (cells) *cells = (int64_t)(v[0] + w[0]);
    if (match_cells) *match_cells = (int64_t)(v[1] + w[1]);
    return HG_OK;
}

extern "C" int hg_ctx_work(hg_ctx_t* c, int64_t* counts, int n)
{
    if (!c || !counts || n < 0) return fail(HG_ERR_ARG, "hg_ctx_work: bad arguments");
    cudaSetDevice(c->ix->device);
    HG_CUDA(cudaStreamSynchronize(c->st));
    unsigned long long v[4] = {0, 0, 0, 0};
    HG_CUDA(cudaMemcpy(v, c->work.p, sizeof(v), cudaMemcpyDeviceToHost));
    for (int i = 0; i < n && i < 4; ++i) counts[i] = (int64_t)v[i];
    if (c->peer) {  // work of the second lane's sub-batches
        int64_t w[4] = {0, 0, 0, 0};
        HG_CUDA(cudaStreamSynchronize(c->peer->st));
        int r = hg_ctx_work(c->peer, w, n < 4 ? n : 4);
        if (r) return r;
        for (int i = 0; i < n && i < 4; ++i) counts[i] += w[i];
    }
    return HG_OK;
}

extern "C" int hg_staged_flags(hg_ctx_t* c, uint32_t* flags)
{
    if (!c || !flags) return fail(HG_ERR_ARG, "hg_staged_flags: bad arguments");
    cudaSetDevice(c->ix->device);
    HG_CUDA(cudaStreamSynchronize(c->st));
    HG_CUDA(cudaMemcpy(flags, c->run_flags.p, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    if (c->peer && c->lanes_used == 2) {
        uint32_t f2 = 0;
        HG_CUDA(cudaMemcpy(&f2, c->peer->run_flags.p, sizeof(uint32_t), cudaMemcpyDeviceToHost));
        *flags |= f2;
    }
    return HG_OK;
}

extern "C" int hg_fetch_staged(hg_ctx_t* c, uint32_t* cigar, int64_t cigar_cap, int64_t* cigar_off, uint8_t* has_ins,
                               uint8_t* rows, int64_t row_stride, uint32_t* status)
{
    if (!c || !c->staged) return fail(HG_ERR_ARG, "hg_fetch_staged: nothing staged");
    cudaSetDevice(c->ix->device);
    if (c->staged_plan.size() != 1)
        return fail(HG_ERR_ARG, "hg_fetch_staged: staged batch spans several sub-batches; fetch needs one");
    const SubPlan& sp = c->staged_plan[0];
    int64_t total = 0;
    const int r = fetch_outputs(c, (int)sp.n, c->s_coff.p, cigar, cigar_cap, 0, cigar_off, has_ins, rows, row_stride,
                                status, &total, c->rows.p);
    if (r) return r;
    HG_CUDA(cudaStreamSynchronize(c->cst));
    return HG_OK;
}

// ------------------------------------------------------ asynchronous form

namespace {

// Pinned staging of the asynchronous form, allocated on first use.
int async_staging(hg_ctx_t* c)
{
    if (c->h_packed) return HG_OK;
    const int64_t M = c->max_n + 1;
    c->h_cig_cap = c->max_bases / 8 + 64 * c->max_n + 1024;  // a few ops per kilobase; longer ones go the slow way
    if ((!c->h_cig && cudaHostAlloc(&c->h_cig, sizeof(uint32_t) * (size_t)c->h_cig_cap, cudaHostAllocMapped) != cudaSuccess) ||
        cudaHostGetDevicePointer(reinterpret_cast<void**>(&c->h_cig_dev), c->h_cig, 0) != cudaSuccess ||
        cudaHostAlloc(&c->h_packed, c->packed.n, cudaHostAllocDefault) != cudaSuccess ||
        cudaHostAlloc(&c->h_i64, sizeof(int64_t) * 5 * M, cudaHostAllocDefault) != cudaSuccess ||
        cudaHostAlloc(&c->h_i32, sizeof(int32_t) * (2 * M + 3 * c->exc_cap), cudaHostAllocDefault) != cudaSuccess ||
        cudaHostAlloc(&c->h_has_ins, (size_t)M, cudaHostAllocDefault) != cudaSuccess ||
        cudaHostAlloc(&c->h_status, sizeof(uint32_t) * M, cudaHostAllocDefault) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->done_ev, cudaEventDisableTiming | cudaEventBlockingSync) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->collected_ev, cudaEventDisableTiming | cudaEventBlockingSync) != cudaSuccess)
        return fail(HG_ERR_NOMEM, "hg_submit: pinned staging allocation");
    return HG_OK;
}

// The staged micro-batch (packed bases at h_packed, per-query offsets,
// lengths and exception runs in h_i64 / h_i32) goes up and through the
// stages on the context stream; results come back behind done_ev.  With
// `runs` the bases are ASCII in pinned memory instead (run r: run_bytes[r]
// bytes of consecutive queries at run_ptr[r], query offsets in h_i64's
// second block): they go up as they are and the device packs them.
int submit_tail(hg_ctx_t* c, int64_t n, int64_t pb, int64_t ne, const char* const* run_ptr = nullptr,
                const int64_t* run_bytes = nullptr, int runs = 0)
{
    const int64_t M = c->max_n + 1;
    int64_t *spoff = c->h_i64, *seoff = c->h_i64 + M, *shoff = c->h_i64 + 2 * M, *scoff = c->h_i64 + 3 * M;
    int32_t *sqlen = c->h_i32, *sorder = c->h_i32 + M, *sexc = c->h_i32 + 2 * M;
    std::vector<int32_t> order;
    std::vector<int64_t> hoff, coff;
    sub_arrays(c, sqlen, n, order, hoff, coff);
    for (int64_t i = 0; i < n; ++i) sorder[i] = order[i], shoff[i] = hoff[i], scoff[i] = coff[i];
    cudaStream_t st = c->st;
    auto& PS = c->pipe[0];
    if (run_ptr) {
        int64_t at = 0;
        for (int r = 0; r < runs; ++r) {
            if (run_bytes[r])
                HG_CUDA(cudaMemcpyAsync(PS.ascii.p + at, run_ptr[r], (size_t)run_bytes[r], cudaMemcpyHostToDevice, st));
            at += run_bytes[r];
        }
        HG_CUDA(cudaMemcpyAsync(PS.aoff.p, seoff, 8 * ((size_t)n + 1), cudaMemcpyHostToDevice, st));
    } else {
        HG_CUDA(cudaMemcpyAsync(c->packed.p, c->h_packed, (size_t)pb, cudaMemcpyHostToDevice, st));
        if (ne) HG_CUDA(cudaMemcpyAsync(c->exc.p, sexc, 12 * (size_t)ne, cudaMemcpyHostToDevice, st));
        HG_CUDA(cudaMemcpyAsync(c->exc_off.p, seoff, 8 * ((size_t)n + 1), cudaMemcpyHostToDevice, st));
    }
    HG_CUDA(cudaMemcpyAsync(c->poff.p, spoff, 8 * (size_t)n, cudaMemcpyHostToDevice, st));
    HG_CUDA(cudaMemcpyAsync(c->qlen.p, sqlen, 4 * (size_t)n, cudaMemcpyHostToDevice, st));
    HG_CUDA(cudaMemcpyAsync(c->order.p, sorder, 4 * (size_t)n, cudaMemcpyHostToDevice, st));
    HG_CUDA(cudaMemcpyAsync(c->hoff.p, shoff, 8 * (size_t)n, cudaMemcpyHostToDevice, st));
    HG_CUDA(cudaMemcpyAsync(c->coff.p, scoff, 8 * (size_t)n, cudaMemcpyHostToDevice, st));
    if (run_ptr)
        HG_CUDA(hg_launch_ascii_pack(PS.ascii.p, PS.aoff.p, (int)n, c->poff.p, c->packed.p, PS.nrun.p, c->exc_off.p,
                                     c->exc.p, c->exc_cap, PS.excflag.p, c->sms, st));
    const hg::BatchDev b = batch_view(c, (int)n, c->packed.p, c->poff.p, c->qlen.p, c->exc.p, c->exc_off.p,
                                      c->order.p, c->hoff.p, c->coff.p);
    int r = run_sub(c, b, false);
    if (r) return r;
    compact_offsets_kernel<<<1, 1024, 0, st>>>(c->n_cig.p, (int)n, c->cig_off.p);
    HG_CUDA(cudaGetLastError());
    compact_copy_kernel<<<c->sms * 4, 256, 0, st>>>(c->cig.p, c->coff.p, c->n_cig.p, c->cig_off.p, (int)n, c->h_cig_dev,
                                                    c->h_cig_cap, 0);
    HG_CUDA(cudaGetLastError());
    HG_CUDA(cudaMemcpyAsync(c->h_i64 + 4 * M, c->cig_off.p, 8 * ((size_t)n + 1), cudaMemcpyDeviceToHost, st));
    HG_CUDA(cudaMemcpyAsync(c->h_has_ins, c->has_ins.p, (size_t)n, cudaMemcpyDeviceToHost, st));
    HG_CUDA(cudaMemcpyAsync(c->h_status, c->status.p, 4 * (size_t)n, cudaMemcpyDeviceToHost, st));
    if (run_ptr) HG_CUDA(cudaMemcpyAsync(PS.h_excflag, PS.excflag.p, 4, cudaMemcpyDeviceToHost, st));
    HG_CUDA(cudaEventRecord(c->done_ev, st));
    c->async_n = n;
    c->async_ascii = run_ptr != nullptr;
    return HG_OK;
}

}  // namespace

int hg::prepare_pinned_ascii(hg_ctx_t* c)
{
    cudaSetDevice(c->ix->device);
    int r = ascii_setup(c, 1);
    return r ? r : async_staging(c);
}

int hg::submit_pinned_ascii(hg_ctx_t* c, const char* const* run_ptr, const int64_t* run_bytes, int runs,
                            const int64_t* lens, int64_t n)
{
    if (!c || n <= 0 || runs < 0 || (runs > 0 && (!run_ptr || !run_bytes)) || !lens)
        return fail(HG_ERR_ARG, "submit_pinned_ascii: bad arguments");
    if (c->async_n >= 0) return fail(HG_ERR_ARG, "submit_pinned_ascii: previous batch not collected");
    cudaSetDevice(c->ix->device);
    int64_t bases = 0, bytes = 0, up = 0;
    for (int64_t i = 0; i < n; ++i) {
        if (lens[i] < 0 || lens[i] > INT32_MAX) return fail(HG_ERR_ARG, "submit_pinned_ascii: bad query");
        bases += lens[i], bytes += (int64_t)padded_bytes(lens[i]);
    }
    for (int r = 0; r < runs; ++r) up += run_bytes[r];
    if (up != bases) return fail(HG_ERR_ARG, "submit_pinned_ascii: the runs do not hold the queries' bytes");
    if (n > c->max_n || bases > c->max_bases || bytes > (int64_t)c->packed.n)
        return fail(HG_ERR_CAPACITY, "submit_pinned_ascii: batch exceeds the context capacity");
    int r = ascii_setup(c, 1);
    if (r || (r = async_staging(c))) return r;
    const int64_t M = c->max_n + 1;
    int64_t *spoff = c->h_i64, *saoff = c->h_i64 + M;
    int32_t* sqlen = c->h_i32;
    int64_t pb = 0, ab = 0;
    for (int64_t i = 0; i < n; ++i) {
        spoff[i] = pb, pb += (int64_t)padded_bytes(lens[i]);
        saoff[i] = ab, ab += lens[i];
        sqlen[i] = (int32_t)lens[i];
    }
    saoff[n] = ab;
    return submit_tail(c, n, pb, 0, run_ptr, run_bytes, runs);
}

bool hg::async_exc_overflow(const hg_ctx_t* c) { return c && c->async_exc_over; }

extern "C" int hg_submit(hg_ctx_t* c, const uint8_t* packed, const int64_t* poff, const int32_t* qlen,
                         const int32_t* exc, const int64_t* exc_off, int64_t n)
{
    if (!c || n <= 0 || !packed || !poff || !qlen || !exc_off) return fail(HG_ERR_ARG, "hg_submit: bad arguments");
    if (c->async_n >= 0) return fail(HG_ERR_ARG, "hg_submit: previous batch not collected");
    cudaSetDevice(c->ix->device);
    int64_t bases = 0, bytes = 0;
    for (int64_t i = 0; i < n; ++i) bases += qlen[i], bytes += (int64_t)padded_bytes(qlen[i]);
    const int64_t ne = exc_off[n] - exc_off[0];
    if (n > c->max_n || bases > c->max_bases || bytes > (int64_t)c->packed.n || ne > c->exc_cap)
        return fail(HG_ERR_CAPACITY, "hg_submit: batch exceeds the context capacity");
    int r = async_staging(c);
    if (r) return r;
    const int64_t M = c->max_n + 1;
    int64_t *spoff = c->h_i64, *seoff = c->h_i64 + M;
    int32_t *sqlen = c->h_i32, *sexc = c->h_i32 + 2 * M;
    int64_t pb = 0;
    for (int64_t i = 0; i < n; ++i) {
        const size_t nb = padded_bytes(qlen[i]);
        std::memcpy(c->h_packed + pb, packed + poff[i], nb);
        spoff[i] = pb, pb += (int64_t)nb;
        sqlen[i] = qlen[i];
    }
    for (int64_t i = 0; i <= n; ++i) seoff[i] = exc_off[i] - exc_off[0];
    if (ne) std::memcpy(sexc, exc + 3 * exc_off[0], 12 * (size_t)ne);
    return submit_tail(c, n, pb, ne);
}

extern "C" int hg_submit_ascii(hg_ctx_t* c, const char* const* seqs, const int64_t* lens, int64_t n)
{
    if (!c || n <= 0 || !seqs || !lens) return fail(HG_ERR_ARG, "hg_submit_ascii: bad arguments");
    if (c->async_n >= 0) return fail(HG_ERR_ARG, "hg_submit_ascii: previous batch not collected");
    cudaSetDevice(c->ix->device);
    int64_t bases = 0, bytes = 0;
    for (int64_t i = 0; i < n; ++i) {
        if (lens[i] < 0 || lens[i] > INT32_MAX || (lens[i] > 0 && !seqs[i]))
            return fail(HG_ERR_ARG, "hg_submit_ascii: bad query");
        bases += lens[i], bytes += (int64_t)padded_bytes(lens[i]);
    }
    if (n > c->max_n || bases > c->max_bases || bytes > (int64_t)c->packed.n)
        return fail(HG_ERR_CAPACITY, "hg_submit_ascii: batch exceeds the context capacity");
    int r = async_staging(c);
    if (r) return r;
    const int64_t M = c->max_n + 1;
    int64_t *spoff = c->h_i64, *seoff = c->h_i64 + M;
    int32_t *sqlen = c->h_i32, *sexc = c->h_i32 + 2 * M;
    int64_t pb = 0;
    for (int64_t i = 0; i < n; ++i) spoff[i] = pb, pb += (int64_t)padded_bytes(lens[i]), sqlen[i] = (int32_t)lens[i];
    // pass 1: bases straight into the pinned staging, queries in parallel
    std::vector<uint8_t> has_exc((size_t)n);
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t i = 0; i < n; ++i) {
        uint8_t* out = c->h_packed + spoff[i];
        const size_t nb = padded_bytes(lens[i]);
        has_exc[i] = pack_one(reinterpret_cast<const unsigned char*>(seqs[i]), lens[i], out) ? 1 : 0;
        const size_t used = (size_t)(lens[i] + 3) / 4;
        if (nb > used) std::memset(out + used, 0, nb - used);
    }
    // pass 2: exception runs of the queries that hold any
    int64_t ne = 0;
    for (int64_t i = 0; i < n; ++i) {
        seoff[i] = ne;
        if (!has_exc[i]) continue;
        const int64_t k = exc_runs(reinterpret_cast<const unsigned char*>(seqs[i]), lens[i], nullptr);
        if (ne + k > c->exc_cap) return fail(HG_ERR_CAPACITY, "hg_submit_ascii: exception runs exceed the context capacity");
        exc_runs(reinterpret_cast<const unsigned char*>(seqs[i]), lens[i], sexc + 3 * ne);
        ne += k;
    }
    seoff[n] = ne;
    return submit_tail(c, n, pb, ne);
}

extern "C" int hg_poll(hg_ctx_t* c)
{
    if (!c || c->async_n < 0) return -HG_ERR_ARG;
    cudaSetDevice(c->ix->device);
    const cudaError_t e = cudaEventQuery(c->done_ev);
    if (e == cudaSuccess) return 1;
    if (e == cudaErrorNotReady) return 0;
    cuda_fail(e, "hg_poll");
    return -HG_ERR_CUDA;
}

extern "C" int hg_collect(hg_ctx_t* c, uint32_t* cigar, int64_t cigar_cap, int64_t* cigar_off, uint8_t* has_ins,
                          uint32_t* status)
{
    if (!c || c->async_n < 0) return fail(HG_ERR_ARG, "hg_collect: nothing submitted");
    cudaSetDevice(c->ix->device);
    HG_CUDA(cudaEventSynchronize(c->done_ev));
    const int64_t n = c->async_n, M = c->max_n + 1;
    c->async_exc_over = c->async_ascii && *c->pipe[0].h_excflag;
    if (c->async_exc_over) {  // the device packing found more exception runs than the context holds
        c->async_n = -1;
        return fail(HG_ERR_CAPACITY, "hg_collect: the exception runs (bytes other than A/C/G/T) of the batch exceed "
                                     "the context's " + std::to_string(c->exc_cap));
    }
    const int64_t* off = c->h_i64 + 4 * M;
    const int64_t total = off[n];
    if (total > cigar_cap) return fail(HG_ERR_CAPACITY, "hg_collect: cigar buffer too small");
    if (total <= c->h_cig_cap) {  // already in host memory
        if (total) std::memcpy(cigar, c->h_cig, 4 * (size_t)total);
    } else {
        const int64_t piece = (int64_t)c->cig_compact.n;
        for (int64_t done = 0; done < total; done += piece) {
            const int64_t m = std::min(piece, total - done);
            compact_copy_kernel<<<c->sms, 256, 0, c->st>>>(c->cig.p, c->coff.p, c->n_cig.p, c->cig_off.p, (int)n,
                                                           c->cig_compact.p, m, done);
            HG_CUDA(cudaGetLastError());
            HG_CUDA(cudaMemcpyAsync(cigar + done, c->cig_compact.p, 4 * (size_t)m, cudaMemcpyDeviceToHost, c->st));
        }
        HG_CUDA(cudaEventRecord(c->collected_ev, c->st));
        HG_CUDA(cudaEventSynchronize(c->collected_ev));
    }
    for (int64_t i = 0; i <= n; ++i) cigar_off[i] = off[i];
    if (has_ins) std::memcpy(has_ins, c->h_has_ins, (size_t)n);
    if (status) std::memcpy(status, c->h_status, 4 * (size_t)n);
    c->async_n = -1;
    return status_error(c->h_status, n);
}

// ---------------------------------------------------------- single calls

extern "C" int64_t hg_global_align_ksw2(const char* ref, int64_t rlen, const char* qry, int64_t qlen, int flag,
                                        uint32_t* cigar, int64_t cap)
{  // globalAlignKSW2 (src/align/align.cpp:22-65)
    if (rlen < 0 || qlen < 0) return -fail(HG_ERR_ARG, "hg_global_align_ksw2: bad lengths");
    if (rlen == 0 || qlen == 0) {
        if (rlen == 0 && qlen > 0) {
            if (cap < 1) return -fail(HG_ERR_CAPACITY, "cigar capacity");
            cigar[0] = (uint32_t)qlen << 4 | 1u;
            return 1;
        }
        if (qlen == 0 && rlen > 0) {
            if (cap < 1) return -fail(HG_ERR_CAPACITY, "cigar capacity");
            cigar[0] = (uint32_t)rlen << 4 | 2u;
            return 1;
        }
        return 0;
    }
    std::vector<uint8_t> re((size_t)rlen), qe((size_t)qlen);
    for (int64_t i = 0; i < rlen; ++i) re[i] = hg::dna5_of((uint8_t)ref[i]);
    for (int64_t i = 0; i < qlen; ++i) qe[i] = hg::dna5_of((uint8_t)qry[i]);
    static const int8_t mat[25] = {5, -4, -4, -4, 0, -4, 5, -4, -4, 0, -4, -4, 5, -4, 0,
                                   -4, -4, -4, 5, 0, 0, 0, 0, 0, 0};
    const int w = hg::auto_band((int)rlen, (int)qlen);
    int32_t ez[10];
    return hg_ksw_extz2((int)qlen, qe.data(), (int)rlen, re.data(), 5, mat, 6, 2, w, -1, 0,
                        flag < 0 ? (hg::kEzGenericSc | hg::kEzRight) : flag, ez, cigar, cap);
}

extern "C" int64_t hg_extend_align_ksw2(const char* ref, int64_t rlen, const char* qry, int64_t qlen, int zdrop,
                                        uint32_t* cigar, int64_t cap)
{  // extendAlignKSW2 (src/align/align.cpp:68-107)
    if (rlen < 0 || qlen < 0 || (rlen > 0 && !ref) || (qlen > 0 && !qry))
        return -fail(HG_ERR_ARG, "hg_extend_align_ksw2: bad arguments");
    if (rlen == 0 || qlen == 0) return 0;  // ksw_extz2_sse returns an empty result
    std::vector<uint8_t> re((size_t)rlen), qe((size_t)qlen);
    for (int64_t i = 0; i < rlen; ++i) re[i] = hg::dna5_of((uint8_t)ref[i]);
    for (int64_t i = 0; i < qlen; ++i) qe[i] = hg::dna5_of((uint8_t)qry[i]);
    static const int8_t mat[25] = {5, -4, -4, -4, 0, -4, 5, -4, -4, 0, -4, -4, 5, -4, 0,
                                   -4, -4, -4, 5, 0, 0, 0, 0, 0, 0};
    int32_t ez[10];
    return hg_ksw_extz2((int)qlen, qe.data(), (int)rlen, re.data(), 5, mat, 6, 2, hg::auto_band((int)rlen, (int)qlen),
                        zdrop, 50, hg::kEzExtzOnly | hg::kEzRight | hg::kEzApproxDrop, ez, cigar, cap);
}

// align::globalAlignMM2 with the caller's anchors against the index's center
// (src/align/align.cpp:189-305): the anchors are sorted as chainAnchors sorts
// them (pos_ref, pos_qry; one center, forward strand), then the chain, gap-
// fill and stitch stages run on one query without minimizer extraction.
namespace {
int global_align_mm2_impl(hg_index_t* ix, const char* qry, int64_t qlen, const uint32_t* anchor_ref,
                          const uint32_t* anchor_qry, int64_t n_anchors, uint32_t* cigar, int64_t cap,
                          uint32_t* status, int64_t* n_out)
{
    if (!ix || (!qry && qlen > 0) || qlen < 0 || qlen > INT32_MAX || n_anchors < 0 ||
        (n_anchors > 0 && (!anchor_ref || !anchor_qry)) || (cap > 0 && !cigar))
        return fail(HG_ERR_ARG, "hg_global_align_mm2: bad arguments");
    std::lock_guard<std::mutex> lock(ix->single_mu);
    const int64_t need_bases = std::max<int64_t>(qlen, 1);
    const int64_t need_bases_for_anchors = (std::max<int64_t>(n_anchors - 65536, 0)) * 4;
    const int64_t want = std::max({need_bases, need_bases_for_anchors, (int64_t)65536});
    if (!ix->single || ix->single->max_bases < want) {
        if (ix->single) hg_ctx_destroy(ix->single), ix->single = nullptr;
        int r = hg_ctx_create(ix, 1, want, &ix->single);
        if (r) return r;
    }
    hg_ctx_t* c = ix->single;
    if (n_anchors > c->acap) return fail(HG_ERR_CAPACITY, "hg_global_align_mm2: too many anchors");
    cudaSetDevice(ix->device);
    const int64_t offs[2] = {0, qlen};
    int64_t pb = 0, ne = 0;
    int r = hg_pack(qry, offs, 1, nullptr, 0, nullptr, nullptr, 0, nullptr, &pb, &ne);
    if (r) return r;
    std::vector<uint8_t> pk((size_t)std::max<int64_t>(pb, 16));
    std::vector<int64_t> poff(1), eoff(2);
    std::vector<int32_t> exc((size_t)std::max<int64_t>(ne, 1) * 3);
    r = hg_pack(qry, offs, 1, pk.data(), (int64_t)pk.size(), poff.data(), exc.data(), ne, eoff.data(), nullptr,
                nullptr);
    if (r) return r;
    // chainAnchors' order for one center on the forward strand: (pos_ref, pos_qry)
    std::vector<uint64_t> key((size_t)n_anchors);
    for (int64_t i = 0; i < n_anchors; ++i) key[i] = (uint64_t)anchor_ref[i] << 32 | anchor_qry[i];
    std::sort(key.begin(), key.end());
    std::vector<uint32_t> ar((size_t)n_anchors), aq((size_t)n_anchors);
    for (int64_t i = 0; i < n_anchors; ++i) ar[i] = (uint32_t)(key[i] >> 32), aq[i] = (uint32_t)key[i];
    const int32_t ql = (int32_t)qlen;
    const int64_t zero64 = 0, coff0 = 0;
    const int32_t na = (int32_t)n_anchors;
    cudaStream_t st = c->st;
    HG_CUDA(cudaMemcpyAsync(c->packed.p, pk.data(), pk.size(), cudaMemcpyHostToDevice, st));
    if (ne) HG_CUDA(cudaMemcpyAsync(c->exc.p, exc.data(), 12 * (size_t)ne, cudaMemcpyHostToDevice, st));
    HG_CUDA(cudaMemcpyAsync(c->poff.p, &zero64, 8, cudaMemcpyHostToDevice, st));
    HG_CUDA(cudaMemcpyAsync(c->qlen.p, &ql, 4, cudaMemcpyHostToDevice, st));
    HG_CUDA(cudaMemcpyAsync(c->exc_off.p, eoff.data(), 16, cudaMemcpyHostToDevice, st));
    HG_CUDA(cudaMemcpyAsync(c->coff.p, &coff0, 8, cudaMemcpyHostToDevice, st));
    HG_CUDA(cudaMemcpyAsync(c->hoff.p, &zero64, 8, cudaMemcpyHostToDevice, st));
    if (n_anchors) {
        HG_CUDA(cudaMemcpyAsync(c->a_ref.p, ar.data(), 4 * (size_t)n_anchors, cudaMemcpyHostToDevice, st));
        HG_CUDA(cudaMemcpyAsync(c->a_qry.p, aq.data(), 4 * (size_t)n_anchors, cudaMemcpyHostToDevice, st));
    }
    HG_CUDA(cudaMemcpyAsync(c->a_base.p, &zero64, 8, cudaMemcpyHostToDevice, st));
    HG_CUDA(cudaMemcpyAsync(c->a_n.p, &na, 4, cudaMemcpyHostToDevice, st));
    hg::BatchDev b = batch_view(c, 1, c->packed.p, c->poff.p, c->qlen.p, c->exc.p, c->exc_off.p, nullptr, c->hoff.p,
                                c->coff.p);
    HG_CUDA(cudaMemsetAsync(c->control.p, 0, sizeof(unsigned long long) * kControlWords, st));
    HG_CUDA(cudaMemsetAsync(c->status.p, 0, 4, st));
    HG_CUDA(cudaMemsetAsync(c->shape_hist.p, 0, sizeof(uint32_t) * hg::kShapeBins, st));
    HG_CUDA(cudaMemsetAsync(c->wave_hist.p, 0, sizeof(uint32_t) * kSortHistWords, st));
    const hg::IndexDev& d = ix->dev;
    HG_CUDA(hg_launch_chain(&d, &b, 1, st));
    HG_CUDA(hg_launch_dp_small(&d, &b, c->sms, st));
    HG_CUDA(hg_launch_dp_thin(&d, &b, c->sms, st));
    HG_CUDA(hg_launch_dp_wave(&d, &b, c->sms, st));
    HG_CUDA(hg_launch_dp_wide(&d, &b, c->sms, st));
    HG_CUDA(hg_launch_dp_large(&d, &b, c->sms, st));
    HG_CUDA(hg_launch_stitch(&d, &b, 1, st));
    int32_t ncig = 0;
    uint32_t stv = 0;
    HG_CUDA(cudaMemcpyAsync(&ncig, c->n_cig.p, 4, cudaMemcpyDeviceToHost, st));
    HG_CUDA(cudaMemcpyAsync(&stv, c->status.p, 4, cudaMemcpyDeviceToHost, st));
    HG_CUDA(cudaStreamSynchronize(st));
    if (status) *status = stv;
    if (stv & HG_ST_ARENA_OVERFLOW) return fail(HG_ERR_CAPACITY, "hg_global_align_mm2: device arena overflow");
    if (stv & HG_ST_CIGAR_OVERFLOW) return fail(HG_ERR_CIGAR, "hg_global_align_mm2: CIGAR length overflow");
    if (ncig > cap) return fail(HG_ERR_CAPACITY, "hg_global_align_mm2: CIGAR capacity");
    if (ncig) HG_CUDA(cudaMemcpy(cigar, c->cig.p, 4 * (size_t)ncig, cudaMemcpyDeviceToHost));
    *n_out = ncig;
    return HG_OK;
}
}  // namespace

extern "C" int64_t hg_global_align_mm2(hg_index_t* ix, const char* qry, int64_t qlen, const uint32_t* anchor_ref,
                                       const uint32_t* anchor_qry, int64_t n_anchors, uint32_t* cigar, int64_t cap,
                                       uint32_t* status)
{
    int64_t n = 0;
    const int r = global_align_mm2_impl(ix, qry, qlen, anchor_ref, anchor_qry, n_anchors, cigar, cap, status, &n);
    return r ? -(int64_t)r : n;
}

extern "C" int64_t hg_align_query(hg_index_t* ix, const char* qry, int64_t qlen, uint32_t* cigar, int64_t cap,
                                  uint32_t* status)
{
    if (!ix || (!qry && qlen > 0) || qlen < 0) return -fail(HG_ERR_ARG, "hg_align_query: bad arguments");
    std::lock_guard<std::mutex> lock(ix->single_mu);
    const int64_t need_bases = std::max<int64_t>(qlen, 1);
    if (!ix->single || ix->single->max_bases < need_bases) {
        if (ix->single) hg_ctx_destroy(ix->single), ix->single = nullptr;
        int r = hg_ctx_create(ix, 1, std::max<int64_t>(need_bases, 65536), &ix->single);
        if (r) return -r;
    }
    const int64_t offs[2] = {0, qlen};
    int64_t pb = 0, ne = 0;
    int r = hg_pack(qry, offs, 1, nullptr, 0, nullptr, nullptr, 0, nullptr, &pb, &ne);
    if (r) return -r;
    std::vector<uint8_t> pk((size_t)std::max<int64_t>(pb, 16));
    std::vector<int64_t> poff(1), eoff(2);
    std::vector<int32_t> exc((size_t)std::max<int64_t>(ne, 1) * 3);
    r = hg_pack(qry, offs, 1, pk.data(), (int64_t)pk.size(), poff.data(), exc.data(), ne, eoff.data(), nullptr,
                nullptr);
    if (r) return -r;
    const int32_t ql = (int32_t)qlen;
    std::vector<uint32_t> cig((size_t)(qlen + ix->L + 8));
    int64_t coff[2];
    uint32_t st = 0;
    r = hg_align_plain(ix->single, pk.data(), poff.data(), &ql, exc.data(), eoff.data(), 1, cig.data(),
                       (int64_t)cig.size(), coff, nullptr, nullptr, 0, &st);
    if (status) *status = st;
    if (r && r != HG_ERR_LENGTH_MISMATCH) return -r;
    const int64_t m = coff[1] - coff[0];
    if (m > cap) return -fail(HG_ERR_CAPACITY, "hg_align_query: CIGAR capacity");
    std::copy(cig.begin(), cig.begin() + m, cigar);
    return m;
}
