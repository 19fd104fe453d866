// ref_harness.cpp - C-callable wrapper around the UNMODIFIED HAlign-4 sources
// of the align-to-center path, compiled directly from the reference tree by
// oracle/build.py into oracle/_ref/libhalign_ref.so.
//
// TEST INFRASTRUCTURE ONLY. This library is the ground truth that pins the C
// restatement in oracle/halign_oracle.c and generates tests/golden fixtures.
// Nothing in the product links or loads it; bench.py never runs it on the GPU
// host (the reference sources are not present there).
//
// Each entry point calls exactly one reference function:
//   ref_extract_minimizer -> minimizer::extractMinimizer   (src/seed/minimizer.cpp:103-177)
//   ref_collect_anchors   -> minimizer::collect_anchors    (src/seed/minimizer.cpp:220-356)
//   ref_chain_anchors     -> anchor::chainAnchors          (src/seed/anchor.cpp:332-461)
//   ref_chain_score       -> anchor::chainScoreSimple      (src/seed/anchor.cpp:254-301)
//   ref_ksw_extz2         -> ksw_extz2_sse                 (src/align/ksw2_extz2_sse.c:23-304)
//   ref_global_align_ksw2 -> align::globalAlignKSW2        (src/align/align.cpp:22-65)
//   ref_global_align_mm2  -> align::globalAlignMM2         (src/align/align.cpp:189-305)
//   ref_align_query       -> RefAligner::globalAlign body  (src/align/ref_aligner.cpp:91-125)
//   ref_del_query         -> cigar::delQueryToRefByCigar   (src/align/cigar.cpp:212-299)
//   ref_pick_consensus    -> consensus::pickConsensusChar  (src/consensus/consensus.cpp:18-35)
//   ref_hash2bit          -> getHash2bit                   (src/mash/hash.cpp)
//   ref_sketch            -> mash::sketchFromSequence      (src/mash/mash.cpp:32-117)
//   ref_jaccard           -> mash::jaccard                 (src/mash/mash.cpp:120-164)
//   ref_align_batch       -> the OpenMP schedule(dynamic,1) query loop of
//                            RefAligner::alignQueryToRef (src/align/ref_aligner.cpp:362-372)
//                            over RefAligner::globalAlign, without the sketch.
#include "align.h"
#include "anchor.h"
#include "consensus.h"
#include "hash.h"
#include "ksw2.h"
#include "mash.h"
#include "seed.h"

#include <omp.h>

#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

extern "C" {
#include "alignment/cigar.h"
#include "wavefront/wavefront_align.h"

// WFA2 is only reached through align::globalAlignWFA2, which is off the
// align-to-center path; these definitions satisfy the linker and abort if
// ever called.
wavefront_aligner_attr_t wavefront_aligner_attr_default;
wavefront_aligner_t* wavefront_aligner_new(wavefront_aligner_attr_t*) { abort(); }
void wavefront_aligner_delete(wavefront_aligner_t*) { abort(); }
int wavefront_align(wavefront_aligner_t*, const char*, const int, const char*, const int) { abort(); }
void cigar_get_CIGAR(cigar_t*, const bool, uint32_t**, int*) { abort(); }
}

namespace {

struct AnchorArrays {
    uint64_t* hash;
    uint32_t* rid_ref;
    uint32_t* pos_ref;
    uint32_t* rid_qry;
    uint32_t* pos_qry;
    uint32_t* span;
    uint8_t* is_rev;
};

anchor::Anchors load_anchors(const AnchorArrays& a, int64_t n)
{
    anchor::Anchors v(static_cast<size_t>(n));
    for (int64_t i = 0; i < n; ++i) {
        v[i].hash = a.hash[i];
        v[i].rid_ref = a.rid_ref[i];
        v[i].pos_ref = a.pos_ref[i];
        v[i].rid_qry = a.rid_qry[i];
        v[i].pos_qry = a.pos_qry[i];
        v[i].span = a.span[i];
        v[i].is_rev = a.is_rev[i] != 0;
    }
    return v;
}

int64_t store_anchors(const anchor::Anchors& v, const AnchorArrays& a, int64_t cap)
{
    const int64_t n = static_cast<int64_t>(v.size());
    if (n > cap) return -n;
    for (int64_t i = 0; i < n; ++i) {
        a.hash[i] = v[i].hash;
        a.rid_ref[i] = v[i].rid_ref;
        a.pos_ref[i] = v[i].pos_ref;
        a.rid_qry[i] = v[i].rid_qry;
        a.pos_qry[i] = v[i].pos_qry;
        a.span[i] = v[i].span;
        a.is_rev[i] = v[i].is_rev ? 1 : 0;
    }
    return n;
}

int64_t store_cigar(const cigar::Cigar_t& c, uint32_t* out, int64_t cap)
{
    const int64_t n = static_cast<int64_t>(c.size());
    if (n > cap) return -n;
    if (n) std::memcpy(out, c.data(), sizeof(uint32_t) * static_cast<size_t>(n));
    return n;
}

minimizer::MinimizerHits load_hits(const uint64_t* xs, const uint64_t* ys, int64_t n)
{
    minimizer::MinimizerHits h(static_cast<size_t>(n));
    for (int64_t i = 0; i < n; ++i) h[i] = minimizer::MinimizerHit(xs[i], ys[i]);
    return h;
}

anchor::SeedFilterParams make_filter(const double* fp)
{
    anchor::SeedFilterParams p;
    if (fp) {
        p.f_top_frac = fp[0];
        p.u_floor = static_cast<size_t>(fp[1]);
        p.u_ceil = static_cast<size_t>(fp[2]);
        p.q_occ_frac = fp[3];
        p.sample_every_bp = static_cast<size_t>(fp[4]);
    }
    return p;
}

anchor::ChainParams make_chain(const int32_t* ip, const float* fp)
{
    anchor::ChainParams p;
    if (ip) {
        p.max_dist_x = ip[0];
        p.max_dist_y = ip[1];
        p.bw = ip[2];
        p.max_skip = ip[3];
        p.max_iter = ip[4];
        p.min_cnt = ip[5];
        p.min_score = ip[6];
    }
    if (fp) {
        p.gap_penalty = fp[0];
        p.skip_penalty = fp[1];
    }
    return p;
}

}  // namespace

extern "C" {

int64_t ref_extract_minimizer(const char* seq, int64_t n, int k, int w, int non_canonical,
                              uint64_t* xs, uint64_t* ys, int64_t cap)
{
    const std::string s(seq, static_cast<size_t>(n));
    const auto hits = minimizer::extractMinimizer(s, static_cast<size_t>(k), static_cast<size_t>(w),
                                                  non_canonical != 0);
    const int64_t m = static_cast<int64_t>(hits.size());
    if (m > cap) return -m;
    for (int64_t i = 0; i < m; ++i) {
        xs[i] = hits[i].x;
        ys[i] = hits[i].y;
    }
    return m;
}

// filter: {f_top_frac, u_floor, u_ceil, q_occ_frac, sample_every_bp} or NULL for defaults
int64_t ref_collect_anchors(const uint64_t* rx, const uint64_t* ry, int64_t nr,
                            const uint64_t* qx, const uint64_t* qy, int64_t nq,
                            const double* filter,
                            uint64_t* hash, uint32_t* rid_ref, uint32_t* pos_ref, uint32_t* rid_qry,
                            uint32_t* pos_qry, uint32_t* span, uint8_t* is_rev, int64_t cap)
{
    const auto r = load_hits(rx, ry, nr);
    const auto q = load_hits(qx, qy, nq);
    const auto anchors = minimizer::collect_anchors(r, q, make_filter(filter));
    return store_anchors(anchors, AnchorArrays{hash, rid_ref, pos_ref, rid_qry, pos_qry, span, is_rev}, cap);
}

// Runs chainAnchors; the input arrays are overwritten with the sorted input
// (chainAnchors sorts its argument in place) and the best chain goes to out_*.
int64_t ref_chain_anchors(uint64_t* hash, uint32_t* rid_ref, uint32_t* pos_ref, uint32_t* rid_qry,
                          uint32_t* pos_qry, uint32_t* span, uint8_t* is_rev, int64_t n,
                          const int32_t* iparams, const float* fparams,
                          uint64_t* o_hash, uint32_t* o_rid_ref, uint32_t* o_pos_ref, uint32_t* o_rid_qry,
                          uint32_t* o_pos_qry, uint32_t* o_span, uint8_t* o_is_rev, int64_t cap)
{
    AnchorArrays in{hash, rid_ref, pos_ref, rid_qry, pos_qry, span, is_rev};
    auto v = load_anchors(in, n);
    const auto chain = anchor::chainAnchors(v, make_chain(iparams, fparams));
    store_anchors(v, in, n);
    return store_anchors(chain, AnchorArrays{o_hash, o_rid_ref, o_pos_ref, o_rid_qry, o_pos_qry, o_span, o_is_rev},
                         cap);
}

int32_t ref_chain_score(uint32_t ai_ref, uint32_t ai_qry, uint32_t aj_ref, uint32_t aj_qry, uint32_t aj_span)
{
    anchor::Anchor ai, aj;
    ai.pos_ref = ai_ref;
    ai.pos_qry = ai_qry;
    aj.pos_ref = aj_ref;
    aj.pos_qry = aj_qry;
    aj.span = aj_span;
    return anchor::chainScoreSimple(ai, aj, anchor::default_chain_params());
}

// out_i: {max, zdropped, max_q, max_t, mqe, mqe_t, mte, mte_q, score, reach_end}
int64_t ref_ksw_extz2(int qlen, const uint8_t* query, int tlen, const uint8_t* target, int8_t m,
                      const int8_t* mat, int8_t q, int8_t e, int w, int zdrop, int end_bonus, int flag,
                      int32_t* out_i, uint32_t* cigar, int64_t cap)
{
    ksw_extz_t ez{};
    ksw_extz2_sse(nullptr, qlen, query, tlen, target, m, mat, q, e, w, zdrop, end_bonus, flag, &ez);
    out_i[0] = static_cast<int32_t>(ez.max);
    out_i[1] = static_cast<int32_t>(ez.zdropped);
    out_i[2] = ez.max_q;
    out_i[3] = ez.max_t;
    out_i[4] = ez.mqe;
    out_i[5] = ez.mqe_t;
    out_i[6] = ez.mte;
    out_i[7] = ez.mte_q;
    out_i[8] = ez.score;
    out_i[9] = ez.reach_end;
    int64_t n = ez.n_cigar;
    if (n > cap) n = -n;
    else if (n > 0) std::memcpy(cigar, ez.cigar, sizeof(uint32_t) * static_cast<size_t>(n));
    free(ez.cigar);
    return n;
}

// flag < 0 keeps KSW2AlignConfig's default flag (GENERIC_SC|RIGHT)
int64_t ref_global_align_ksw2(const char* ref, int64_t rlen, const char* qry, int64_t qlen, int flag,
                              uint32_t* cigar, int64_t cap)
{
    align::KSW2AlignConfig cfg;
    if (flag >= 0) cfg.flag = flag;
    const auto c = align::globalAlignKSW2(std::string(ref, rlen), std::string(qry, qlen), cfg);
    return store_cigar(c, cigar, cap);
}

int64_t ref_global_align_mm2(const char* ref, int64_t rlen, const char* qry, int64_t qlen,
                             uint64_t* hash, uint32_t* rid_ref, uint32_t* pos_ref, uint32_t* rid_qry,
                             uint32_t* pos_qry, uint32_t* span, uint8_t* is_rev, int64_t n,
                             uint32_t* cigar, int64_t cap)
{
    const auto anchors = load_anchors(AnchorArrays{hash, rid_ref, pos_ref, rid_qry, pos_qry, span, is_rev}, n);
    const auto c = align::globalAlignMM2(std::string(ref, rlen), std::string(qry, qlen), anchors);
    return store_cigar(c, cigar, cap);
}

int64_t ref_align_query(const char* center, int64_t clen, const char* qry, int64_t qlen, int k, int w,
                        uint32_t* cigar, int64_t cap)
{
    const std::string ref(center, clen), q(qry, qlen);
    const auto rmz = minimizer::extractMinimizer(ref, k, w, true);
    const auto qmz = minimizer::extractMinimizer(q, k, w, true);
    const auto anchors = minimizer::collect_anchors(rmz, qmz);
    const auto c = align::globalAlignMM2(ref, q, anchors);
    return store_cigar(c, cigar, cap);
}

// Aligns n queries (concatenated, offsets[n+1]) to the center with nthreads
// OpenMP threads, schedule(dynamic,1). CIGAR of query i goes to
// cigar[i*cap_per_query ...], its op count to n_cigar[i] (negative = overflow).
// Returns the wall time in seconds of the parallel loop.
double ref_align_batch(const char* center, int64_t clen, const char* seqs, const int64_t* offsets, int64_t n,
                       int k, int w, int nthreads, uint32_t* cigar, int64_t cap_per_query, int64_t* n_cigar)
{
    const std::string ref(center, clen);
    const auto rmz = minimizer::extractMinimizer(ref, k, w, true);
    const double t0 = omp_get_wtime();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
    for (int64_t i = 0; i < n; ++i) {
        const std::string q(seqs + offsets[i], static_cast<size_t>(offsets[i + 1] - offsets[i]));
        const auto qmz = minimizer::extractMinimizer(q, k, w, true);
        const auto anchors = minimizer::collect_anchors(rmz, qmz);
        const auto c = align::globalAlignMM2(ref, q, anchors);
        n_cigar[i] = store_cigar(c, cigar + i * cap_per_query, cap_per_query);
    }
    return omp_get_wtime() - t0;
}

// Projects a query onto the center by its CIGAR (I removed, D -> '-').
// Returns the row length written to out (capacity cap), or -needed.
int64_t ref_del_query(const char* qry, int64_t qlen, const uint32_t* cigar, int64_t n_cigar, char* out, int64_t cap)
{
    std::string q(qry, qlen);
    cigar::delQueryToRefByCigar(q, cigar::Cigar_t(cigar, cigar + n_cigar));
    const int64_t m = static_cast<int64_t>(q.size());
    if (m > cap) return -m;
    std::memcpy(out, q.data(), static_cast<size_t>(m));
    return m;
}

// padQueryToRefByCigar (insertions kept, D -> '-').
int64_t ref_pad_query(const char* qry, int64_t qlen, const uint32_t* cigar, int64_t n_cigar, char* out, int64_t cap)
{
    std::string q(qry, qlen);
    cigar::padQueryToRefByCigar(q, cigar::Cigar_t(cigar, cigar + n_cigar));
    const int64_t m = static_cast<int64_t>(q.size());
    if (m > cap) return -m;
    std::memcpy(out, q.data(), static_cast<size_t>(m));
    return m;
}

int64_t ref_extend_align_ksw2(const char* ref, int64_t rlen, const char* qry, int64_t qlen, int zdrop,
                              uint32_t* cigar, int64_t cap)
{
    const auto c = align::extendAlignKSW2(std::string(ref, rlen), std::string(qry, qlen), zdrop);
    return store_cigar(c, cigar, cap);
}

// generateConsensusSequence on an aligned FASTA; the consensus goes to out
// (capacity cap), the files to out_fasta / out_json.  Returns its length.
int64_t ref_generate_consensus(const char* aligned_fasta, const char* out_fasta, const char* out_json,
                               uint64_t seq_limit, int64_t batch_size, char* out, int64_t cap)
{
    const std::string s = consensus::generateConsensusSequence(aligned_fasta, out_fasta, out_json, seq_limit, 1,
                                                               static_cast<size_t>(batch_size));
    const int64_t m = static_cast<int64_t>(s.size());
    if (m > cap) return -m;
    std::memcpy(out, s.data(), static_cast<size_t>(m));
    return m;
}

int64_t ref_cigar_to_string(const uint32_t* cigar, int64_t n, char* out, int64_t cap)
{
    const auto s = cigar::cigarToString(cigar::Cigar_t(cigar, cigar + n));
    const int64_t m = static_cast<int64_t>(s.size());
    if (m + 1 > cap) return -m;
    std::memcpy(out, s.c_str(), static_cast<size_t>(m + 1));
    return m;
}

// counts: {a,c,g,t,u,n,dash}
char ref_pick_consensus(const uint32_t* counts)
{
    consensus::SiteCount sc;
    sc.a = counts[0];
    sc.c = counts[1];
    sc.g = counts[2];
    sc.t = counts[3];
    sc.u = counts[4];
    sc.n = counts[5];
    sc.dash = counts[6];
    return consensus::pickConsensusChar(sc);
}

int ref_auto_band(int qlen, int tlen) { return align::auto_band(qlen, tlen); }

uint64_t ref_hash2bit(uint64_t code, uint32_t seed) { return getHash2bit(code, seed); }

// mash::sketchFromSequence into out (capacity cap); returns the sketch size
int64_t ref_sketch(const char* seq, int64_t n, int k, int64_t sketch_size, int noncanonical, int seed, uint64_t* out,
                   int64_t cap)
{
    const mash::Sketch sk = mash::sketchFromSequence(std::string(seq, static_cast<size_t>(n)), static_cast<size_t>(k),
                                                     static_cast<size_t>(sketch_size), noncanonical != 0, seed);
    const int64_t m = static_cast<int64_t>(sk.hashes.size());
    if (m > cap) return -m;
    std::memcpy(out, sk.hashes.data(), sizeof(uint64_t) * static_cast<size_t>(m));
    return m;
}

double ref_jaccard(const uint64_t* a, int64_t na, const uint64_t* b, int64_t nb, int k)
{
    mash::Sketch x, y;
    x.k = y.k = static_cast<size_t>(k);
    x.hashes.assign(a, a + na);
    y.hashes.assign(b, b + nb);
    return mash::jaccard(x, y);
}

}  // extern "C"
