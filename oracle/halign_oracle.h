/* halign_oracle.h - CPU restatement of HAlign-4's align-to-center path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker: tests/, the smoke check
 * and bench.py's CPU-baseline leg call it to verify and to time the CPU path.
 * The product (the CUDA library in halign-4_gb300/) never links or calls it.
 *
 * Parity pin: every function here is checked against the unmodified reference
 * sources compiled by oracle/build.py (oracle/_ref/libhalign_ref.so, the
 * reference CLI oracle/_ref/halign4) and against golden vectors in
 * tests/golden that those produced.
 */
#ifndef HALIGN_ORACLE_H
#define HALIGN_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Mirrors anchor::Anchor (include/anchor.h:39-50). */
typedef struct {
    uint64_t hash;
    uint32_t rid_ref, pos_ref, rid_qry, pos_qry, span;
    uint32_t is_rev;
} ho_anchor;

/* Mirrors anchor::ChainParams (include/anchor.h:116-127). */
typedef struct {
    int32_t max_dist_x, max_dist_y, bw, max_skip, max_iter, min_cnt, min_score;
    float gap_penalty, skip_penalty;
} ho_chain_params;

/* Mirrors anchor::SeedFilterParams (include/anchor.h:65-71). */
typedef struct {
    double f_top_frac;
    uint64_t u_floor, u_ceil;
    double q_occ_frac;
    uint64_t sample_every_bp;
} ho_filter_params;

/* Mirrors ksw_extz_t (include/ksw2.h:33-42) minus the CIGAR buffer. */
typedef struct {
    int32_t max, zdropped, max_q, max_t, mqe, mqe_t, mte, mte_q, score, reach_end;
} ho_extz;

void ho_default_chain_params(ho_chain_params* p);
void ho_default_filter_params(ho_filter_params* p);

/* log2f(x) for x = 0..512 as produced by the reference host's libm; the
 * chain-score penalty only evaluates it at 2..501. */
const float* ho_log2_table(void);

/* A1: minimizer::extractMinimizer (src/seed/minimizer.cpp:103-177). Packed
 * MinimizerHit words (x = hash56<<8|span, y = strand<<63|rid<<32|pos).
 * Returns the hit count, or -count when cap is too small. */
int64_t ho_extract_minimizer(const char* seq, int64_t n, int k, int w, int non_canonical,
                             uint64_t* xs, uint64_t* ys, int64_t cap);

/* Ring-slot indices past the window capacity used by the last call on this
 * thread; the reference's RingMinQueue writes past its vector there. */
int64_t ho_last_ring_oob(void);

/* A2: minimizer::collect_anchors (src/seed/minimizer.cpp:220-356). */
int64_t ho_collect_anchors(const uint64_t* rx, const uint64_t* ry, int64_t nr,
                           const uint64_t* qx, const uint64_t* qy, int64_t nq,
                           const ho_filter_params* fp, ho_anchor* out, int64_t cap);
uint64_t ho_ref_occ_threshold(const uint64_t* occs, int64_t n, const ho_filter_params* fp);

/* A3: anchor::chainScoreSimple (src/seed/anchor.cpp:254-301); INT32_MIN if unlinkable. */
int32_t ho_chain_score(const ho_anchor* ai, const ho_anchor* aj, const ho_chain_params* p);
/* A4: anchor::chainAnchors (src/seed/anchor.cpp:332-461). Sorts a[] in place. */
int64_t ho_chain_anchors(ho_anchor* a, int64_t n, const ho_chain_params* p, ho_anchor* out, int64_t cap);
/* The same, also returning the DP arrays of the sorted anchors: f (best chain
 * score ending at each anchor) and p (its predecessor, -1 if none). */
int64_t ho_chain_anchors_fp(ho_anchor* a, int64_t n, const ho_chain_params* p, ho_anchor* out, int64_t cap,
                            int32_t* f_out, int64_t* p_out);

/* A7+A8: ksw_extz2_sse (src/align/ksw2_extz2_sse.c:23-304, SSE2 build) with
 * ksw_backtrack (include/ksw2.h:129-161), with the full matrix
 * (KSW_EZ_GENERIC_SC) or match/mismatch scoring (extendAlignKSW2's).
 * Returns the CIGAR length (or -len when cap is too small). */
int64_t ho_ksw_extz2(int qlen, const uint8_t* query, int tlen, const uint8_t* target, int8_t m,
                     const int8_t* mat, int8_t q, int8_t e, int w, int zdrop, int end_bonus, int flag,
                     ho_extz* ez, uint32_t* cigar, int64_t cap);

/* A6: align::auto_band (include/align.h:159-172) and globalAlignKSW2
 * (src/align/align.cpp:22-65). flag < 0 selects GENERIC_SC|RIGHT. */
int ho_auto_band(int qlen, int tlen);
int64_t ho_global_align_ksw2(const char* ref, int64_t rlen, const char* qry, int64_t qlen, int flag,
                             uint32_t* cigar, int64_t cap);

/* A5: align::globalAlignMM2 (src/align/align.cpp:189-305). */
int64_t ho_global_align_mm2(const char* ref, int64_t rlen, const char* qry, int64_t qlen,
                            const ho_anchor* anchors, int64_t n, uint32_t* cigar, int64_t cap);

/* A9: CIGAR algebra (src/align/cigar.cpp). */
int64_t ho_cigar_ref_len(const uint32_t* c, int64_t n);
int64_t ho_cigar_query_len(const uint32_t* c, int64_t n);
int ho_cigar_has_insertion(const uint32_t* c, int64_t n);

/* A12: RefAligner::globalAlign with one center (src/align/ref_aligner.cpp:91-125).
 * center_mz: the center's minimizer hits (x,y) as extractMinimizer returns
 * them; center_dp: the string the DP aligns against (the consensus of the
 * single center record). */
int64_t ho_align_query(const char* center_dp, int64_t clen, const uint64_t* cmx, const uint64_t* cmy,
                       int64_t ncm, const char* qry, int64_t qlen, int k, int w, uint32_t* cigar, int64_t cap);

/* The OpenMP schedule(dynamic,1) query loop of RefAligner::alignQueryToRef
 * (src/align/ref_aligner.cpp:362-372) over ho_align_query. Returns seconds. */
double ho_align_batch(const char* center_dp, int64_t clen, const char* center_raw, int64_t raw_len,
                      const char* seqs, const int64_t* offsets, int64_t n, int k, int w, int nthreads,
                      uint32_t* cigar, int64_t cap_per_query, int64_t* n_cigar);

/* A10: cigar::delQueryToRefByCigar (src/align/cigar.cpp:212-299).
 * Returns the row length (or -len when cap is too small). */
int64_t ho_del_query(const char* qry, int64_t qlen, const uint32_t* c, int64_t n, char* out, int64_t cap);

/* A11: SiteCount accumulation (src/consensus/consensus.cpp:304-411) over
 * rows of length L (counts7: L x {A,C,G,T,U,N,-}), and insertion-event
 * counting (ins: L+1 slots; slot c counts I operations that sit between
 * center columns c-1 and c). */
void ho_count_rows(const char* rows, int64_t n_rows, int64_t L, uint32_t* counts7);
void ho_count_insertions(const uint32_t* c, int64_t n, uint32_t* ins, int64_t L);
char ho_pick_consensus(const uint32_t* counts7);

/* Multi-reference mode (MinHash).
 * ho_hash2bit: getHash2bit (src/mash/hash.cpp), i.e. XXH3_64bits_withSeed of
 *   the 8 big-endian bytes of a 2-bit k-mer code (xxHash 0.8.3, vendored as
 *   include/xxhash.h; the 4..8-byte input branch of the published XXH3).
 * ho_sketch: mash::sketchFromSequence (src/mash/mash.cpp:32-117): the
 *   sketch_size smallest distinct hashes of the valid k-mers, ascending.
 *   Returns the count written (<= sketch_size).
 * ho_jaccard: mash::jaccard (src/mash/mash.cpp:120-164) over sorted
 *   distinct sketches: |a & b| / min(|a|, |b|), 1 when both are empty.
 * ho_best_reference: the selection loop of RefAligner::alignOneQueryToRef
 *   (src/align/ref_aligner.cpp:232-241): first reference of largest
 *   jaccard, strict '>' from -1. */
uint64_t ho_hash2bit(uint64_t code, uint32_t seed);
int64_t ho_sketch(const char* seq, int64_t n, int k, int64_t sketch_size, int noncanonical, int seed,
                  uint64_t* out);
double ho_jaccard(const uint64_t* a, int64_t na, const uint64_t* b, int64_t nb);
int32_t ho_best_reference(const uint64_t* q, int64_t nq, const uint64_t* ref_h, const int64_t* ref_off,
                          int32_t n_refs, double* best_j);

#ifdef __cplusplus
}
#endif
#endif
