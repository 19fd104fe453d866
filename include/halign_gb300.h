/* halign_gb300.h - C ABI of the GB300-native align-to-center path.
 *
 * Plain pointers, sizes and int status codes; no C++ or CUDA types cross the
 * boundary.  One hg_ctx_t owns one CUDA stream and its device buffers; a
 * host thread that shares a context with others must serialise its calls, or
 * use its own context (contexts of one index may run concurrently).
 *
 * Each entry point names the reference interface it replaces (paths in the
 * HAlign-4 source tree).
 */
#ifndef HALIGN_GB300_H
#define HALIGN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HG_OK 0
#define HG_ERR_CUDA 1            /* CUDA runtime error (hg_last_error has the text) */
#define HG_ERR_ARG 2             /* invalid argument / unsupported flag */
#define HG_ERR_NOMEM 3           /* device or host allocation failed */
#define HG_ERR_CAPACITY 4        /* a caller buffer or a configured capacity is too small */
#define HG_ERR_LENGTH_MISMATCH 5 /* a row does not span the center: the reference throws
                                    "Sequence length mismatch" (src/align/ref_aligner.cpp:654-662) */
#define HG_ERR_CIGAR 6           /* CIGAR length above 2^28-1: cigarToInt/appendCigar throw
                                    (src/align/cigar.cpp:51-59, 319-322) */

/* per-query status bits (hg_align_batch's status array) */
#define HG_ST_ARENA_OVERFLOW 0x01u
#define HG_ST_PARTIAL_CIGAR 0x02u
#define HG_ST_CIGAR_OVERFLOW 0x08u
#define HG_ST_LENGTH_MISMATCH 0x10u

typedef struct hg_index hg_index_t;
typedef struct hg_ctx hg_ctx_t;

/* Seeding + chaining parameters; defaults = anchor::SeedFilterParams and
 * anchor::ChainParams (include/anchor.h:65-71, 116-127). */
typedef struct {
    double f_top_frac;
    uint64_t u_floor, u_ceil;
    double q_occ_frac;
    uint64_t sample_every_bp;
    int32_t max_dist_x, max_dist_y, bw, max_skip, max_iter, min_cnt, min_score;
    float gap_penalty, skip_penalty;
} hg_params_t;

/* Last error message of the calling thread. */
const char* hg_last_error(void);
void hg_default_params(hg_params_t* p);
/* Number of visible CUDA devices (0 without a GPU); never fails. */
int hg_device_count(void);
/* Make device `ordinal` current for the calling thread: hg_index_create then
 * places the index (and every context made from it) there, and every later
 * call on that index or its contexts switches to it first.  One process per
 * GPU calls this with its local rank before creating an index.  No reference
 * counterpart (the reference runs on the host). */
int hg_set_device(int ordinal);
/* The device an index lives on: its ordinal and (when pci_bus_id is given)
 * its PCI bus id string, e.g. "0000:1B:00.0" (len >= 13). */
int hg_index_device(const hg_index_t* ix, int* ordinal, char* pci_bus_id, int len);

/* ---- resident center index --------------------------------------------
 * Replaces the per-center set-up of RefAligner (src/align/ref_aligner.cpp:
 * 20-73: consensus of the single -c record, extractMinimizer of the center)
 * and the per-call index build inside minimizer::collect_anchors
 * (src/seed/minimizer.cpp:238-272), done once and kept in HBM.
 * k, w: --kmer-size / --kmer-window.  params may be NULL. */
int hg_index_create(const char* center, int64_t len, int k, int w, const hg_params_t* params, hg_index_t** out);
void hg_index_destroy(hg_index_t* ix);
/* Distinct center minimizer hashes / total center minimizers / the -f/-U
 * occurrence threshold (anchor::compute_ref_occ_threshold). */
int hg_index_info(const hg_index_t* ix, int64_t* n_distinct, int64_t* n_hits, uint64_t* occ_threshold);

/* ---- batch context ------------------------------------------------------
 * max_queries / max_bases bound one device sub-batch; hg_align_batch splits
 * larger inputs into sub-batches internally. */
int hg_ctx_create(hg_index_t* ix, int64_t max_queries, int64_t max_bases, hg_ctx_t** out);
void hg_ctx_destroy(hg_ctx_t* ctx);

/* Pack ASCII queries into the device input format: 2 bits per A/C/G/T
 * (A=0 C=1 G=2 T=3, base i at bits 2*(i%4) of byte i/4), each query on a
 * 16-byte boundary, every other byte kept as an exception run
 * {start, len, byte}.  With packed == NULL only sizes are returned.  With
 * packed given and exc too small (or NULL), the bases are packed, *n_exc and
 * exc_off are set and HG_ERR_CAPACITY is returned: a caller may size `exc`
 * from *n_exc and call again. */
int hg_pack(const char* seqs, const int64_t* offsets, int64_t n, uint8_t* packed, int64_t packed_cap,
            int64_t* poff, int32_t* exc, int64_t exc_cap, int64_t* exc_off, int64_t* packed_bytes,
            int64_t* n_exc);

/* ---- align a batch (the align-to-center hot path) -----------------------
 * Replaces the OpenMP query loop of RefAligner::alignQueryToRef
 * (src/align/ref_aligner.cpp:286-398) over RefAligner::globalAlign
 * (extractMinimizer -> collect_anchors -> globalAlignMM2, :91-125), and the
 * per-row projection of mergeAlignedResults with --keep-length
 * (delQueryToRefByCigar, src/align/ref_aligner.cpp:172-192).
 * Inputs are host buffers in hg_pack's format.  Outputs (host):
 *   cigar/cigar_off: CIGAR of query i at cigar[cigar_off[i] .. cigar_off[i+1])
 *                    (len<<4|op, op 0=M 1=I 2=D), cigar_cap entries;
 *   has_ins[i]:      1 when the CIGAR holds an insertion (the row goes to the
 *                    insertion group, src/align/ref_aligner.cpp:253-259);
 *   rows:            n x row_stride bytes, row i = query i projected onto the
 *                    center (L bytes, then padding), or NULL to skip;
 *   status[i]:       HG_ST_* bits.
 * The per-column SiteCount counters of the context accumulate every row.
 * Returns HG_OK, or the first error (HG_ERR_LENGTH_MISMATCH when a row would
 * not span the center, as the reference's merge throws). */
int hg_align_batch(hg_ctx_t* ctx, const uint8_t* packed, const int64_t* poff, const int32_t* qlen,
                   const int32_t* exc, const int64_t* exc_off, int64_t n, uint32_t* cigar, int64_t cigar_cap,
                   int64_t* cigar_off, uint8_t* has_ins, uint8_t* rows, int64_t row_stride, uint32_t* status);

/* hg_align_batch on ASCII queries (query i = seqs[offsets[i] .. offsets[i+1]),
 * the reference's std::string bytes), packed on the device: each sub-batch's
 * bytes upload as they are while the previous one computes, and kernels pack
 * them into hg_pack's format on the stream that aligns them, so no host pass
 * reads the bases.  Outputs, errors and results are hg_align_batch's on
 * hg_pack's output.  HG_ERR_CAPACITY when a sub-batch holds more exception
 * runs (runs of one byte other than A/C/G/T) than max_bases / 16 + 4096:
 * pack such input with hg_pack.  `seqs` in pinned memory (cudaHostAlloc)
 * lets the uploads overlap the compute; pageable memory is staged by the
 * driver on the calling thread. */
int hg_align_ascii(hg_ctx_t* ctx, const char* seqs, const int64_t* offsets, int64_t n, uint32_t* cigar,
                   int64_t cigar_cap, int64_t* cigar_off, uint8_t* has_ins, uint8_t* rows, int64_t row_stride,
                   uint32_t* status);

/* Same computation, one launch sequence per query (the plain form). */
int hg_align_plain(hg_ctx_t* ctx, const uint8_t* packed, const int64_t* poff, const int32_t* qlen,
                   const int32_t* exc, const int64_t* exc_off, int64_t n, uint32_t* cigar, int64_t cigar_cap,
                   int64_t* cigar_off, uint8_t* has_ins, uint8_t* rows, int64_t row_stride, uint32_t* status);

/* Device-resident form for throughput measurement: hg_stage copies a packed
 * batch into HBM once; hg_run_staged aligns it (outputs stay on the device,
 * counters accumulate); hg_fetch_staged copies the outputs of the last run
 * back in hg_align_batch's layout. */
int hg_stage(hg_ctx_t* ctx, const uint8_t* packed, const int64_t* poff, const int32_t* qlen, const int32_t* exc,
             const int64_t* exc_off, int64_t n);
int hg_run_staged(hg_ctx_t* ctx);
int hg_fetch_staged(hg_ctx_t* ctx, uint32_t* cigar, int64_t cigar_cap, int64_t* cigar_off, uint8_t* has_ins,
                    uint8_t* rows, int64_t row_stride, uint32_t* status);
/* Launch shape of the sub-batch stages, in CTAs per SM: [0] seed (1..32),
 * [1] anchor (1..6), [2] chain (1..64), [3] dp_small (1..32), [4] stitch
 * (1..32), [5] rows (1..32); and two DP tier boundaries: [6] the longest
 * query side the thin tier takes (0..32; 0 switches the tier off), [7] the
 * most cells the square tier takes (0..12288).  Segments a tier declines go
 * to the next one (thin, square, then the wavefront or exact tiers); every
 * tier computes the same alignment, so the knobs change speed only.  [8]
 * small-tier form (0: one segment per thread in int32 lanes; 1: two
 * same-shape segments per thread in the 16-bit halves of 32-bit words).
 * [9] compute lanes of a staged run of several sub-batches (1 or 2): with 2,
 * every other sub-batch runs on a second context of the same capacity and
 * its own streams (created on first use, so the device memory of the
 * context doubles; without room for it the context keeps one lane), and the
 * two overlap on the GPU.  [10] host-buffer calls moving 32 MB or more
 * (inputs + rows): the first two and the last two sub-batches are re-cut
 * so that the first and the last two parts hold s percent (0..24; 0 = off)
 * of their bases each: both lanes start after a small upload, and the rows
 * of the large parts copy to the host while the small last parts compute.
 * Defaults 6 6 12 12 8 6 32 3072 0 2 10.  Setting
 * them drops the context's cached CUDA graphs (the autotuner,
 * halign-4_gb300/autotune.py, searches them).  No reference counterpart:
 * launch geometry. */
#define HG_LAUNCH_KNOBS 11
int hg_ctx_set_launch(hg_ctx_t* ctx, const int32_t* ctas_per_sm, int n);
int hg_ctx_get_launch(const hg_ctx_t* ctx, int32_t* ctas_per_sm, int n);

/* Timing of the last hg_run_staged from CUDA events on the context stream:
 * total device ms (start to end of the run), per-stage ms in stage order
 * seed, anchor, chain, dp_small, dp_large, stitch, rows, count (8 entries,
 * only with hg_set_timing on), and the kernel launches of that run. */
int hg_last_timing(hg_ctx_t* ctx, float* total_ms, float* stage_ms, int64_t* launches, int64_t* cells);
/* cells: extz2 band cells of the last hg_run_staged, i.e. the sum over DP
 * calls of sum_r (en0 - st0 + 1) with the band bounds of
 * src/align/ksw2_extz2_sse.c:107-110 (the GCUPS numerator). */
/* The same cells and the part of them in match segments, whose extz2
 * result (d M) is emitted without running the DP: cells - match_cells is
 * what the DP kernels computed. */
int hg_last_cells(hg_ctx_t* ctx, int64_t* cells, int64_t* match_cells);
/* Work totals of every batched sub-batch since the context was created:
 * counts[0] anchors (after the collect_anchors filters), counts[1] segment
 * records (a run of match segments and anchor spans counts once),
 * counts[2] DP segments (work-list entries of all tiers).  n <= 4 words are
 * written; the difference of two reads is the work of the runs between
 * them (the measurement's unit counts). */
int hg_ctx_work(hg_ctx_t* ctx, int64_t* counts, int n);
/* OR of the HG_ST_* bits of every query of the last hg_run_staged
 * (0 = every query aligned completely). */
int hg_staged_flags(hg_ctx_t* ctx, uint32_t* flags);
/* Integer throughput ceilings of the current GPU, measured by short
 * full-grid kernels (about 20 ms in all): out[0] int32 add + max element
 * operations per second, out[1] DPX max(a + b, c) on int32, out[2] the same
 * on int16x2, out[3] DPX three-way max on int16x2, out[4] 64-bit
 * multiply-adds, out[5] integer-pipe warp instructions per second, out[6]
 * int16x2 subtracts, out[7] int16x2 compares.  n <= 8 values are written.  The roofline of this integer path; no
 * reference counterpart. */
int hg_int_peaks(double* out, int n);

/* Self-test of the small DP tier's two-cells-per-instruction form (int16x2
 * SIMD): every input a band-free cell can see, both gap modes, against the
 * int32 cell; *mismatches gets the disagreeing cases (0 expected).  Test
 * support; no reference counterpart. */
int hg_dp_lane_selftest(uint32_t* mismatches);

/* Enable per-stage event timing for staged runs (off by default). */
int hg_set_timing(hg_ctx_t* ctx, int on);

/* Asynchronous form (continuous batching): hg_submit enqueues one packed
 * batch (within the context's capacity) on the context's stream and returns;
 * hg_poll returns 1 once its results are ready (0 while running, < 0 on
 * error); hg_collect copies them out in hg_align_batch's layout and frees the
 * context for the next hg_submit.  The batch's last kernel writes its
 * compacted CIGARs into mapped pinned memory of the context (up to
 * max_bases / 8 + 64 x max_queries + 1024 ops), so a collect within that
 * size is a host copy with no device work; longer ones are copied out from
 * the device in pieces.  Several contexts of one index overlap on the GPU;
 * each keeps its own stream and arenas. */
int hg_submit(hg_ctx_t* ctx, const uint8_t* packed, const int64_t* poff, const int32_t* qlen, const int32_t* exc,
              const int64_t* exc_off, int64_t n);
/* hg_submit for ASCII queries (seqs[i], lens[i] bytes each): they are packed
 * straight into the context's pinned staging (OpenMP over queries) instead of
 * being packed by the caller and copied there, so a server's host work per
 * request is one pass over its bytes. */
int hg_submit_ascii(hg_ctx_t* ctx, const char* const* seqs, const int64_t* lens, int64_t n);
int hg_poll(hg_ctx_t* ctx);
int hg_collect(hg_ctx_t* ctx, uint32_t* cigar, int64_t cigar_cap, int64_t* cigar_off, uint8_t* has_ins,
               uint32_t* status);

/* Stage outputs of one query of the last hg_run_staged (the staged batch
 * must fit one sub-batch): its anchors as the chain stage saw them - the
 * collect_anchors output (src/seed/minimizer.cpp:220-356) in chainAnchors'
 * sorted order (src/seed/anchor.cpp:343-349), as center / query positions -
 * the chain DP arrays f and p over those anchors (p[i] = -1: no
 * predecessor) and the best chain (chain_end: its last anchor, -1 if none;
 * n_chain: its length after the min_score / min_cnt checks, 0 = rejected).
 * *n_anchors is always set; arrays are written when cap >= *n_anchors.
 * A test and debugging view of the batch kernels; no reference counterpart. */
int hg_fetch_chain(hg_ctx_t* ctx, int64_t query, uint32_t* pos_ref, uint32_t* pos_qry, int32_t* f, int32_t* p,
                   int64_t cap, int64_t* n_anchors, int64_t* chain_end, int64_t* n_chain);

/* ---- files: query FASTA in, aligned FASTA out ---------------------------
 * The align-to-center run of the reference CLI with --keep-length
 * (halign4 -c center.fa -i queries.fa --keep-length), streamed: one record
 * in center_fasta is the center (k, w: --kmer-size, --kmer-window); several
 * records (of one length) are multi-reference mode, each query aligned to
 * its best reference (hg_refset_align; sketch size 2000, seed 42, as the
 * CLI), the output being the CLI's when its MSA tool returns the references
 * unchanged.  Queries are read in chunks of chunk_queries records
 * (KseqReader::next, src/utils/seq_io.cpp:134-155), aligned with rows on the
 * GPU while the next chunk is read and the previous one written, and written
 * in the reference's order (src/align/ref_aligner.cpp:676-740): the center
 * record(s) through clean_table, then every row with an insertion, then the
 * others, each group in input order, one line per row.  *n_aligned (may be
 * NULL) gets the query count.  Errors as hg_align_batch's
 * (HG_ERR_LENGTH_MISMATCH where the reference throws); HG_ERR_ARG for
 * references of different lengths. */
int hg_align_fasta(const char* center_fasta, const char* queries_fasta, const char* out_fasta, int k, int w,
                   int64_t chunk_queries, int64_t* n_aligned);

/* Center construction without a center file (the CLI run without -c):
 * preprocessInputFasta's Top-K of the queries (src/utils/preprocess.cpp:
 * 111-150; TopKLongestSelector, src/consensus/selector.cpp: the cons_n
 * longest records, ties to the earlier one), each through clean_table, then
 * generateConsensusSequence over them (src/consensus/consensus.cpp:611-703,
 * at most cons_n records, batch size 4096) on the device.  The reference
 * runs its external MSA over the selection first; here the selected records
 * must already share one length (HG_ERR_ARG otherwise), which is the CLI's
 * result when its MSA command returns them unchanged.  *len gets the center
 * length; HG_ERR_CAPACITY when cap is smaller (out may then be NULL). */
int hg_build_center(const char* queries_fasta, int64_t cons_n, char* out, int64_t cap, int64_t* len);

/* halign4 -i queries.fa --keep-length --cons-n cons_n (no -c), streamed:
 * hg_build_center, then hg_align_fasta's run against that center, written
 * as the record ">consensus" first. */
int hg_align_fasta_consensus(const char* queries_fasta, const char* out_fasta, int k, int w, int64_t cons_n,
                             int64_t chunk_queries, int64_t* n_aligned);

/* ---- serving loop (continuous batching) ---------------------------------
 * A request loop around one resident index: requests (one ASCII query each,
 * copied at submission into a ring of pinned host memory of 2 x contexts x
 * slot_bases bytes, at most 8 GiB or 2 x slot_bases if that is more) wait
 * in a FIFO; a submitting thread fills every free context with the oldest
 * waiting requests (up to slot_queries and slot_bases per micro-batch) and
 * enqueues it asynchronously - its bytes upload straight from the ring and
 * the device packs them (hg_align_ascii's packing) - and a collecting
 * thread polls the busy contexts, files each finished request's CIGAR and
 * status for hg_serve_result and frees its ring bytes.  Requests that
 * arrive while others run join as contexts free up; micro-batches of
 * different contexts overlap on the GPU.  The contexts' device arenas are allocated at
 * creation; n_slots is reduced to what budget_bytes of device memory holds
 * (at least one context must fit).  Submission and result calls are
 * thread-safe.  HAlign-4 has no serving mode: this is the request-level use
 * of the align-to-center path (RefAligner::globalAlign per request). */
typedef struct hg_server hg_server_t;
int hg_serve_create(hg_index_t* ix, int n_slots, int64_t slot_queries, int64_t slot_bases, int64_t budget_bytes,
                    hg_server_t** out);
/* Stops the loop after the requests in flight finish, frees everything. */
void hg_serve_destroy(hg_server_t* s);
/* Queues one request; returns its id (0, 1, 2, ... in submission order) or a
 * negative HG_ERR_* (HG_ERR_CAPACITY: longer than slot_bases).  Waits while
 * the request ring is full.  A micro-batch whose bytes other than A/C/G/T
 * form more runs than its context holds (slot_bases / 16 + 4096) fails the
 * loop with HG_ERR_CAPACITY. */
int64_t hg_serve_submit(hg_server_t* s, const char* seq, int64_t len);
/* Queues a burst of n requests (concatenated in seqs, request i at
 * [offsets[i], offsets[i+1])) with one time stamp, in chunks that join the
 * FIFO as they are copied (waiting while the ring is full); returns the
 * first id (the burst's ids are consecutive) or a negative HG_ERR_*
 * (nothing queued on a bad argument; on a loop failure in mid-burst the
 * queued part fails with the loop). */
int64_t hg_serve_submit_many(hg_server_t* s, const char* seqs, const int64_t* offsets, int64_t n);
/* Up to max_n finished requests at once, waiting up to timeout_ms for the
 * first (< 0: no limit): ids[j], status[j], latency_ms[j] (optional) and the
 * CIGARs concatenated in cigar with cigar_off[0..m]; stops before a CIGAR
 * that would pass cigar_cap.  Returns m (0 on time-out) or a negative
 * HG_ERR_* (HG_ERR_CAPACITY when not even the first CIGAR fits). */
int64_t hg_serve_results(hg_server_t* s, int64_t max_n, int64_t* ids, uint32_t* status, double* latency_ms,
                         uint32_t* cigar, int64_t cigar_cap, int64_t* cigar_off, int timeout_ms);
/* The next finished request, waiting up to timeout_ms (< 0: no limit):
 * returns 1 with *id, *status (HG_ST_* bits), *latency_ms (submission to
 * result) and its CIGAR (*n_cigar ops; up to cap written, the rest dropped
 * when cap is smaller), 0 on time-out, or a negative HG_ERR_*. */
int hg_serve_result(hg_server_t* s, int64_t* id, uint32_t* status, double* latency_ms, uint32_t* cigar, int64_t cap,
                    int64_t* n_cigar, int timeout_ms);
/* Statistics since creation (or the last reset): out[0] p50 ms, [1] p99 ms,
 * [2] mean ms, [3] max ms, [4] finished requests, [5] bases, [6] micro-
 * batches, [7] seconds from the first submission to the last result,
 * [8] contexts, [9] device bytes of their arenas. */
int hg_serve_stats(hg_server_t* s, double* out, int n, int reset);
/* Per-column counters summed over the server's contexts (hg_counters). */
int hg_serve_counters(hg_server_t* s, uint32_t* counts7, uint32_t* ins, int reset);

/* Consensus counters: counts7 = L x {A,C,G,T,U,N,-} (consensus::SiteCount,
 * include/consensus.h:78-99), ins = L+1 insertion events (slot c: I before
 * center column c).  reset != 0 clears them after reading. */
int hg_counters(hg_ctx_t* ctx, uint32_t* counts7, uint32_t* ins, int reset);

/* ---- single-call entry points (the C++ drop-in shim uses these) -------- */

/* minimizer::extractMinimizer (include/seed.h:283-286); writes MinimizerHit
 * words (x = hash56<<8|span, y = strand<<63|rid<<32|pos).  Returns the hit
 * count (>= 0) or a negative HG_ERR_* value; -HG_ERR_CAPACITY means cap is
 * smaller than the count, which is then in *needed. */
int64_t hg_extract_minimizer(const char* seq, int64_t len, int k, int w, int non_canonical, uint64_t* xs,
                             uint64_t* ys, int64_t cap, int64_t* needed);

/* ksw_extz2_sse (include/ksw2.h:64-65): the full m x m matrix with
 * KSW_EZ_GENERIC_SC, otherwise match (mat[0]) / mismatch (mat[1]) scoring
 * with symbol m-1 as the wildcard, as the reference's SSE2 kernel.
 * ez_out: {max, zdropped, max_q, max_t, mqe, mqe_t, mte, mte_q, score,
 * reach_end}; returns the CIGAR length or a negative HG_ERR_*.  Single calls
 * (this one, hg_extract_minimizer, hg_collect_anchors, hg_chain_anchors,
 * hg_project_row, hg_count_rows) run on a per-thread, per-device stream and
 * grow-only scratch, so repeated calls allocate nothing once the scratch has
 * grown to the largest call; each host thread may call them concurrently. */
int64_t hg_ksw_extz2(int qlen, const uint8_t* query, int tlen, const uint8_t* target, int8_t m, const int8_t* mat,
                     int8_t q, int8_t e, int w, int zdrop, int end_bonus, int flag, int32_t* ez_out, uint32_t* cigar,
                     int64_t cap);

/* Allocation-free ksw_extz2 (no counterpart in the reference: the reference's
 * ksw_extz2_sse allocates its work arrays with malloc on every call).
 * For callers that cannot allocate device memory: code whose device memory
 * belongs to a pool or caching allocator that must account for every byte,
 * and latency-sensitive loops that cannot take the device-wide
 * synchronisation of cudaFree.  Inputs and outputs are DEVICE pointers owned
 * by the caller: d_query/d_target (codes < m), d_mat (m*m), d_ez (11 int32:
 * the ez fields of hg_ksw_extz2 followed by the CIGAR length) and d_cigar
 * (cap entries; a length above cap means the CIGAR did not fit, and nothing
 * is written past cap).  The sequences live on the device, so the host cannot
 * check them: the kernel does, and a code >= m makes the call compute nothing
 * and write -1 as the CIGAR length (d_ez[10]).  The call
 * only enqueues one kernel on `stream` (NULL = default stream) and allocates
 * nothing; the DP scratch is one HG_NOALLOC_SCRATCH_BYTES array per GPU,
 * held until the process exits.  A call whose scratch need exceeds it returns
 * HG_ERR_CAPACITY before launching (err, when non-NULL, gets the message).
 * All calls on a GPU share that array: calls that may overlap on the GPU
 * race and must be serialised.  The first call on a device looks up the
 * array's address with that device current; make it before any stream
 * capture.  That address is kept per device ordinal for the primary context:
 * it does not carry over to another driver context or past cudaDeviceReset. */
#define HG_NOALLOC_SCRATCH_BYTES (1u << 20)
int hg_ksw_extz2_noalloc(int qlen, const uint8_t* d_query, int tlen, const uint8_t* d_target, int8_t m,
                         const int8_t* d_mat, int8_t q, int8_t e, int w, int zdrop, int end_bonus, int flag,
                         int32_t* d_ez, uint32_t* d_cigar, int64_t cap, void* stream, char* err, int64_t err_cap);

/* anchor::Anchor (include/anchor.h:39-50) as a C record (32 bytes; is_rev
 * is 0 or 1). */
typedef struct {
    uint64_t hash;
    uint32_t rid_ref, pos_ref, rid_qry, pos_qry, span;
    uint32_t is_rev;
} hg_anchor_t;

/* Reference-side half of minimizer::collect_anchors (src/seed/minimizer.cpp:
 * 238-272) for any hit list (several sequences, both strands): the hits
 * sorted by (hash, rid, pos, strand), grouped by hash, the -f/-U occurrence
 * threshold from params (f_top_frac, u_floor, u_ceil; NULL = defaults) and a
 * hash table, built once and kept on the current device.  The reference
 * rebuilds this on every call; a caller keeps the handle while its reference
 * hits stay the same.  Hits of equal sort key keep their input order (the
 * reference's std::sort leaves that order unspecified). */
typedef struct hg_hits hg_hits_t;
int hg_hits_create(const uint64_t* ref_x, const uint64_t* ref_y, int64_t n, const hg_params_t* params,
                   hg_hits_t** out);
void hg_hits_destroy(hg_hits_t* h);

/* anchor::compute_ref_occ_threshold and compute_occ_cutoff_top_frac
 * (src/seed/anchor.cpp:73-117) over n per-hash occurrence counts with
 * params' f_top_frac, u_floor, u_ceil (NULL = defaults): returns the
 * threshold; *cutoff_top_frac (may be NULL) gets the -f cutoff alone
 * (UINT64_MAX when nothing is skipped).  Host arithmetic of the index
 * set-up; it never fails. */
uint64_t hg_occ_threshold(const uint64_t* occs, int64_t n, const hg_params_t* params, uint64_t* cutoff_top_frac);

/* minimizer::collect_anchors (src/seed/minimizer.cpp:220-356) against a
 * hits handle, on the GPU: the --q-occ-frac and -e filters (params'
 * q_occ_frac, sample_every_bp; NULL = defaults), then one anchor per kept
 * query hit and reference occurrence, in the reference's order (query-hit
 * order, occurrences in sorted order).  Returns the anchor count, or a
 * negative HG_ERR_*; -HG_ERR_CAPACITY when cap is below the count, which is
 * then in *needed. */
int64_t hg_collect_anchors(const hg_hits_t* h, const uint64_t* qry_x, const uint64_t* qry_y, int64_t n_qry,
                           const hg_params_t* params, hg_anchor_t* out, int64_t cap, int64_t* needed);

/* anchor::chainAnchors (src/seed/anchor.cpp:332-461) with chainScoreSimple
 * (:254-301), on the GPU: anchors[] is sorted in place by (rid_ref, is_rev,
 * pos_ref, pos_qry) as the reference sorts it (equal keys keep their input
 * order), the DP runs with params' chain fields (NULL = defaults) and chain[]
 * gets the best chain as ascending indices into the sorted anchors.  Returns
 * the chain length (0: no chain passes min_score / min_cnt) or a negative
 * HG_ERR_*; -HG_ERR_CAPACITY when cap is below the length.  f and p (each n
 * entries, may be NULL) get the DP arrays of the sorted anchors.  rid_ref
 * must be below 2^31 (MinimizerHit's rid field). */
int64_t hg_chain_anchors(hg_anchor_t* anchors, int64_t n, const hg_params_t* params, int64_t* chain, int64_t cap,
                         int32_t* f, int64_t* p);

/* cigar::delQueryToRefByCigar (pad == 0; src/align/cigar.cpp:212-299) and
 * cigar::padQueryToRefByCigar (pad != 0; :150-209) on the GPU: the query
 * projected onto the reference by its CIGAR.  An empty CIGAR leaves the query
 * as it is.  Returns the row length or a negative HG_ERR_*: HG_ERR_ARG when
 * the CIGAR does not consume exactly qlen query bases (the reference asserts)
 * or holds an op code above 8 (intToCigar throws), HG_ERR_CAPACITY when cap
 * is below the row length. */
int64_t hg_project_row(const char* qry, int64_t qlen, const uint32_t* cigar, int64_t n_cigar, int pad, char* out,
                       int64_t cap);

/* SiteCount accumulation (consensus::processBatchParallelWithLocals,
 * src/consensus/consensus.cpp:304-411) of n_rows aligned rows of L columns
 * (row i at rows + i * row_stride) on the GPU, with k_base_map's classes
 * (include/consensus.h:126-145).  counts7 is L x {A,C,G,T,U,N,-} uint32;
 * accumulate != 0 adds to its values, else it is overwritten. */
int hg_count_rows(const char* rows, int64_t n_rows, int64_t L, int64_t row_stride, uint32_t* counts7,
                  int accumulate);

/* align::globalAlignKSW2 (src/align/align.cpp:22-65); flag < 0 selects the
 * default KSW_EZ_GENERIC_SC|KSW_EZ_RIGHT. */
int64_t hg_global_align_ksw2(const char* ref, int64_t rlen, const char* qry, int64_t qlen, int flag, uint32_t* cigar,
                             int64_t cap);

/* align::extendAlignKSW2 (src/align/align.cpp:68-107): DNA5 codes, the
 * default matrix and gaps, match/mismatch scoring with N the wildcard (no
 * KSW_EZ_GENERIC_SC), KSW_EZ_EXTZ_ONLY | RIGHT | APPROX_DROP, end bonus 50,
 * the caller's z-drop, auto_band.  Returns the CIGAR length (0 for an empty
 * sequence) or a negative HG_ERR_*. */
int64_t hg_extend_align_ksw2(const char* ref, int64_t rlen, const char* qry, int64_t qlen, int zdrop,
                             uint32_t* cigar, int64_t cap);

/* align::globalAlignMM2 (src/align/align.cpp:189-305, include/align.h) with
 * the caller's anchors (anchor::Anchor pos_ref / pos_qry, include/anchor.h:
 * 39-50) against the index's center: anchors of one center on the forward
 * strand with span = the index's k, as collect_anchors makes them on the
 * align-to-center path.  The anchors are sorted as chainAnchors sorts them
 * (globalAlignMM2 takes them const and chains a copy; the input arrays are
 * left untouched).  Returns the CIGAR length, or -status.  *status gets the
 * HG_ST_* bits (partial CIGAR / length mismatch as in hg_align_query). */
int64_t hg_global_align_mm2(hg_index_t* ix, const char* qry, int64_t qlen, const uint32_t* anchor_ref,
                            const uint32_t* anchor_qry, int64_t n_anchors, uint32_t* cigar, int64_t cap,
                            uint32_t* status);

/* RefAligner::globalAlign for one query against the index's center
 * (src/align/ref_aligner.cpp:91-125): the plain single-query path. */
int64_t hg_align_query(hg_index_t* ix, const char* qry, int64_t qlen, uint32_t* cigar, int64_t cap,
                       uint32_t* status);

/* ---- multi-reference mode ------------------------------------------------
 * Replaces RefAligner with several records in the reference FASTA
 * (src/align/ref_aligner.cpp:21-70 and 212-283): MinHash sketches
 * (mash::sketchFromSequence, src/mash/mash.cpp:32-117; non-canonical
 * k-mers, the path's setting), the first reference of largest jaccard
 * (mash::jaccard, :120-164; selection loop :232-241), alignment to it, and
 * the consensus re-check without --keep-length (:273-282). */

/* Largest sketch_size one CTA holds in shared memory (the reference's default
 * is 2000). */
#define HG_SKETCH_MAX 8192

/* mash::sketchFromSequence for every query of a packed batch (hg_pack
 * format): the sketch_size smallest distinct getHash2bit hashes (XXH3-64,
 * src/mash/hash.cpp) of the valid k-mers, ascending, into
 * hashes[i * stride ...], their number into counts[i].  k outside 1..32 or
 * a query shorter than k gives an empty sketch, as in the reference (k = 32
 * reproduces its mask of 0: every code is 0).  noncanonical = 0 hashes
 * min(forward, reverse-complement) codes. */
int hg_sketch_batch(const uint8_t* packed, const int64_t* poff, const int32_t* qlen, const int32_t* exc,
                    const int64_t* exc_off, int64_t n, int k, int sketch_size, int noncanonical, int seed,
                    uint64_t* hashes, int64_t stride, int32_t* counts);

/* Resident reference set: per reference an index (hg_index_create; one
 * reference aligns to its consensus, one of several to itself, as RefAligner
 * does), its sketch, and one batch context created on first use
 * (max_queries / max_bases as hg_ctx_create).  With references of one
 * length the consensus of the re-check path is built as the reference
 * builds it from the references' alignment when its MSA tool returns them
 * unchanged (generateConsensusSequence, batch size 4096); otherwise give it
 * with hg_refset_set_consensus.  seed is RefAligner's random_seed (42). */
typedef struct hg_refset hg_refset_t;
int hg_refset_create(const char* const* refs, const int64_t* lens, int n_refs, int k, int w, int sketch_size,
                     int seed, const hg_params_t* params, int64_t max_queries, int64_t max_bases, hg_refset_t** out);
void hg_refset_destroy(hg_refset_t* rs);
int hg_refset_info(const hg_refset_t* rs, int* n_refs, int64_t* max_len, int64_t* consensus_len);
int hg_refset_sketch(const hg_refset_t* rs, int ref, uint64_t* hashes, int64_t cap, int64_t* n);
int hg_refset_consensus(const hg_refset_t* rs, char* out, int64_t cap, int64_t* len);
int hg_refset_set_consensus(hg_refset_t* rs, const char* seq, int64_t len);

/* Best reference of every query of a packed batch: best[i] the first
 * reference of largest jaccard, jaccard[i] its value (one device launch). */
int hg_refset_select(hg_refset_t* rs, const uint8_t* packed, const int64_t* poff, const int32_t* qlen,
                     const int32_t* exc, const int64_t* exc_off, int64_t n, int32_t* best, double* jaccard);

/* Device time of the last hg_refset_select launch (sketch + selection
 * kernel, CUDA events on the set's stream), in milliseconds. */
int hg_refset_last_ms(const hg_refset_t* rs, float* select_ms);

/* alignOneQueryToRef for a batch.  keep_length != 0: every query aligned to
 * its best reference (rows have that reference's length; row_stride >= the
 * longest reference); keep_length == 0: aligned to the consensus (the
 * reference's discarded first alignment is not run).  One reference: aligned
 * to it either way.  best / jaccard (optional) get the selection; the other
 * outputs are hg_align_batch's, in input order. */
int hg_refset_align(hg_refset_t* rs, const uint8_t* packed, const int64_t* poff, const int32_t* qlen,
                    const int32_t* exc, const int64_t* exc_off, int64_t n, int keep_length, int32_t* best,
                    double* jaccard, uint32_t* cigar, int64_t cigar_cap, int64_t* cigar_off, uint8_t* has_ins,
                    uint8_t* rows, int64_t row_stride, uint32_t* status);

#ifdef __cplusplus
}
#endif
#endif
