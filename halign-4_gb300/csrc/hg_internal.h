// hg_internal.h - host-side helpers shared by the runtime translation units
// (hg_runtime.cu: index, contexts, batch path; hg_single.cu: single-call
// entry points).  Not part of the public C ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/halign_gb300.h"

namespace hg {

// Error reporting: the calling thread's message for hg_last_error().
int set_error(int code, const std::string& msg);
inline int cuda_error(cudaError_t e, const char* where)
{
    return set_error(HG_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define HG_CUDA(call)                                             \
    do {                                                          \
        cudaError_t e_ = (call);                                  \
        if (e_ != cudaSuccess) return hg::cuda_error(e_, #call);  \
    } while (0)

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { free(); }
    cudaError_t alloc(size_t count)
    {
        free();
        n = count;
        return count ? cudaMalloc(&p, sizeof(T) * count) : cudaSuccess;
    }
    void free()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

// compute_ref_occ_threshold (src/seed/anchor.cpp:73-117): max(u_floor,
// min(u_ceil, the n_skip-th largest occurrence)), n_skip = floor(f * #distinct).
uint64_t occ_threshold(std::vector<uint64_t> occs, const hg_params_t& p);

// log2f(i) for i in [0, n) as the chain penalty reads it (mg_log2,
// src/seed/anchor.cpp:227-230): the float nearest to log2(i), 0 below 1.
std::vector<float> log2_table(int n);

// Per-thread, per-device workspace of the single-call entry points: one
// non-blocking stream, grow-only device buffers by slot and a grow-only
// pinned staging buffer.  Calls reuse it, so a single call allocates only
// when it needs more than any earlier call on this thread did; the buffers
// are released when the thread exits.
struct Workspace {
    static constexpr int kSlots = 16;
    int device = -1;
    cudaStream_t st = nullptr;
    void* dptr[kSlots] = {};
    size_t dcap[kSlots] = {};
    void* hptr = nullptr;
    size_t hcap = 0;
    ~Workspace();
    // device buffer `slot` with at least `bytes` bytes (256-byte aligned)
    cudaError_t dev(int slot, size_t bytes, void** out);
    // pinned host staging with at least `bytes` bytes
    cudaError_t host(size_t bytes, void** out);
};
// The calling thread's workspace for the current device (created on first use).
int workspace(Workspace** out);

// hg_index_create with the DP center chosen: dp_consensus aligns against
// the consensus of the single record (RefAligner with one reference aligns
// to consensus_seq, src/align/ref_aligner.cpp:242-245), otherwise against
// the record as given (one of several references, :232-240).
int index_create(const char* center, int64_t len, int k, int w, const hg_params_t* params, bool dp_consensus,
                 hg_index_t** out);

// generateConsensusSequence over aligned records of one length (at most
// `limit` of them, 0 = all; batch size 4096 with the reference's dropped
// record after each full batch): the per-column majority, on the device.
int consensus_of_rows(const std::vector<std::string>& recs, size_t limit, std::string& out);

// Length of an index's center.
int64_t index_length(const hg_index_t* ix);

// Asynchronous submission (hg_submit's form) of n ASCII queries of lengths
// lens[] whose bytes lie in pinned host memory as `runs` runs of
// consecutive queries back to back (run r: run_bytes[r] bytes at
// run_ptr[r]): the runs upload as they are and the device packs them
// (hg_align_ascii's packing).  The bytes must stay in place until the batch
// is collected.  hg_collect then returns HG_ERR_CAPACITY when the batch's
// exception runs exceeded the context's buffer; async_exc_overflow tells
// that case from a short CIGAR buffer.  prepare_pinned_ascii allocates the
// device and pinned buffers of this form up front.
int prepare_pinned_ascii(hg_ctx_t* c);
int submit_pinned_ascii(hg_ctx_t* c, const char* const* run_ptr, const int64_t* run_bytes, int runs,
                        const int64_t* lens, int64_t n);
bool async_exc_overflow(const hg_ctx_t* c);

// Minimizers of one sequence through the batch seed kernel (hg_index_create
// and hg_extract_minimizer).
int run_extract(int k, int w, int non_canonical, const char* seq, int64_t len, std::vector<uint64_t>& xs,
                std::vector<uint64_t>& ys);

}  // namespace hg
