// hg_refset.cpp - multi-reference mode of the align-to-center path.
//
// RefAligner (src/align/ref_aligner.cpp) with several records in the
// reference FASTA:
//   * the constructor (:21-70) sketches and indexes every reference and
//     builds the consensus of their alignment (generateConsensusSequence
//     over the MSA of the references, batch size 4096);
//   * alignOneQueryToRef (:212-283) sketches the query, picks the first
//     reference of largest jaccard, aligns to it (globalAlign with that
//     reference's minimizers); with --keep-length that alignment is the
//     result, otherwise the query is aligned again to the consensus and that
//     alignment is the result (the first one is discarded).
//
// Here the references' indexes and sketches stay resident; a batch is
// sketched and matched on the device in one launch (hg_sketch.cu), then
// aligned per chosen reference with the batch path (one context per
// reference, created on first use) and put back in input order.  Without
// --keep-length only the consensus alignment is run: the discarded first
// alignment is skipped, which changes no output.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/halign_gb300.h"
#include "hg_internal.h"

extern "C" {
size_t hg_sketch_smem(int sketch_size, int* cap);
cudaError_t hg_launch_sketch(const uint8_t* packed, const int64_t* poff, const int32_t* qlen, const int32_t* exc,
                             const int64_t* exc_off, int n, int k, int s, int noncanonical, int seed, uint64_t* out,
                             int64_t out_stride, int32_t* out_n, const uint64_t* ref_h, const int64_t* ref_off,
                             int n_refs, const ulonglong2* ref_tab, uint32_t ref_tab_mask, int32_t* best,
                             double* best_j, unsigned* queue, int sms, cudaStream_t st);
}

namespace {

using hg::DevBuf;

size_t padded_bytes(int64_t len) { return (size_t)(((len + 3) / 4 + 15) / 16 * 16); }

int sm_count()
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

// A packed batch on the device (grow-only buffers on one stream).
struct DevBatch {
    DevBuf<uint8_t> packed;
    DevBuf<int64_t> poff, eoff;
    DevBuf<int32_t> qlen, exc;
    std::vector<uint8_t> gather;
    std::vector<int64_t> spoff, seoff;

    template <typename T>
    static cudaError_t fit(DevBuf<T>& b, size_t n)
    {
        return n <= b.n && b.p ? cudaSuccess : b.alloc(std::max<size_t>(n, 1) + n / 2);
    }

    // Upload queries [0, n) of a caller batch (hg_pack format, query blocks
    // anywhere in `packed`) as one contiguous block.
    int upload(const uint8_t* packed_h, const int64_t* poff_h, const int32_t* qlen_h, const int32_t* exc_h,
               const int64_t* exc_off_h, int64_t n, cudaStream_t st)
    {
        spoff.resize((size_t)n), seoff.resize((size_t)n + 1);
        int64_t pb = 0;
        bool contiguous = true;
        for (int64_t i = 0; i < n; ++i) {
            spoff[i] = pb;
            contiguous = contiguous && poff_h[i] == poff_h[0] + pb;
            pb += (int64_t)padded_bytes(qlen_h[i]);
        }
        for (int64_t i = 0; i <= n; ++i) seoff[i] = exc_off_h[i] - exc_off_h[0];
        const int64_t ne = seoff[n];
        cudaError_t e;
        if ((e = fit(packed, (size_t)pb + 16)) || (e = fit(poff, (size_t)n)) || (e = fit(eoff, (size_t)n + 1)) ||
            (e = fit(qlen, (size_t)n)) || (e = fit(exc, (size_t)ne * 3)))
            return hg::cuda_error(e, "multi-reference batch buffers");
        const uint8_t* src = packed_h + (n ? poff_h[0] : 0);
        if (!contiguous) {
            gather.resize((size_t)pb);
            for (int64_t i = 0; i < n; ++i)
                std::memcpy(gather.data() + spoff[i], packed_h + poff_h[i], padded_bytes(qlen_h[i]));
            src = gather.data();
        }
        if (pb) HG_CUDA(cudaMemcpyAsync(packed.p, src, (size_t)pb, cudaMemcpyHostToDevice, st));
        if (n) {
            HG_CUDA(cudaMemcpyAsync(poff.p, spoff.data(), 8 * (size_t)n, cudaMemcpyHostToDevice, st));
            HG_CUDA(cudaMemcpyAsync(qlen.p, qlen_h, 4 * (size_t)n, cudaMemcpyHostToDevice, st));
        }
        HG_CUDA(cudaMemcpyAsync(eoff.p, seoff.data(), 8 * ((size_t)n + 1), cudaMemcpyHostToDevice, st));
        if (ne) HG_CUDA(cudaMemcpyAsync(exc.p, exc_h + 3 * exc_off_h[0], 12 * (size_t)ne, cudaMemcpyHostToDevice, st));
        return HG_OK;
    }
};

// Sketches of a host batch; out is n x stride (stride >= s), counts n.
int sketch_batch(DevBatch& B, DevBuf<uint64_t>& dout, DevBuf<int32_t>& dn, DevBuf<unsigned>& queue,
                 const uint8_t* packed, const int64_t* poff, const int32_t* qlen, const int32_t* exc,
                 const int64_t* exc_off, int64_t n, int k, int s, int noncanonical, int seed, uint64_t* out,
                 int64_t stride, int32_t* counts, cudaStream_t st)
{
    int r = B.upload(packed, poff, qlen, exc, exc_off, n, st);
    if (r) return r;
    const size_t per = (size_t)std::max(s, 1);
    cudaError_t e;
    if ((e = DevBatch::fit(dout, (size_t)n * per)) || (e = DevBatch::fit(dn, (size_t)n)) ||
        (e = DevBatch::fit(queue, 1)))
        return hg::cuda_error(e, "hg_sketch_batch: buffers");
    HG_CUDA(hg_launch_sketch(B.packed.p, B.poff.p, B.qlen.p, B.exc.p, B.eoff.p, (int)n, k, s, noncanonical, seed,
                             dout.p, (int64_t)per, dn.p, nullptr, nullptr, 0, nullptr, 0u, nullptr, nullptr, queue.p,
                             sm_count(), st));
    if (n) {
        HG_CUDA(cudaMemcpyAsync(counts, dn.p, 4 * (size_t)n, cudaMemcpyDeviceToHost, st));
        if (s > 0)
            HG_CUDA(cudaMemcpy2DAsync(out, 8 * (size_t)stride, dout.p, 8 * per, 8 * (size_t)s, (size_t)n,
                                      cudaMemcpyDeviceToHost, st));
    }
    HG_CUDA(cudaStreamSynchronize(st));
    return HG_OK;
}

bool sketch_args_ok(int64_t n, int sketch_size, std::string* why)
{
    if (n < 0 || n > INT32_MAX) return *why = "query count out of range", false;
    if (sketch_size > HG_SKETCH_MAX) return *why = "sketch_size above HG_SKETCH_MAX", false;
    return true;
}

// pickConsensusChar (src/consensus/consensus.cpp:18-35) over {A,C,G,T,U,N,-}
char pick_consensus(const uint32_t* c)
{
    uint32_t best = c[0];
    char ch = 'A';
    if (c[1] > best) best = c[1], ch = 'C';
    if (c[2] > best) best = c[2], ch = 'G';
    if (c[3] > best) best = c[3], ch = 'T';
    if (c[4] > best) best = c[4], ch = 'U';
    return ch;
}

}  // namespace

struct hg_refset {
    int device = 0;
    int k = 15, w = 10, s = 2000, seed = 42;
    hg_params_t prm{};
    int64_t max_q = 0, max_b = 0;
    std::vector<std::string> refs;
    std::vector<hg_index_t*> ix;
    std::vector<hg_ctx_t*> ctx;
    std::vector<std::vector<uint64_t>> sk;
    std::string consensus;
    hg_index_t* cons_ix = nullptr;
    hg_ctx_t* cons_ctx = nullptr;
    cudaStream_t st = nullptr;
    DevBuf<uint64_t> ref_h, sk_out;
    DevBuf<int64_t> ref_off;
    DevBuf<ulonglong2> ref_tab;  // up to 64 references: hash -> mask of the references holding it
    uint32_t ref_tab_mask = 0;
    DevBuf<int32_t> best, sk_n;
    DevBuf<double> best_j;
    DevBuf<unsigned> queue;
    DevBatch batch;
    cudaEvent_t ev[2] = {nullptr, nullptr};  // around the last selection launch
    float last_ms = 0.0f;
    // grow-only pinned staging of one reference's group: packed inputs and rows
    struct Pinned {
        uint8_t* p = nullptr;
        size_t n = 0;
        cudaError_t fit(size_t want)
        {
            if (want <= n) return cudaSuccess;
            if (p) cudaFreeHost(p);
            p = nullptr, n = 0;
            const cudaError_t e = cudaHostAlloc(reinterpret_cast<void**>(&p), want, cudaHostAllocDefault);
            if (e == cudaSuccess) n = want;
            return e;
        }
        ~Pinned()
        {
            if (p) cudaFreeHost(p);
        }
    } h_packed, h_rows;
    ~hg_refset()
    {
        cudaSetDevice(device);
        if (st) cudaStreamSynchronize(st);
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
        for (auto* c : ctx) hg_ctx_destroy(c);
        for (auto* x : ix) hg_index_destroy(x);
        hg_ctx_destroy(cons_ctx);
        hg_index_destroy(cons_ix);
        if (st) cudaStreamDestroy(st);
    }
};

namespace {

int fail(int code, const std::string& msg) { return hg::set_error(code, msg); }

int ctx_of(hg_refset_t* R, int r, hg_ctx_t** out)
{
    if (!R->ctx[r]) {
        const int rc = hg_ctx_create(R->ix[r], R->max_q, R->max_b, &R->ctx[r]);
        if (rc) return rc;
    }
    *out = R->ctx[r];
    return HG_OK;
}

int cons_ctx_of(hg_refset_t* R, hg_ctx_t** out)
{
    if (R->consensus.empty())
        return fail(HG_ERR_ARG, "multi-reference: no consensus (references of different lengths: "
                                "give one with hg_refset_set_consensus)");
    if (!R->cons_ix) {
        const int rc = hg::index_create(R->consensus.data(), (int64_t)R->consensus.size(), R->k, R->w, &R->prm,
                                        true, &R->cons_ix);
        if (rc) return rc;
    }
    if (!R->cons_ctx) {
        const int rc = hg_ctx_create(R->cons_ix, R->max_q, R->max_b, &R->cons_ctx);
        if (rc) return rc;
    }
    *out = R->cons_ctx;
    return HG_OK;
}

// The consensus of the references when they share one length (their
// alignment by an MSA command that returns them unchanged); otherwise none.
int refs_consensus(const std::vector<std::string>& refs, std::string& out)
{
    for (const auto& r : refs)
        if (r.size() != refs[0].size()) return HG_OK;
    return hg::consensus_of_rows(refs, 0, out);
}

}  // namespace

// generateConsensusSequence (src/consensus/consensus.cpp:611-703) over
// aligned records of one length, batch size 4096: SiteCount per column
// (hg_count_rows on the device) over at most `limit` records (0: all), the
// record read after each full batch dropped as the reference's loop does,
// pickConsensusChar per column.
int hg::consensus_of_rows(const std::vector<std::string>& recs, size_t limit, std::string& out)
{
    if (recs.empty()) return set_error(HG_ERR_ARG, "consensus: no records");
    const size_t L = recs[0].size();
    const size_t batch = 4096;
    std::vector<uint32_t> counts(7 * L, 0);
    std::string rows;
    size_t i = 0, num = 0;
    while (i < recs.size() && (limit == 0 || num < limit)) {
        rows.clear();
        size_t m = 0;
        for (; m < batch && i < recs.size() && (limit == 0 || num < limit); ++m, ++i, ++num) rows += recs[i];
        const int rc = hg_count_rows(rows.data(), (int64_t)m, (int64_t)L, (int64_t)L, counts.data(), 1);
        if (rc) return rc;
        if (m == batch && i < recs.size()) ++i;  // read, then dropped
    }
    out.resize(L);
    for (size_t c = 0; c < L; ++c) out[c] = pick_consensus(&counts[7 * c]);
    return HG_OK;
}

extern "C" int hg_sketch_batch(const uint8_t* packed, const int64_t* poff, const int32_t* qlen, const int32_t* exc,
                               const int64_t* exc_off, int64_t n, int k, int sketch_size, int noncanonical, int seed,
                               uint64_t* hashes, int64_t stride, int32_t* counts)
{
    std::string why;
    if (!sketch_args_ok(n, sketch_size, &why)) return fail(HG_ERR_ARG, "hg_sketch_batch: " + why);
    if (n && (!packed || !poff || !qlen || !exc_off || !counts || (sketch_size > 0 && (!hashes || stride < sketch_size))))
        return fail(HG_ERR_ARG, "hg_sketch_batch: bad arguments");
    if (hg_device_count() <= 0) return fail(HG_ERR_CUDA, "hg_sketch_batch: no CUDA device");
    if (n == 0) return HG_OK;
    hg::Workspace* ws = nullptr;
    int r = hg::workspace(&ws);
    if (r) return r;
    // this entry point's grow-only device buffers, per thread and device
    // (freed at thread exit; cudaFree takes another device's pointer)
    struct Bufs {
        DevBatch B;
        DevBuf<uint64_t> out;
        DevBuf<int32_t> n;
        DevBuf<unsigned> queue;
    };
    thread_local std::map<int, std::unique_ptr<Bufs>> per_device;
    auto& slot = per_device[ws->device];
    if (!slot) slot.reset(new Bufs());
    return sketch_batch(slot->B, slot->out, slot->n, slot->queue, packed, poff, qlen, exc, exc_off, n, k,
                        std::max(sketch_size, 0), noncanonical, seed, hashes, stride, counts, ws->st);
}

extern "C" int hg_refset_create(const char* const* refs, const int64_t* lens, int n_refs, int k, int w,
                                int sketch_size, int seed, const hg_params_t* params, int64_t max_queries,
                                int64_t max_bases, hg_refset_t** out)
{
    if (!out || !refs || !lens || n_refs <= 0 || max_queries <= 0 || max_bases <= 0)
        return fail(HG_ERR_ARG, "hg_refset_create: bad arguments");
    if (sketch_size <= 0 || sketch_size > HG_SKETCH_MAX)
        return fail(HG_ERR_ARG, "hg_refset_create: sketch_size must be in 1..HG_SKETCH_MAX");
    for (int r = 0; r < n_refs; ++r)
        if (!refs[r] || lens[r] <= 0) return fail(HG_ERR_ARG, "hg_refset_create: empty reference " + std::to_string(r));
    if (hg_device_count() <= 0) return fail(HG_ERR_CUDA, "hg_refset_create: no CUDA device");
    auto* R = new hg_refset();
    cudaGetDevice(&R->device);
    R->k = k, R->w = w, R->s = sketch_size, R->seed = seed;
    if (params) R->prm = *params;
    else hg_default_params(&R->prm);
    R->max_q = max_queries, R->max_b = max_bases;
    cudaError_t e = cudaStreamCreateWithFlags(&R->st, cudaStreamNonBlocking);
    if (!e) e = cudaEventCreate(&R->ev[0]);
    if (!e) e = cudaEventCreate(&R->ev[1]);
    if (e) {
        delete R;
        return hg::cuda_error(e, "hg_refset_create: stream");
    }
    int rc = HG_OK;
    for (int r = 0; r < n_refs && !rc; ++r) {
        R->refs.emplace_back(refs[r], (size_t)lens[r]);
        hg_index_t* x = nullptr;
        // one reference aligns to its consensus, one of several to itself
        rc = hg::index_create(refs[r], lens[r], k, w, &R->prm, n_refs == 1, &x);
        R->ix.push_back(x);
    }
    R->ctx.assign((size_t)n_refs, nullptr);
    // reference sketches: the same device sketch of the packed records
    if (!rc) {
        std::string cat;
        std::vector<int64_t> off{0};
        for (const auto& s : R->refs) cat += s, off.push_back((int64_t)cat.size());
        int64_t pb = 0, ne = 0;
        rc = hg_pack(cat.data(), off.data(), n_refs, nullptr, 0, nullptr, nullptr, 0, nullptr, &pb, &ne);
        std::vector<uint8_t> packed((size_t)std::max<int64_t>(pb, 16));
        std::vector<int64_t> poff((size_t)n_refs), eoff((size_t)n_refs + 1);
        std::vector<int32_t> exc((size_t)std::max<int64_t>(ne, 1) * 3), qlen((size_t)n_refs), cnt((size_t)n_refs);
        if (!rc)
            rc = hg_pack(cat.data(), off.data(), n_refs, packed.data(), (int64_t)packed.size(), poff.data(), exc.data(),
                         ne, eoff.data(), nullptr, nullptr);
        for (int r = 0; r < n_refs; ++r) qlen[r] = (int32_t)lens[r];
        std::vector<uint64_t> hs((size_t)n_refs * sketch_size);
        if (!rc)
            rc = sketch_batch(R->batch, R->sk_out, R->sk_n, R->queue, packed.data(), poff.data(), qlen.data(),
                              exc.data(), eoff.data(), n_refs, k, sketch_size, 1, seed, hs.data(), sketch_size,
                              cnt.data(), R->st);
        std::vector<uint64_t> flat;
        std::vector<int64_t> roff{0};
        for (int r = 0; r < n_refs && !rc; ++r) {
            R->sk.emplace_back(hs.begin() + (size_t)r * sketch_size, hs.begin() + (size_t)r * sketch_size + cnt[r]);
            flat.insert(flat.end(), R->sk.back().begin(), R->sk.back().end());
            roff.push_back((int64_t)flat.size());
        }
        if (!rc) {
            if ((e = R->ref_h.alloc(std::max<size_t>(flat.size(), 1))) || (e = R->ref_off.alloc(roff.size())) ||
                (flat.size() && (e = cudaMemcpy(R->ref_h.p, flat.data(), 8 * flat.size(), cudaMemcpyHostToDevice))) ||
                (e = cudaMemcpy(R->ref_off.p, roff.data(), 8 * roff.size(), cudaMemcpyHostToDevice)))
                rc = hg::cuda_error(e, "hg_refset_create: reference sketches");
        }
        // with up to 64 references, an open-addressing table hash -> mask of
        // the references whose sketch holds it (load <= 1/2, linear probing)
        if (!rc && n_refs <= 64) {
            uint32_t size = 16;
            while (size < 2 * flat.size() + 16) size <<= 1;
            std::vector<ulonglong2> tab(size, ulonglong2{0, 0});
            for (int r = 0; r < n_refs; ++r)
                for (uint64_t h : R->sk[r]) {
                    uint32_t sl = (uint32_t)h & (size - 1);
                    while (tab[sl].y != 0 && tab[sl].x != h) sl = (sl + 1) & (size - 1);
                    tab[sl].x = h, tab[sl].y |= 1ull << r;
                }
            R->ref_tab_mask = size - 1;
            if ((e = R->ref_tab.alloc(size)) ||
                (e = cudaMemcpy(R->ref_tab.p, tab.data(), sizeof(ulonglong2) * size, cudaMemcpyHostToDevice)))
                rc = hg::cuda_error(e, "hg_refset_create: reference table");
        }
    }
    if (!rc) rc = refs_consensus(R->refs, R->consensus);
    if (rc) {
        delete R;
        return rc;
    }
    *out = R;
    return HG_OK;
}

extern "C" void hg_refset_destroy(hg_refset_t* R) { delete R; }

extern "C" int hg_refset_info(const hg_refset_t* R, int* n_refs, int64_t* max_len, int64_t* consensus_len)
{
    if (!R) return fail(HG_ERR_ARG, "hg_refset_info: bad arguments");
    int64_t m = 0;
    for (const auto& s : R->refs) m = std::max(m, (int64_t)s.size());
    if (n_refs) *n_refs = (int)R->refs.size();
    if (max_len) *max_len = m;
    if (consensus_len) *consensus_len = (int64_t)R->consensus.size();
    return HG_OK;
}

extern "C" int hg_refset_sketch(const hg_refset_t* R, int r, uint64_t* hashes, int64_t cap, int64_t* n)
{
    if (!R || r < 0 || r >= (int)R->sk.size() || !n) return fail(HG_ERR_ARG, "hg_refset_sketch: bad arguments");
    const auto& v = R->sk[r];
    *n = (int64_t)v.size();
    if ((int64_t)v.size() > cap || (!hashes && !v.empty())) return fail(HG_ERR_CAPACITY, "hg_refset_sketch: cap");
    if (!v.empty()) std::memcpy(hashes, v.data(), 8 * v.size());
    return HG_OK;
}

extern "C" int hg_refset_consensus(const hg_refset_t* R, char* out, int64_t cap, int64_t* len)
{
    if (!R || !len) return fail(HG_ERR_ARG, "hg_refset_consensus: bad arguments");
    *len = (int64_t)R->consensus.size();
    if (*len > cap || (!out && *len)) return fail(HG_ERR_CAPACITY, "hg_refset_consensus: cap");
    if (*len) std::memcpy(out, R->consensus.data(), (size_t)*len);
    return HG_OK;
}

extern "C" int hg_refset_set_consensus(hg_refset_t* R, const char* seq, int64_t len)
{
    if (!R || !seq || len <= 0) return fail(HG_ERR_ARG, "hg_refset_set_consensus: bad arguments");
    cudaSetDevice(R->device);
    hg_ctx_destroy(R->cons_ctx);
    hg_index_destroy(R->cons_ix);
    R->cons_ctx = nullptr, R->cons_ix = nullptr;
    R->consensus.assign(seq, (size_t)len);
    return HG_OK;
}

extern "C" int hg_refset_select(hg_refset_t* R, const uint8_t* packed, const int64_t* poff, const int32_t* qlen,
                                const int32_t* exc, const int64_t* exc_off, int64_t n, int32_t* best, double* jaccard)
{
    if (!R || n < 0 || n > INT32_MAX || (n && (!packed || !poff || !qlen || !exc_off || !best || !jaccard)))
        return fail(HG_ERR_ARG, "hg_refset_select: bad arguments");
    if (n == 0) return HG_OK;
    cudaSetDevice(R->device);
    int r = R->batch.upload(packed, poff, qlen, exc, exc_off, n, R->st);
    if (r) return r;
    cudaError_t e;
    if ((e = DevBatch::fit(R->best, (size_t)n)) || (e = DevBatch::fit(R->best_j, (size_t)n)) ||
        (e = DevBatch::fit(R->queue, 1)))
        return hg::cuda_error(e, "hg_refset_select: buffers");
    HG_CUDA(cudaEventRecord(R->ev[0], R->st));
    HG_CUDA(hg_launch_sketch(R->batch.packed.p, R->batch.poff.p, R->batch.qlen.p, R->batch.exc.p, R->batch.eoff.p,
                             (int)n, R->k, R->s, 1, R->seed, nullptr, 0, nullptr, R->ref_h.p, R->ref_off.p,
                             (int)R->refs.size(), R->ref_tab.p, R->ref_tab_mask, R->best.p, R->best_j.p, R->queue.p,
                             sm_count(), R->st));
    HG_CUDA(cudaEventRecord(R->ev[1], R->st));
    if (n) {
        HG_CUDA(cudaMemcpyAsync(best, R->best.p, 4 * (size_t)n, cudaMemcpyDeviceToHost, R->st));
        HG_CUDA(cudaMemcpyAsync(jaccard, R->best_j.p, 8 * (size_t)n, cudaMemcpyDeviceToHost, R->st));
    }
    HG_CUDA(cudaStreamSynchronize(R->st));
    HG_CUDA(cudaEventElapsedTime(&R->last_ms, R->ev[0], R->ev[1]));
    return HG_OK;
}

extern "C" int hg_refset_last_ms(const hg_refset_t* R, float* select_ms)
{
    if (!R || !select_ms) return fail(HG_ERR_ARG, "hg_refset_last_ms: bad arguments");
    *select_ms = R->last_ms;
    return HG_OK;
}

extern "C" int hg_refset_align(hg_refset_t* R, const uint8_t* packed, const int64_t* poff, const int32_t* qlen,
                               const int32_t* exc, const int64_t* exc_off, int64_t n, int keep_length, int32_t* best,
                               double* jaccard, uint32_t* cigar, int64_t cigar_cap, int64_t* cigar_off,
                               uint8_t* has_ins, uint8_t* rows, int64_t row_stride, uint32_t* status)
{
    if (!R || n < 0 || (n && (!packed || !poff || !qlen || !exc_off || !cigar || !cigar_off)))
        return fail(HG_ERR_ARG, "hg_refset_align: bad arguments");
    int64_t max_len = 0;
    hg_refset_info(R, nullptr, &max_len, nullptr);
    const int n_refs = (int)R->refs.size();
    std::vector<int32_t> best_l;
    std::vector<double> jac_l;
    if (!best) best_l.resize((size_t)n), best = best_l.data();
    if (!jaccard) jac_l.resize((size_t)n), jaccard = jac_l.data();
    int rc = hg_refset_select(R, packed, poff, qlen, exc, exc_off, n, best, jaccard);
    if (rc) return rc;
    // the batches: with --keep-length and several references, the queries of
    // each reference; otherwise every query against the one reference or the
    // consensus (the re-check).  Each runs through pinned staging and comes
    // back in input order.
    struct Group {
        hg_ctx_t* ctx = nullptr;
        int64_t L = 0;
        std::vector<int64_t> m;
    };
    std::vector<Group> groups;
    if (n_refs == 1 || !keep_length) {
        Group g;
        rc = n_refs == 1 ? ctx_of(R, 0, &g.ctx) : cons_ctx_of(R, &g.ctx);
        if (rc) return rc;
        g.L = hg::index_length(n_refs == 1 ? R->ix[0] : R->cons_ix);
        g.m.resize((size_t)n);
        for (int64_t i = 0; i < n; ++i) g.m[(size_t)i] = i;
        groups.push_back(std::move(g));
    } else {
        groups.resize((size_t)n_refs);
        for (int64_t i = 0; i < n; ++i) groups[(size_t)best[i]].m.push_back(i);
        for (int r = 0; r < n_refs; ++r) {
            groups[(size_t)r].L = (int64_t)R->refs[(size_t)r].size();
            if (!groups[(size_t)r].m.empty() && (rc = ctx_of(R, r, &groups[(size_t)r].ctx))) return rc;
        }
    }
    for (const auto& g : groups)
        if (rows && !g.m.empty() && row_stride < g.L)
            return fail(HG_ERR_ARG, "hg_refset_align: row_stride below the aligned-to length");
    const int n_groups = (int)groups.size();
    std::vector<std::vector<uint32_t>> cig_g((size_t)n_groups);
    std::vector<std::vector<int64_t>> off_g((size_t)n_groups);
    std::vector<int64_t> n_cig((size_t)n, 0);
    std::vector<uint8_t> ins_l;
    std::vector<uint32_t> st_l;
    if (!has_ins) ins_l.resize((size_t)n), has_ins = ins_l.data();
    if (!status) st_l.resize((size_t)n), status = st_l.data();
    int first_err = HG_OK;
    std::string first_msg;
    std::vector<int64_t> gpoff, geoff;
    std::vector<int32_t> gq, gexc;
    std::vector<uint8_t> gins;
    std::vector<uint32_t> gst;
    for (int r = 0; r < n_groups; ++r) {
        const auto& m = groups[(size_t)r].m;
        const int64_t ng = (int64_t)m.size();
        if (!ng) continue;
        hg_ctx_t* c = groups[(size_t)r].ctx;
        // gather the group's inputs
        int64_t pb = 0, ne = 0, bases = 0;
        for (int64_t i : m) pb += (int64_t)padded_bytes(qlen[i]), ne += exc_off[i + 1] - exc_off[i], bases += qlen[i];
        cudaError_t pe = R->h_packed.fit((size_t)std::max<int64_t>(pb, 16));
        if (!pe && rows) pe = R->h_rows.fit((size_t)(ng * row_stride));
        if (pe) return hg::cuda_error(pe, "hg_refset_align: pinned staging");
        uint8_t* gp = R->h_packed.p;
        uint8_t* grows = rows ? R->h_rows.p : nullptr;
        gpoff.resize((size_t)ng), geoff.resize((size_t)ng + 1), gq.resize((size_t)ng);
        gexc.resize((size_t)std::max<int64_t>(ne, 1) * 3);
        int64_t o = 0, eo = 0;
        geoff[0] = 0;
        for (int64_t j = 0; j < ng; ++j) {  // offsets first, then the copies in parallel
            const int64_t i = m[(size_t)j];
            gpoff[j] = o, gq[j] = qlen[i];
            o += (int64_t)padded_bytes(qlen[i]);
            eo += exc_off[i + 1] - exc_off[i];
            geoff[j + 1] = eo;
        }
#pragma omp parallel for schedule(dynamic, 64)
        for (int64_t j = 0; j < ng; ++j) {
            const int64_t i = m[(size_t)j];
            std::memcpy(gp + gpoff[j], packed + poff[i], padded_bytes(qlen[i]));
            const int64_t ei = exc_off[i + 1] - exc_off[i];
            if (ei) std::memcpy(gexc.data() + 3 * geoff[j], exc + 3 * exc_off[i], 12 * (size_t)ei);
        }
        const int64_t L = groups[(size_t)r].L;
        int64_t cap = bases / 8 + 64 * ng + 1024;
        cig_g[r].resize((size_t)cap), off_g[r].resize((size_t)ng + 1);
        gins.resize((size_t)ng), gst.resize((size_t)ng);
        rc = hg_align_batch(c, gp, gpoff.data(), gq.data(), gexc.data(), geoff.data(), ng, cig_g[r].data(), cap,
                            off_g[r].data(), gins.data(), grows, row_stride, gst.data());
        if (rc == HG_ERR_CAPACITY) {  // CIGARs longer than the first guess: the worst case fits
            cap = bases + ng * (L + 4);
            cig_g[r].resize((size_t)cap);
            rc = hg_align_batch(c, gp, gpoff.data(), gq.data(), gexc.data(), geoff.data(), ng, cig_g[r].data(),
                                cap, off_g[r].data(), gins.data(), grows, row_stride, gst.data());
        }
        if (rc && rc != HG_ERR_LENGTH_MISMATCH && rc != HG_ERR_CIGAR) return rc;
        if (rc && !first_err) first_err = rc, first_msg = hg_last_error();
#pragma omp parallel for schedule(dynamic, 64)
        for (int64_t j = 0; j < ng; ++j) {
            const int64_t i = m[(size_t)j];
            n_cig[i] = off_g[r][j + 1] - off_g[r][j];
            has_ins[i] = gins[j], status[i] = gst[j];
            if (rows) std::memcpy(rows + i * row_stride, grows + j * row_stride, (size_t)row_stride);
        }
    }
    // CIGARs in input order
    cigar_off[0] = 0;
    for (int64_t i = 0; i < n; ++i) cigar_off[i + 1] = cigar_off[i] + n_cig[i];
    if (n && cigar_off[n] > cigar_cap) return fail(HG_ERR_CAPACITY, "hg_refset_align: cigar buffer too small");
    for (int r = 0; r < n_groups; ++r) {
        const auto& m = groups[(size_t)r].m;
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t j = 0; j < (int64_t)m.size(); ++j) {
            const int64_t i = m[(size_t)j];
            if (n_cig[i]) std::memcpy(cigar + cigar_off[i], cig_g[r].data() + off_g[r][j], 4 * (size_t)n_cig[i]);
        }
    }
    if (first_err) return fail(first_err, first_msg);
    return HG_OK;
}
