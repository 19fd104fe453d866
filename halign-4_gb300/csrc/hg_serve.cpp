// hg_serve.cpp - the continuous-batching request loop behind hg_serve_*
// (include/halign_gb300.h): a FIFO of submitted requests whose bytes are
// copied into a ring of pinned host memory, a pool of contexts over one
// resident index, a submitting thread that admits micro-batches into free
// contexts (their bytes upload straight from the ring and the device packs
// them) and a collecting thread that polls, collects and files them.
//
// Host code only; every alignment runs through the context calls of the C
// ABI.  Requests are independent, so a request's result in the mix is its
// result alone.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/halign_gb300.h"
#include "hg_internal.h"
#include "hg_ring.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    int64_t pos = 0, len = 0;     // bytes at ring position pos (monotonic; ring offset pos % capacity)
    bool released = false;        // filed: its ring bytes may be reused
    Clock::time_point t_in;
    double latency_ms = 0;
    uint32_t status = 0;
    std::vector<uint32_t> cigar;  // filled when finished
    bool returned = false;        // handed out by hg_serve_result
};

struct Slot {
    hg_ctx_t* ctx = nullptr;
    std::vector<int64_t> ids;     // requests of the micro-batch in flight
    std::vector<uint32_t> cig;
    std::vector<int64_t> off;
    std::vector<uint8_t> ins;
    std::vector<uint32_t> st;
    int state = 0;  // 0 free, 1 packing (submitting thread), 2 in flight (collecting thread)
};

}  // namespace

struct hg_server {
    hg_index_t* ix = nullptr;
    int device = 0;
    int64_t slot_q = 0, slot_b = 0;
    int64_t arena_bytes = 0;
    std::vector<Slot> slots;
    std::mutex mu;
    std::condition_variable cv_work, cv_done, cv_busy, cv_space;
    // request bytes: a ring of pinned host memory (hg_ring.h).  Writers take
    // submit_mu, so ring order is id order and the ring is free before the
    // oldest unreleased request (rel_id).
    char* ring = nullptr;
    hg::ByteRing rb;
    int64_t rel_id = 0;
    std::mutex submit_mu;
    std::deque<Request> reqs;     // request id - base_id indexes it
    int64_t base_id = 0;
    std::deque<int64_t> pending;  // submitted, not yet admitted
    std::deque<int64_t> done;     // finished, not yet returned
    std::vector<float> lat;       // latencies of finished requests (stats)
    int64_t bases_done = 0, batches = 0;
    Clock::time_point t_first, t_last;
    bool have_first = false;
    bool stop = false;
    int error = HG_OK;
    std::string error_msg;
    bool submitter_done = false;
    std::thread sub, col;
};

namespace {

int64_t arena_of(hg_index_t* ix, int64_t q, int64_t b, hg_ctx_t** out)
{
    size_t f0 = 0, f1 = 0, tot = 0;
    cudaMemGetInfo(&f0, &tot);
    int r = hg_ctx_create(ix, q, b, out);
    if (r) return -r;
    if ((r = hg::prepare_pinned_ascii(*out))) {  // the device-packing buffers count against the budget too
        hg_ctx_destroy(*out);
        *out = nullptr;
        return -r;
    }
    cudaMemGetInfo(&f1, &tot);
    return f0 > f1 ? (int64_t)(f0 - f1) : 0;
}

// Fills slot s with the oldest waiting requests: their ids, lengths and the
// runs of the ring that hold their bytes back to back (one run, or two where
// the ring wraps).  Called with the lock held.
void admit(hg_server* S, std::vector<int64_t>& take, std::vector<int64_t>& len, std::vector<const char*>& run_ptr,
           std::vector<int64_t>& run_bytes, int64_t max_q)
{
    take.clear(), len.clear(), run_ptr.clear(), run_bytes.clear();
    int64_t bases = 0, end = -1;
    while (!S->pending.empty() && (int64_t)take.size() < max_q) {
        const int64_t id = S->pending.front();
        const Request& r = S->reqs[(size_t)(id - S->base_id)];
        if (!take.empty() && bases + r.len > S->slot_b) break;
        S->pending.pop_front();
        take.push_back(id);
        len.push_back(r.len);
        bases += r.len;
        if (r.len == 0) continue;
        if (S->rb.continues(end, r.pos)) {
            run_bytes.back() += r.len;
        } else {
            run_ptr.push_back(S->ring + S->rb.offset(r.pos));
            run_bytes.push_back(r.len);
        }
        end = r.pos + r.len;
    }
}

// After requests were released: the ring is free up to the oldest
// unreleased request (or all queued bytes).  Called with the lock held.
void advance_ring(hg_server* S)
{
    const int64_t end = S->base_id + (int64_t)S->reqs.size();
    S->rel_id = std::max(S->rel_id, S->base_id);
    while (S->rel_id < end && S->reqs[(size_t)(S->rel_id - S->base_id)].released) ++S->rel_id;
    if (S->rel_id < end) S->rb.release_before(S->reqs[(size_t)(S->rel_id - S->base_id)].pos);
    else S->rb.release_all();
}

void fail_all(hg_server* S, int code, const std::string& msg)
{
    std::lock_guard<std::mutex> lock(S->mu);
    S->error = code;
    S->error_msg = msg;
    S->cv_done.notify_all();
    S->cv_work.notify_all();
    S->cv_busy.notify_all();
    S->cv_space.notify_all();
}

// Submitting thread: whenever a context is free and requests wait, admit the
// oldest (under the lock, so micro-batches leave the FIFO in order; fewer
// while most contexts are idle) and enqueue them: their ring bytes upload as
// they are and the device packs them; the context is then the collecting
// thread's to poll.
void submitter(hg_server* S)
{
    cudaSetDevice(S->device);
    std::vector<int64_t> take, len, run_bytes;
    std::vector<const char*> run_ptr;
    const int ns = (int)S->slots.size();
    for (;;) {
        int s = -1;
        {
            std::unique_lock<std::mutex> lock(S->mu);
            S->cv_work.wait(lock, [&] {
                if (S->error || (S->stop && S->pending.empty())) return true;
                if (S->pending.empty()) return false;
                for (const Slot& sl : S->slots)
                    if (sl.state == 0) return true;
                return false;
            });
            if (S->error || (S->stop && S->pending.empty())) {
                S->submitter_done = true;
                S->cv_busy.notify_all();
                return;
            }
            int busy = 0;
            for (int i = 0; i < ns; ++i) {
                if (S->slots[i].state == 0 && s < 0) s = i;
                busy += S->slots[i].state != 0;
            }
            // ramp: with b contexts busy a micro-batch takes at most (b + 1) / ns
            // of a context's queries, so an idle GPU starts on a small micro-batch
            // instead of a full one; with all others busy it takes a full one
            const int64_t max_q = std::max<int64_t>(std::min<int64_t>(S->slot_q, 1024), S->slot_q * (busy + 1) / ns);
            admit(S, take, len, run_ptr, run_bytes, max_q);
            S->slots[s].ids = take;
            S->slots[s].state = 1;  // packing
            ++S->batches;
        }
        // the ring bytes stay put until the requests are filed (only the
        // collecting thread releases them), so this runs without the lock
        const int r = hg::submit_pinned_ascii(S->slots[s].ctx, run_ptr.data(), run_bytes.data(), (int)run_ptr.size(),
                                              len.data(), (int64_t)take.size());
        if (r) {
            fail_all(S, r, hg_last_error());
            return;
        }
        {
            std::lock_guard<std::mutex> lock(S->mu);
            S->slots[s].state = 2;  // in flight
        }
        S->cv_busy.notify_all();
    }
}

// Collecting thread: poll the contexts in flight, collect a finished one's
// CIGARs and statuses, file them per request and free the context.
void collector(hg_server* S)
{
    cudaSetDevice(S->device);
    const int ns = (int)S->slots.size();
    std::vector<int> inflight;
    std::vector<std::vector<uint32_t>> cigs;
    for (;;) {
        inflight.clear();
        {
            std::unique_lock<std::mutex> lock(S->mu);
            S->cv_busy.wait(lock, [&] {
                if (S->error) return true;
                bool busy = false;
                for (const Slot& sl : S->slots) {
                    if (sl.state == 2) return true;
                    busy = busy || sl.state != 0;
                }
                return S->submitter_done && !busy;
            });
            if (S->error) return;
            for (int i = 0; i < ns; ++i)
                if (S->slots[i].state == 2) inflight.push_back(i);
            if (inflight.empty()) return;  // the submitter stopped and nothing is left
        }
        bool progressed = false;
        for (const int s : inflight) {
            Slot& sl = S->slots[s];
            const int p = hg_poll(sl.ctx);
            if (p < 0) {
                fail_all(S, -p, hg_last_error());
                return;
            }
            if (p == 0) continue;
            const size_t n = sl.ids.size();
            int64_t bases = 0;
            {
                std::lock_guard<std::mutex> lock(S->mu);
                for (int64_t id : sl.ids) bases += S->reqs[(size_t)(id - S->base_id)].len;
            }
            sl.cig.resize((size_t)bases / 8 + 64 * n + 1024);  // a few ops per kilobase; grown below if short
            sl.off.resize(n + 1), sl.ins.resize(n), sl.st.resize(n);
            int r = hg_collect(sl.ctx, sl.cig.data(), (int64_t)sl.cig.size(), sl.off.data(), sl.ins.data(), sl.st.data());
            if (r == HG_ERR_CAPACITY && !hg::async_exc_overflow(sl.ctx)) {
                // rare: CIGARs longer than the first guess; the worst case fits
                sl.cig.resize((size_t)bases + n * (size_t)(hg::index_length(S->ix) + 4));
                r = hg_collect(sl.ctx, sl.cig.data(), (int64_t)sl.cig.size(), sl.off.data(), sl.ins.data(),
                               sl.st.data());
            }
            if (r && r != HG_ERR_LENGTH_MISMATCH) {
                fail_all(S, r, hg_last_error());
                return;
            }
            const auto now = Clock::now();
            cigs.resize(n);
            for (size_t j = 0; j < n; ++j) cigs[j].assign(sl.cig.begin() + sl.off[j], sl.cig.begin() + sl.off[j + 1]);
            {
                std::lock_guard<std::mutex> lock(S->mu);
                for (size_t j = 0; j < n; ++j) {
                    Request& q = S->reqs[(size_t)(sl.ids[j] - S->base_id)];
                    q.cigar.swap(cigs[j]);
                    q.status = sl.st[j];
                    q.latency_ms = std::chrono::duration<double, std::milli>(now - q.t_in).count();
                    q.released = true;
                    S->lat.push_back((float)q.latency_ms);
                    S->done.push_back(sl.ids[j]);
                }
                advance_ring(S);
                S->bases_done += bases;
                S->t_last = now;
                sl.ids.clear();
                sl.state = 0;
            }
            S->cv_done.notify_all();
            S->cv_work.notify_all();
            S->cv_space.notify_all();
            progressed = true;
        }
        if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
}

}  // namespace

extern "C" int hg_serve_create(hg_index_t* ix, int n_slots, int64_t slot_queries, int64_t slot_bases,
                               int64_t budget_bytes, hg_server_t** out)
{
    if (!ix || !out || n_slots <= 0 || slot_queries <= 0 || slot_bases <= 0 || budget_bytes <= 0)
        return hg::set_error(HG_ERR_ARG, "hg_serve_create: bad arguments");
    int dev = 0;
    if (hg_index_device(ix, &dev, nullptr, 0) != HG_OK) return HG_ERR_ARG;
    cudaSetDevice(dev);
    auto* S = new hg_server();
    S->ix = ix, S->device = dev, S->slot_q = slot_queries, S->slot_b = slot_bases;
    for (int i = 0; i < n_slots; ++i) {
        hg_ctx_t* c = nullptr;
        const int64_t bytes = arena_of(ix, slot_queries, slot_bases, &c);
        if (bytes < 0) {
            hg_serve_destroy(S);
            return (int)-bytes;
        }
        if (S->arena_bytes + bytes > budget_bytes) {  // the budget holds no more contexts
            hg_ctx_destroy(c);
            break;
        }
        S->arena_bytes += bytes;
        S->slots.push_back(Slot{});
        S->slots.back().ctx = c;
    }
    if (S->slots.empty()) {
        hg_serve_destroy(S);
        return hg::set_error(HG_ERR_CAPACITY, "hg_serve_create: one context does not fit the device-memory budget");
    }
    // the ring holds what every context can take at once and as much again
    // waiting (at most 8 GiB unless one request needs more: a request of up
    // to slot_bases always fits, wrap included, in 2 x slot_bases); it is
    // pinned, so micro-batches upload from it directly.  Where the host
    // cannot pin that much, smaller rings down to that floor are tried.
    const int64_t floor_b = std::max<int64_t>(2 * slot_bases, 1 << 20);
    S->rb.cap = std::max(floor_b, std::min<int64_t>(2 * (int64_t)S->slots.size() * slot_bases, 8LL << 30));
    while (cudaHostAlloc(reinterpret_cast<void**>(&S->ring), (size_t)S->rb.cap, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        S->ring = nullptr;
        if (S->rb.cap <= floor_b) {
            hg_serve_destroy(S);
            return hg::set_error(HG_ERR_NOMEM, "hg_serve_create: pinned request ring");
        }
        S->rb.cap = std::max(floor_b, S->rb.cap / 2);
    }
    S->sub = std::thread(submitter, S);
    S->col = std::thread(collector, S);
    *out = S;
    return HG_OK;
}

extern "C" void hg_serve_destroy(hg_server_t* S)
{
    if (!S) return;
    {
        std::lock_guard<std::mutex> lock(S->mu);
        S->stop = true;
        S->pending.clear();
    }
    S->cv_work.notify_all();
    S->cv_space.notify_all();
    if (S->sub.joinable()) S->sub.join();
    if (S->col.joinable()) S->col.join();
    for (auto& sl : S->slots) hg_ctx_destroy(sl.ctx);
    if (S->ring) cudaFreeHost(S->ring);
    delete S;
}

namespace {

// Queues requests i = 0..n-1 (bytes at seqs + offsets[i] .. offsets[i+1])
// with one time stamp: in chunks, each reserved in the ring under the lock
// (waiting while it is full), copied without it and then queued, so the
// submitting thread starts on the first chunk while later ones copy.
// Returns the first id or a negative HG_ERR_*.
int64_t enqueue(hg_server* S, const char* seqs, const int64_t* offsets, int64_t n, const char* who)
{
    for (int64_t i = 0; i < n; ++i) {
        const int64_t len = offsets[i + 1] - offsets[i];
        if (len < 0) return -hg::set_error(HG_ERR_ARG, std::string(who) + ": offsets not ascending");
        if (len > S->slot_b) return -hg::set_error(HG_ERR_CAPACITY, std::string(who) + ": request longer than slot_bases");
    }
    const auto now = Clock::now();
    std::lock_guard<std::mutex> writer(S->submit_mu);  // ring order = id order
    if (n == 0) {
        std::lock_guard<std::mutex> lock(S->mu);
        return S->base_id + (int64_t)S->reqs.size();
    }
    int64_t first = -1;
    std::vector<int64_t> pos;
    for (int64_t i = 0; i < n;) {
        int64_t j = i;
        {
            std::unique_lock<std::mutex> lock(S->mu);
            S->cv_space.wait(lock, [&] { return S->error || S->stop || S->rb.fits(offsets[i + 1] - offsets[i]); });
            if (S->error) return -hg::set_error(S->error, S->error_msg);
            if (S->stop) return -hg::set_error(HG_ERR_ARG, std::string(who) + ": the server is stopping");
            pos.clear();
            int64_t bytes = 0;
            while (j < n && j - i < 8192 && bytes < (64 << 20)) {
                const int64_t len = offsets[j + 1] - offsets[j];
                if (!S->rb.fits(len)) break;
                pos.push_back(S->rb.reserve(len));
                bytes += len;
                ++j;
            }
        }
        const int64_t m = j - i;
#pragma omp parallel for schedule(dynamic, 64) if (m > 256)
        for (int64_t k = 0; k < m; ++k) {
            const int64_t len = offsets[i + k + 1] - offsets[i + k];
            if (len) std::memcpy(S->ring + S->rb.offset(pos[(size_t)k]), seqs + offsets[i + k], (size_t)len);
        }
        {
            std::lock_guard<std::mutex> lock(S->mu);
            if (S->error) return -hg::set_error(S->error, S->error_msg);
            if (!S->have_first) S->t_first = now, S->have_first = true;
            const int64_t id0 = S->base_id + (int64_t)S->reqs.size();
            if (first < 0) first = id0;
            for (int64_t k = 0; k < m; ++k) {
                Request r;
                r.pos = pos[(size_t)k], r.len = offsets[i + k + 1] - offsets[i + k];
                r.t_in = now;
                S->reqs.push_back(std::move(r));
                S->pending.push_back(id0 + k);
            }
            S->rb.publish();
        }
        S->cv_work.notify_one();
        i = j;
    }
    return first;
}

}  // namespace

extern "C" int64_t hg_serve_submit(hg_server_t* S, const char* seq, int64_t len)
{
    if (!S || len < 0 || (len > 0 && !seq)) return -hg::set_error(HG_ERR_ARG, "hg_serve_submit: bad arguments");
    const int64_t off[2] = {0, len};
    return enqueue(S, seq, off, 1, "hg_serve_submit");
}

extern "C" int64_t hg_serve_submit_many(hg_server_t* S, const char* seqs, const int64_t* offsets, int64_t n)
{
    if (!S || n < 0 || (n > 0 && (!seqs || !offsets)))
        return -hg::set_error(HG_ERR_ARG, "hg_serve_submit_many: bad arguments");
    return enqueue(S, seqs, offsets, n, "hg_serve_submit_many");
}

extern "C" int64_t hg_serve_results(hg_server_t* S, int64_t max_n, int64_t* ids, uint32_t* status,
                                    double* latency_ms, uint32_t* cigar, int64_t cigar_cap, int64_t* cigar_off,
                                    int timeout_ms)
{
    if (!S || max_n <= 0 || !ids || !cigar_off || (cigar_cap > 0 && !cigar))
        return -hg::set_error(HG_ERR_ARG, "hg_serve_results: bad arguments");
    std::unique_lock<std::mutex> lock(S->mu);
    auto ready = [&] { return !S->done.empty() || S->error; };
    if (timeout_ms < 0) S->cv_done.wait(lock, ready);
    else if (!S->cv_done.wait_for(lock, std::chrono::milliseconds(timeout_ms), ready)) return 0;
    if (S->done.empty()) return -hg::set_error(S->error, S->error_msg);
    int64_t m = 0, used = 0;
    cigar_off[0] = 0;
    while (m < max_n && !S->done.empty()) {
        const int64_t rid = S->done.front();
        Request& r = S->reqs[(size_t)(rid - S->base_id)];
        const int64_t nc = (int64_t)r.cigar.size();
        if (used + nc > cigar_cap) {
            if (m == 0) return -hg::set_error(HG_ERR_CAPACITY, "hg_serve_results: cigar_cap below the next CIGAR");
            break;
        }
        S->done.pop_front();
        ids[m] = rid;
        if (status) status[m] = r.status;
        if (latency_ms) latency_ms[m] = r.latency_ms;
        if (nc) std::memcpy(cigar + used, r.cigar.data(), sizeof(uint32_t) * (size_t)nc);
        used += nc;
        cigar_off[++m] = used;
        std::vector<uint32_t>().swap(r.cigar);
        r.returned = true;
    }
    while (!S->reqs.empty() && S->reqs.front().returned) {
        S->reqs.pop_front();
        ++S->base_id;
    }
    return m;
}

extern "C" int hg_serve_result(hg_server_t* S, int64_t* id, uint32_t* status, double* latency_ms, uint32_t* cigar,
                               int64_t cap, int64_t* n_cigar, int timeout_ms)
{
    if (!S || !id) return -hg::set_error(HG_ERR_ARG, "hg_serve_result: bad arguments");
    std::unique_lock<std::mutex> lock(S->mu);
    auto ready = [&] { return !S->done.empty() || S->error; };
    if (timeout_ms < 0) S->cv_done.wait(lock, ready);
    else if (!S->cv_done.wait_for(lock, std::chrono::milliseconds(timeout_ms), ready)) return 0;
    if (S->done.empty()) return -hg::set_error(S->error, S->error_msg);
    const int64_t rid = S->done.front();
    S->done.pop_front();
    Request& r = S->reqs[(size_t)(rid - S->base_id)];
    *id = rid;
    if (status) *status = r.status;
    if (latency_ms) *latency_ms = r.latency_ms;
    if (n_cigar) *n_cigar = (int64_t)r.cigar.size();
    if (cigar && cap > 0) std::memcpy(cigar, r.cigar.data(), sizeof(uint32_t) * std::min<size_t>((size_t)cap, r.cigar.size()));
    std::vector<uint32_t>().swap(r.cigar);
    r.returned = true;
    while (!S->reqs.empty() && S->reqs.front().returned) {  // the store keeps only unreturned requests
        S->reqs.pop_front();
        ++S->base_id;
    }
    return 1;
}

extern "C" int hg_serve_stats(hg_server_t* S, double* out, int n, int reset)
{
    if (!S || !out || n <= 0) return hg::set_error(HG_ERR_ARG, "hg_serve_stats: bad arguments");
    std::lock_guard<std::mutex> lock(S->mu);
    std::vector<float> v = S->lat;
    double res[10] = {};
    if (!v.empty()) {
        std::sort(v.begin(), v.end());
        auto pct = [&](double q) { return (double)v[std::min(v.size() - 1, (size_t)(q * (double)(v.size() - 1) + 0.5))]; };
        double sum = 0;
        for (float x : v) sum += x;
        res[0] = pct(0.50), res[1] = pct(0.99), res[2] = sum / (double)v.size(), res[3] = v.back();
    }
    res[4] = (double)v.size(), res[5] = (double)S->bases_done, res[6] = (double)S->batches;
    res[7] = S->have_first && !v.empty() ? std::chrono::duration<double>(S->t_last - S->t_first).count() : 0.0;
    res[8] = (double)S->slots.size(), res[9] = (double)S->arena_bytes;
    for (int i = 0; i < n && i < 10; ++i) out[i] = res[i];
    if (reset) {
        S->lat.clear();
        S->bases_done = 0, S->batches = 0;
        S->have_first = false;
    }
    return HG_OK;
}

extern "C" int hg_serve_counters(hg_server_t* S, uint32_t* counts7, uint32_t* ins, int reset)
{
    if (!S || !counts7 || !ins) return hg::set_error(HG_ERR_ARG, "hg_serve_counters: bad arguments");
    const int64_t L = hg::index_length(S->ix);
    std::vector<uint32_t> c((size_t)L * 7), i((size_t)L + 1);
    std::fill(counts7, counts7 + 7 * L, 0u);
    std::fill(ins, ins + L + 1, 0u);
    for (auto& sl : S->slots) {  // uint32 sums wrap as SiteCount's counters do
        const int r = hg_counters(sl.ctx, c.data(), i.data(), reset);
        if (r) return r;
        for (size_t k = 0; k < c.size(); ++k) counts7[k] += c[k];
        for (size_t k = 0; k < i.size(); ++k) ins[k] += i[k];
    }
    return HG_OK;
}
