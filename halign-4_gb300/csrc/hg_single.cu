// hg_single.cu - single-call entry points of the C ABI: the functions the
// C++ drop-in surface (include/halign4/*.h, implemented over this ABI by
// hg_shim.cpp) calls one sequence or one anchor list at a time.
//
// * extractMinimizer and ksw_extz2 single calls (the batch kernels on one
//   input);
// * collect_anchors and chainAnchors for arbitrary hit and anchor lists
//   (several sequences, both strands, per-anchor spans), which the batch
//   path never needs because it aligns one forward-strand center;
// * delQueryToRefByCigar / padQueryToRefByCigar row projection and
//   SiteCount accumulation of caller rows.
//
// Every single call runs on the calling thread's Workspace: one non-blocking
// stream and grow-only device buffers per thread and device, so a call
// allocates only while the buffers grow to the largest call seen.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/halign_gb300.h"
#include "hg_batch.cuh"
#include "hg_internal.h"

extern "C" {
cudaError_t hg_launch_seed(const hg::IndexDev*, const hg::BatchDev*, int, uint64_t*, uint64_t*, int, cudaStream_t);
size_t hg_ksw_scratch_bytes(int, int, int, int);
cudaError_t hg_launch_ksw_single(int, const uint8_t*, int, const uint8_t*, int, const int8_t*, int, int, int, int,
                                 int, int, uint8_t*, uint32_t*, int, void*, cudaStream_t);
cudaError_t hg_launch_count(const uint8_t*, int64_t, int, int, uint32_t*, cudaStream_t);
}

static_assert(sizeof(hg_anchor_t) == 32, "hg_anchor_t is anchor::Anchor's 32-byte record");

namespace hg {

// ------------------------------------------------------------ workspace

Workspace::~Workspace()
{
    // the buffers belong to `device`; errors at process teardown are ignored
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess) cur = -1;
    if (device >= 0) cudaSetDevice(device);
    if (st) cudaStreamSynchronize(st);
    for (int i = 0; i < kSlots; ++i)
        if (dptr[i]) cudaFree(dptr[i]);
    if (hptr) cudaFreeHost(hptr);
    if (st) cudaStreamDestroy(st);
    if (cur >= 0) cudaSetDevice(cur);
    cudaGetLastError();
}

cudaError_t Workspace::dev(int slot, size_t bytes, void** out)
{
    if (bytes > dcap[slot]) {
        // growing frees the old buffer: work queued on the stream may still read it
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return e;
        const size_t old = dcap[slot];
        if (dptr[slot]) cudaFree(dptr[slot]);
        dptr[slot] = nullptr, dcap[slot] = 0;
        const size_t want = std::max<size_t>((bytes + 255) / 256 * 256, 4096);
        const size_t grown = std::max(want, (old + old / 2 + 255) / 256 * 256);
        e = cudaMalloc(&dptr[slot], grown);
        if (e != cudaSuccess) return e;
        dcap[slot] = grown;
    }
    *out = dptr[slot];
    return cudaSuccess;
}

cudaError_t Workspace::host(size_t bytes, void** out)
{
    if (bytes > hcap) {
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return e;
        if (hptr) cudaFreeHost(hptr);
        hptr = nullptr, hcap = 0;
        const size_t want = std::max<size_t>(bytes, 1 << 16);
        e = cudaMallocHost(&hptr, want);
        if (e != cudaSuccess) return e;
        hcap = want;
    }
    *out = hptr;
    return cudaSuccess;
}

namespace {
thread_local std::map<int, std::unique_ptr<Workspace>> tl_ws;
}

int workspace(Workspace** out)
{
    int dev = 0;
    HG_CUDA(cudaGetDevice(&dev));
    auto& slot = tl_ws[dev];
    if (!slot) {
        auto ws = std::make_unique<Workspace>();
        ws->device = dev;
        HG_CUDA(cudaStreamCreateWithFlags(&ws->st, cudaStreamNonBlocking));
        slot = std::move(ws);
    }
    *out = slot.get();
    return HG_OK;
}

template <typename T>
static cudaError_t ws_dev(Workspace* ws, int slot, size_t count, T** out)
{
    void* p = nullptr;
    const cudaError_t e = ws->dev(slot, sizeof(T) * std::max<size_t>(count, 1), &p);
    *out = static_cast<T*>(p);
    return e;
}

// ------------------------------------------------ minimizers of one sequence

int run_extract(int k, int w, int non_canonical, const char* seq, int64_t len, std::vector<uint64_t>& xs,
                std::vector<uint64_t>& ys)
{
    xs.clear(), ys.clear();
    if (len < k || k <= 0 || k > 31 || w <= 0 || w >= 256) return HG_OK;
    const int64_t offs[2] = {0, len};
    int64_t pbytes = 0, nexc = 0;
    int r = hg_pack(seq, offs, 1, nullptr, 0, nullptr, nullptr, 0, nullptr, &pbytes, &nexc);
    if (r) return r;
    std::vector<uint8_t> pk((size_t)pbytes);
    std::vector<int64_t> poff(1), eoff(2);
    std::vector<int32_t> exc((size_t)std::max<int64_t>(nexc, 1) * 3);
    r = hg_pack(seq, offs, 1, pk.data(), pbytes, poff.data(), exc.data(), nexc, eoff.data(), nullptr, nullptr);
    if (r) return r;
    Workspace* ws = nullptr;
    if ((r = workspace(&ws))) return r;
    cudaStream_t st = ws->st;
    const int64_t cap = len - k + 1;
    // small per-call words in one slot: poff, eoff[2], hoff (int64); qlen, n_hits, n_matched (int32);
    // exact list + queue heads (uint32)
    uint8_t* small = nullptr;
    uint8_t* d_pk = nullptr;
    int32_t* d_exc = nullptr;
    uint64_t *d_x = nullptr, *d_y = nullptr;
    HG_CUDA(ws_dev(ws, 0, 256, &small));
    HG_CUDA(ws_dev(ws, 1, pk.size() + 64, &d_pk));
    HG_CUDA(ws_dev(ws, 2, exc.size(), &d_exc));
    HG_CUDA(ws_dev(ws, 3, (size_t)cap, &d_x));
    HG_CUDA(ws_dev(ws, 4, (size_t)cap, &d_y));
    int64_t* d_poff = reinterpret_cast<int64_t*>(small);
    int64_t* d_eoff = d_poff + 1;
    int64_t* d_hoff = d_poff + 3;
    int32_t* d_qlen = reinterpret_cast<int32_t*>(small + 32);
    int32_t* d_nh = d_qlen + 1;
    int32_t* d_nm = d_qlen + 2;
    uint32_t* d_exact = reinterpret_cast<uint32_t*>(small + 64);
    unsigned int* d_q = reinterpret_cast<unsigned int*>(small + 128);
    // pinned staging: the small words at 0, packed bases at 64, exception runs after them, hits at hoff
    const size_t hoff = (64 + pk.size() + 4 * exc.size() + 15) / 16 * 16;
    uint8_t* h = nullptr;
    HG_CUDA(ws->host(hoff + 16 * (size_t)cap, reinterpret_cast<void**>(&h)));
    int64_t* hw = reinterpret_cast<int64_t*>(h);
    hw[0] = 0, hw[1] = eoff[0], hw[2] = eoff[1], hw[3] = 0;
    reinterpret_cast<int32_t*>(h + 32)[0] = (int32_t)len;
    std::memcpy(h + 64, pk.data(), pk.size());
    std::memcpy(h + 64 + pk.size(), exc.data(), 4 * exc.size());
    HG_CUDA(cudaMemsetAsync(small, 0, 256, st));
    HG_CUDA(cudaMemcpyAsync(small, h, 36, cudaMemcpyHostToDevice, st));
    HG_CUDA(cudaMemcpyAsync(d_pk, h + 64, pk.size(), cudaMemcpyHostToDevice, st));
    HG_CUDA(cudaMemcpyAsync(d_exc, h + 64 + pk.size(), 4 * exc.size(), cudaMemcpyHostToDevice, st));
    IndexDev ixd{};
    ixd.k = k, ixd.w = w, ixd.non_canonical = non_canonical;
    BatchDev bd{};
    bd.n = 1, bd.packed = d_pk, bd.poff = d_poff, bd.qlen = d_qlen, bd.exc = d_exc, bd.exc_off = d_eoff;
    bd.hoff = d_hoff, bd.n_hits = d_nh, bd.n_matched = d_nm, bd.queues = d_q;
    bd.exact_list = d_exact, bd.n_exact = d_q + 8;
    bd.ring_slots = 2 * w + 16;
    HG_CUDA(hg_launch_seed(&ixd, &bd, 1, d_x, d_y, 1, st));
    int32_t* h_nh = reinterpret_cast<int32_t*>(h + 48);
    HG_CUDA(cudaMemcpyAsync(h_nh, d_nh, 4, cudaMemcpyDeviceToHost, st));
    HG_CUDA(cudaStreamSynchronize(st));
    const int32_t nh = *h_nh;
    if (nh < 0 || nh > cap) return set_error(HG_ERR_CUDA, "extract: bad hit count");
    xs.resize((size_t)nh), ys.resize((size_t)nh);
    if (nh) {
        uint64_t* hx = reinterpret_cast<uint64_t*>(h + hoff);
        HG_CUDA(cudaMemcpyAsync(hx, d_x, 8 * (size_t)nh, cudaMemcpyDeviceToHost, st));
        HG_CUDA(cudaMemcpyAsync(hx + nh, d_y, 8 * (size_t)nh, cudaMemcpyDeviceToHost, st));
        HG_CUDA(cudaStreamSynchronize(st));
        std::memcpy(xs.data(), hx, 8 * (size_t)nh);
        std::memcpy(ys.data(), hx + nh, 8 * (size_t)nh);
    }
    return HG_OK;
}

// ------------------------------------------------ device sort of 128-bit keys
//
// Bitonic network over P = 2^m keys (padded with all-ones keys that sort
// last): tiles of kSortTile keys sort in shared memory, longer merges take
// one grid-wide pass per stride down to the tile, then finish in shared
// memory.  Keys are unique (the low word carries the input index), so the
// order is total and stable.

struct Key128 {
    unsigned long long hi, lo;
};

__device__ __forceinline__ bool key_gt(const Key128& a, const Key128& b)
{
    return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo);
}

constexpr int kSortTile = 2048;
constexpr int kSortThreads = 1024;

// Compare-exchange of pair k (of the P/2 pairs) at `stride` inside a merge of
// `size` keys; ascending where (index & size) == 0.
__device__ __forceinline__ void bitonic_pair(Key128* k, unsigned base, unsigned pair, unsigned size, unsigned stride)
{
    const unsigned i = 2 * stride * (pair / stride) + (pair % stride);
    const unsigned j = i + stride;
    Key128 a = k[i], b = k[j];
    const bool asc = ((base + i) & size) == 0;
    if (asc ? key_gt(a, b) : key_gt(b, a)) k[i] = b, k[j] = a;
}

// Sorts each tile (sizes 2 .. tile) or, with merge_size > 0, finishes the
// merge of size merge_size inside each tile (strides tile/2 .. 1).
__global__ void __launch_bounds__(kSortThreads) sort_tile_kernel(Key128* keys, unsigned tile, unsigned merge_size)
{
    __shared__ Key128 s[kSortTile];
    const unsigned base = blockIdx.x * tile;
    for (unsigned i = threadIdx.x; i < tile; i += blockDim.x) s[i] = keys[base + i];
    __syncthreads();
    if (merge_size == 0) {
        for (unsigned size = 2; size <= tile; size <<= 1)
            for (unsigned stride = size >> 1; stride > 0; stride >>= 1) {
                for (unsigned pr = threadIdx.x; pr < tile / 2; pr += blockDim.x) bitonic_pair(s, base, pr, size, stride);
                __syncthreads();
            }
    } else {
        for (unsigned stride = tile >> 1; stride > 0; stride >>= 1) {
            for (unsigned pr = threadIdx.x; pr < tile / 2; pr += blockDim.x) bitonic_pair(s, base, pr, merge_size, stride);
            __syncthreads();
        }
    }
    for (unsigned i = threadIdx.x; i < tile; i += blockDim.x) keys[base + i] = s[i];
}

__global__ void sort_step_kernel(Key128* keys, unsigned P, unsigned size, unsigned stride)
{
    for (unsigned pr = blockIdx.x * blockDim.x + threadIdx.x; pr < P / 2; pr += gridDim.x * blockDim.x)
        bitonic_pair(keys, 0, pr, size, stride);
}

static unsigned sort_pad(int64_t n)
{
    unsigned P = 2;
    while ((int64_t)P < n) P <<= 1;
    return P;
}

static cudaError_t sort_keys(Key128* keys, unsigned P, cudaStream_t st)
{
    const unsigned tile = P < (unsigned)kSortTile ? P : (unsigned)kSortTile;
    const unsigned tiles = P / tile;
    const unsigned threads = std::min<unsigned>(kSortThreads, tile / 2);
    sort_tile_kernel<<<tiles, threads, 0, st>>>(keys, tile, 0);
    for (unsigned size = 2 * tile; size <= P; size <<= 1) {
        for (unsigned stride = size >> 1; stride >= tile; stride >>= 1) {
            const unsigned blocks = std::min<unsigned>((P / 2 + 255) / 256, 4096);
            sort_step_kernel<<<blocks, 256, 0, st>>>(keys, P, size, stride);
        }
        sort_tile_kernel<<<tiles, threads, 0, st>>>(keys, tile, size);
    }
    return cudaGetLastError();
}

// ------------------------------------------------ collect_anchors

// Reference-side hits on the device: hash table (hash56 -> entry), per entry
// {start in the sorted hits, count | over-threshold << 31}, the sorted hits.
struct HitsDev {
    const ulonglong2* tab;
    uint32_t mask;
    uint32_t n_ent;
    const uint2* ent;
    const unsigned long long* rx;
    const unsigned long long* ry;
};

__device__ __forceinline__ uint32_t hits_find(const HitsDev& h, uint64_t key)
{
    uint32_t s = (uint32_t)key & h.mask;
    for (;;) {
        const ulonglong2 e = h.tab[s];
        if (e.x == key) return (uint32_t)e.y;
        if (e.x == kNoHash) return kEmptyKey;
        s = (s + 1) & h.mask;
    }
}

// Pass 1: each query hit's entry, and per entry the query-side occurrence
// count of its hash (the --q-occ-frac count, src/seed/minimizer.cpp:280-288).
__global__ void collect_probe_kernel(HitsDev h, const unsigned long long* qx, int64_t nq, uint32_t* qent,
                                     uint32_t* qocc)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nq; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t e = hits_find(h, qx[i] >> 8);
        qent[i] = e;
        if (e != kEmptyKey) atomicAdd(&qocc[e], 1u);
    }
}

// Pass 2: anchors each query hit expands to after the filters
// (src/seed/minimizer.cpp:300-330).
__global__ void collect_size_kernel(HitsDev h, const unsigned long long* qy, int64_t nq, const uint32_t* qent,
                                    const uint32_t* qocc, double q_occ_frac, unsigned long long sample_every,
                                    unsigned long long* cnt)
{
    const double q_occ_limit = q_occ_frac * (double)nq;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nq; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t e = qent[i];
        unsigned long long n = 0;
        if (e != kEmptyKey) {
            const uint2 m = h.ent[e];
            bool keep = !(q_occ_frac > 0.0 && (double)qocc[e] > q_occ_limit);
            if (keep && (m.y >> 31)) {
                const unsigned long long pos = (uint32_t)qy[i];
                keep = sample_every != 0 && pos % sample_every == 0;
            }
            n = keep ? (m.y & 0x7fffffffu) : 0;
        }
        cnt[i] = n;
    }
}

// Exclusive scan of n counts into off[0..n], one CTA.
__global__ void __launch_bounds__(1024) scan_counts_kernel(const unsigned long long* cnt, int64_t n,
                                                            unsigned long long* off)
{
    __shared__ unsigned long long part[1024];
    const int tid = threadIdx.x;
    const int64_t per = (n + 1023) / 1024;
    const int64_t i0 = min(tid * per, n), i1 = min(i0 + per, n);
    unsigned long long s = 0;
    for (int64_t i = i0; i < i1; ++i) s += cnt[i];
    part[tid] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const unsigned long long v = tid >= o ? part[tid - o] : 0;
        __syncthreads();
        part[tid] += v;
        __syncthreads();
    }
    unsigned long long run = part[tid] - s;
    for (int64_t i = i0; i < i1; ++i) {
        off[i] = run;
        run += cnt[i];
    }
    if (tid == 1023) off[n] = part[1023];
}

// Pass 3: the anchors of each query hit at its scanned offset
// (src/seed/minimizer.cpp:334-352).
__global__ void collect_emit_kernel(HitsDev h, const unsigned long long* qx, const unsigned long long* qy, int64_t nq,
                                    const uint32_t* qent, const unsigned long long* cnt,
                                    const unsigned long long* off, hg_anchor_t* out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nq; i += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long n = cnt[i];
        if (!n) continue;
        const uint32_t start = h.ent[qent[i]].x;
        const unsigned long long x = qx[i], y = qy[i];
        const uint32_t qspan = (uint32_t)(x & 0xff);
        const uint32_t qrid = (uint32_t)(y >> 32) & 0x7fffffffu, qstrand = (uint32_t)(y >> 63);
        hg_anchor_t a;
        a.hash = x >> 8;
        a.rid_qry = qrid;
        a.pos_qry = (uint32_t)y;
        hg_anchor_t* o = out + off[i];
        for (unsigned long long k = 0; k < n; ++k) {
            const unsigned long long rx = h.rx[start + k], ry = h.ry[start + k];
            const uint32_t rspan = (uint32_t)(rx & 0xff);
            a.rid_ref = (uint32_t)(ry >> 32) & 0x7fffffffu;
            a.pos_ref = (uint32_t)ry;
            a.span = rspan < qspan ? rspan : qspan;
            a.is_rev = ((uint32_t)(ry >> 63)) != qstrand ? 1u : 0u;
            o[k] = a;
        }
    }
}

// ------------------------------------------------ chainAnchors, general form
//
// One warp chains one anchor list with the reference's serial semantics
// (src/seed/anchor.cpp:360-430): for anchor i the 32 candidates j of a chunk
// are scored at once; every valid lane marks t[p[j]] = i before any lane
// tests t[j] (p[j] < j, so a mark only targets a candidate the serial scan
// reaches later, and marks from lanes past a break target candidates it
// never tests), improvements are the lanes whose total beats the
// running maximum (warp prefix max), and n_skip follows the closed form of
// the recurrence max(n + d, 0) over the chunk (prefix sum and prefix min).
// Unlike the batch chain kernel it takes per-anchor sequence ids, strands
// and spans.

struct ChainGen {
    int n;
    const uint32_t* ref;   // sorted pos_ref
    const uint32_t* qry;   // sorted pos_qry
    const uint32_t* span;  // sorted span
    const uint32_t* grp;   // rid_ref << 1 | is_rev
    int32_t* f;
    int32_t* p;
    int32_t* t;
    int32_t* chain;        // ascending indices of the best chain
    int32_t* res;          // [0] chain length, [1] best end, [2] best f
    int max_dist_x, max_dist_y, bw, max_skip, max_iter, min_cnt, min_score;
    float gap_pen, skip_pen;
    const float* lg2;      // log2f(i), i < n_lg2 (covers dd + 1)
};

__device__ __forceinline__ int32_t gen_score(const ChainGen& a, uint32_t ri, uint32_t qi, uint32_t gi, uint32_t rj,
                                             uint32_t qj, uint32_t gj, int32_t span_j)
{  // chainScoreSimple (src/seed/anchor.cpp:254-301)
    if (gi != gj) return INT32_MIN;
    const int32_t dq = (int32_t)qi - (int32_t)qj;
    if (dq <= 0 || dq > a.max_dist_x) return INT32_MIN;
    const int32_t dr = (int32_t)ri - (int32_t)rj;
    if (dr <= 0 || dr > a.max_dist_y) return INT32_MIN;
    const int32_t dd = dr > dq ? dr - dq : dq - dr;
    if (dd > a.bw) return INT32_MIN;
    const int32_t dg = dr < dq ? dr : dq;
    int32_t sc = span_j < dg ? span_j : dg;
    if (dd > 0 || dg > span_j) {
        const float lin = __fadd_rn(__fmul_rn(a.gap_pen, (float)dd), __fmul_rn(a.skip_pen, (float)dg));
        const float lg = dd >= 1 ? a.lg2[dd + 1] : 0.0f;
        sc -= __float2int_rz(__fadd_rn(lin, __fmul_rn(0.5f, lg)));
    }
    return sc;
}

__device__ __forceinline__ int32_t wincl_max(int32_t v)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v = max(v, u);
    }
    return v;
}

__device__ __forceinline__ int32_t wincl_sum(int32_t v)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    return v;
}

__device__ __forceinline__ int32_t wincl_min(int32_t v)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v = min(v, u);
    }
    return v;
}

__global__ void __launch_bounds__(32) chain_general_kernel(ChainGen a)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x;
    const int n = a.n;
    for (int i = lane; i < n; i += 32) a.t[i] = -1;
    __syncwarp();
    int st = 0, best = -1;
    int32_t best_f = 0;
    for (int i = 0; i < n; ++i) {
        const uint32_t ri = a.ref[i], qi = a.qry[i], gi = a.grp[i];
        // window start: skip anchors of another sequence / strand or further
        // than max_dist_x on the reference (src/seed/anchor.cpp:375-385)
        while (st < i && (a.grp[st] != gi || (int32_t)(ri - a.ref[st]) > a.max_dist_x)) ++st;
        const int it0 = (int64_t)i - st > (int64_t)a.max_iter ? (int)((int64_t)i - a.max_iter) : st;
        int32_t max_f = (int32_t)a.span[i];
        int max_j = -1, n_skip = 0;
        for (int jb = i - 1; jb >= it0; jb -= 32) {
            const int j = jb - lane;
            int32_t sc = INT32_MIN;
            if (j >= it0) sc = gen_score(a, ri, qi, gi, a.ref[j], a.qry[j], a.grp[j], (int32_t)a.span[j]);
            const bool valid = sc != INT32_MIN;
            int32_t fj = 0, pj = -1;
            if (valid) fj = a.f[j], pj = a.p[j];
            if (valid && pj >= 0) a.t[pj] = i;
            __syncwarp();
            const bool marked = valid && a.t[j] == i;
            const int32_t tot = fj + sc;
            const int32_t vmax = wincl_max(valid ? tot : INT32_MIN);
            int32_t prev = __shfl_up_sync(FULL, vmax, 1);
            if (lane == 0) prev = INT32_MIN;
            prev = max(prev, max_f);
            const bool rec = valid && tot > prev;
            const int d = rec ? -1 : (marked ? 1 : 0);
            const int S = wincl_sum(d);
            const int mS = wincl_min(S);
            const int X = S + max(n_skip, -mS);
            const unsigned brk = __ballot_sync(FULL, d == 1 && X > a.max_skip);
            unsigned recm = __ballot_sync(FULL, rec);
            if (brk) recm &= (1u << (__ffs(brk) - 1)) - 1u;
            if (recm) {
                const int L = 31 - __clz(recm);
                max_f = __shfl_sync(FULL, tot, L);
                max_j = __shfl_sync(FULL, j, L);
            }
            if (brk) break;
            n_skip = __shfl_sync(FULL, X, 31);
            __syncwarp();
        }
        if (lane == 0) a.f[i] = max_f, a.p[i] = max_j;
        __syncwarp();
        if (max_f > best_f) best_f = max_f, best = i;
    }
    if (lane == 0) {
        int len = 0;
        if (!(best_f < a.min_score || best < 0)) {
            for (int c = best; c >= 0; c = a.p[c]) ++len;
            if (len < a.min_cnt) len = 0;
            int k = len;
            if (len)
                for (int c = best; c >= 0; c = a.p[c]) a.chain[--k] = c;
        }
        a.res[0] = len, a.res[1] = best, a.res[2] = best_f;
    }
}

// Sort keys of chainAnchors' order (rid_ref, is_rev, pos_ref, pos_qry) with
// the input index as the last key; padding sorts last.
__global__ void chain_keys_kernel(const hg_anchor_t* in, int n, unsigned P, Key128* keys)
{
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < P; i += gridDim.x * blockDim.x) {
        Key128 k;
        if (i < (unsigned)n) {
            const hg_anchor_t a = in[i];
            k.hi = (unsigned long long)a.rid_ref << 33 | (unsigned long long)(a.is_rev ? 1u : 0u) << 32 | a.pos_ref;
            k.lo = (unsigned long long)a.pos_qry << 32 | i;
        } else {
            k.hi = k.lo = ~0ull;
        }
        keys[i] = k;
    }
}

__global__ void chain_gather_kernel(const hg_anchor_t* in, const Key128* keys, int n, hg_anchor_t* sorted,
                                    uint32_t* ref, uint32_t* qry, uint32_t* span, uint32_t* grp)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const hg_anchor_t a = in[(uint32_t)keys[i].lo];
        sorted[i] = a;
        ref[i] = a.pos_ref, qry[i] = a.pos_qry, span[i] = a.span;
        grp[i] = a.rid_ref << 1 | (a.is_rev ? 1u : 0u);
    }
}

// ------------------------------------------------ row projection

// Per op: query bases consumed, row columns produced, and whether the op
// copies query bases into the row (cigar.cpp:150-299).  Op codes: 0 M, 1 I,
// 2 D, 3 N, 4 S, 5 H, 6 P, 7 =, 8 X.
__host__ __device__ __forceinline__ void op_effect(uint32_t op, uint32_t len, int pad, uint32_t& qcons,
                                                   uint32_t& rcols, int& copies)
{
    qcons = rcols = 0;
    copies = 0;
    if (op == 5 || op == 6) return;
    if (op == 2 || op == 3) {
        rcols = len;
        return;
    }
    if (op == 1) {
        qcons = len;
        if (pad) rcols = len, copies = 1;
        return;
    }
    qcons = rcols = len, copies = 1;
}

__global__ void project_scan_kernel(const uint32_t* cig, int64_t n, int pad, unsigned long long* qoff,
                                    unsigned long long* roff)
{  // one CTA: exclusive scans of query bases and row columns over the ops
    __shared__ unsigned long long pq[1024], pr[1024];
    const int tid = threadIdx.x;
    const int64_t per = (n + 1023) / 1024;
    const int64_t i0 = min(tid * per, n), i1 = min(i0 + per, n);
    unsigned long long sq = 0, sr = 0;
    for (int64_t i = i0; i < i1; ++i) {
        uint32_t qc, rc;
        int cp;
        op_effect(cig[i] & 0xfu, cig[i] >> 4, pad, qc, rc, cp);
        sq += qc, sr += rc;
    }
    pq[tid] = sq, pr[tid] = sr;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const unsigned long long a = tid >= o ? pq[tid - o] : 0, b = tid >= o ? pr[tid - o] : 0;
        __syncthreads();
        pq[tid] += a, pr[tid] += b;
        __syncthreads();
    }
    unsigned long long rq = pq[tid] - sq, rr = pr[tid] - sr;
    for (int64_t i = i0; i < i1; ++i) {
        qoff[i] = rq, roff[i] = rr;
        uint32_t qc, rc;
        int cp;
        op_effect(cig[i] & 0xfu, cig[i] >> 4, pad, qc, rc, cp);
        rq += qc, rr += rc;
    }
    if (tid == 1023) qoff[n] = pq[1023], roff[n] = pr[1023];
}

__global__ void project_fill_kernel(const char* qry, const uint32_t* cig, int64_t n, int pad,
                                    const unsigned long long* qoff, const unsigned long long* roff, char* out)
{  // one warp per op
    const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = w; i < n; i += nw) {
        uint32_t qc, rc;
        int cp;
        op_effect(cig[i] & 0xfu, cig[i] >> 4, pad, qc, rc, cp);
        char* o = out + roff[i];
        const char* s = qry + qoff[i];
        for (uint32_t k = lane; k < rc; k += 32) o[k] = cp ? s[k] : '-';
    }
}

}  // namespace hg

using hg::set_error;
using hg::Workspace;

namespace {
int fail(int code, const std::string& msg) { return set_error(code, msg); }
}  // namespace

// ------------------------------------------------------------ C ABI

extern "C" int64_t hg_extract_minimizer(const char* seq, int64_t len, int k, int w, int non_canonical, uint64_t* xs,
                                        uint64_t* ys, int64_t cap, int64_t* needed)
{  // minimizer::extractMinimizer (src/seed/minimizer.cpp:103-177)
    if ((!seq && len > 0) || len < 0) return -fail(HG_ERR_ARG, "hg_extract_minimizer: null sequence");
    if (hg_device_count() <= 0) return -fail(HG_ERR_CUDA, "hg_extract_minimizer: no CUDA device");
    std::vector<uint64_t> x, y;
    const int r = hg::run_extract(k, w, non_canonical, seq, len, x, y);
    if (r) return -r;
    const int64_t m = (int64_t)x.size();
    if (needed) *needed = m;
    if (m > cap) return -fail(HG_ERR_CAPACITY, "hg_extract_minimizer: output capacity");
    std::copy(x.begin(), x.end(), xs);
    std::copy(y.begin(), y.end(), ys);
    return m;
}

extern "C" int64_t hg_ksw_extz2(int qlen, const uint8_t* query, int tlen, const uint8_t* target, int8_t m,
                                const int8_t* mat, int8_t q, int8_t e, int w, int zdrop, int end_bonus, int flag,
                                int32_t* ez_out, uint32_t* cigar, int64_t cap)
{  // ksw_extz2_sse (src/align/ksw2_extz2_sse.c:23-304)
    if (!ez_out || (qlen > 0 && !query) || (tlen > 0 && !target) || !mat || m <= 0 || m > 16)
        return -fail(HG_ERR_ARG, "hg_ksw_extz2: bad arguments");
    for (int i = 0; i < qlen; ++i)
        if (query[i] >= m) return -fail(HG_ERR_ARG, "hg_ksw_extz2: query symbol >= m");
    for (int i = 0; i < tlen; ++i)
        if (target[i] >= m) return -fail(HG_ERR_ARG, "hg_ksw_extz2: target symbol >= m");
    if (hg_device_count() <= 0) return -fail(HG_ERR_CUDA, "hg_ksw_extz2: no CUDA device");
    const int32_t init[10] = {0, 0, -1, -1, hg::kNegInf, -1, hg::kNegInf, -1, hg::kNegInf, 0};
    if (qlen <= 0 || tlen <= 0) {
        std::copy(init, init + 10, ez_out);
        return 0;
    }
    Workspace* ws = nullptr;
    int r = hg::workspace(&ws);
    if (r) return -r;
    cudaStream_t st = ws->st;
    const size_t scratch = hg_ksw_scratch_bytes(qlen, tlen, w, flag);
    const int ccap = qlen + tlen + 4;
    const size_t in_bytes = (size_t)qlen + tlen + (size_t)m * m;
    uint8_t *d_in = nullptr, *d_s = nullptr;
    uint32_t* d_c = nullptr;
    int32_t* d_r = nullptr;
    auto cu = [&](cudaError_t ce, const char* where) -> int64_t { return -(int64_t)hg::cuda_error(ce, where); };
    cudaError_t ce;
    if ((ce = hg::ws_dev(ws, 0, in_bytes + 64, &d_in)) != cudaSuccess) return cu(ce, "hg_ksw_extz2: scratch");
    if ((ce = hg::ws_dev(ws, 1, scratch + 256, &d_s)) != cudaSuccess) return cu(ce, "hg_ksw_extz2: scratch");
    if ((ce = hg::ws_dev(ws, 2, (size_t)ccap, &d_c)) != cudaSuccess) return cu(ce, "hg_ksw_extz2: scratch");
    if ((ce = hg::ws_dev(ws, 3, 16, &d_r)) != cudaSuccess) return cu(ce, "hg_ksw_extz2: scratch");
    uint8_t* h = nullptr;
    if ((ce = ws->host(in_bytes + 64 + 4 * (size_t)ccap, reinterpret_cast<void**>(&h))) != cudaSuccess)
        return cu(ce, "hg_ksw_extz2: staging");
    std::memcpy(h, query, (size_t)qlen);
    std::memcpy(h + qlen, target, (size_t)tlen);
    std::memcpy(h + qlen + tlen, mat, (size_t)m * m);
    if ((ce = cudaMemcpyAsync(d_in, h, in_bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return cu(ce, "hg_ksw_extz2: upload");
    if ((ce = hg_launch_ksw_single(qlen, d_in, tlen, d_in + qlen, m, reinterpret_cast<const int8_t*>(d_in + qlen + tlen),
                                   q, e, w, zdrop, end_bonus, flag, d_s, d_c, ccap, d_r, st)) != cudaSuccess)
        return cu(ce, "hg_ksw_extz2: launch");
    int32_t* hres = reinterpret_cast<int32_t*>(h + (in_bytes + 15) / 16 * 16);
    uint32_t* hcig = reinterpret_cast<uint32_t*>(hres + 12);
    if ((ce = cudaMemcpyAsync(hres, d_r, 11 * sizeof(int32_t), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return cu(ce, "hg_ksw_extz2: read-back");
    if ((ce = cudaStreamSynchronize(st)) != cudaSuccess) return cu(ce, "hg_ksw_extz2: run");
    std::copy(hres, hres + 10, ez_out);
    const int nc = hres[10];
    if (nc > ccap) return -fail(HG_ERR_CAPACITY, "hg_ksw_extz2: internal CIGAR overflow");
    if (nc > cap) return -fail(HG_ERR_CAPACITY, "hg_ksw_extz2: CIGAR capacity");
    if (nc) {
        if ((ce = cudaMemcpyAsync(hcig, d_c, 4 * (size_t)nc, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (ce = cudaStreamSynchronize(st)) != cudaSuccess)
            return cu(ce, "hg_ksw_extz2: CIGAR read-back");
        std::memcpy(cigar, hcig, 4 * (size_t)nc);
    }
    return nc;
}

// ---- collect_anchors

struct hg_hits {
    int device = 0;
    int64_t n_ref = 0;
    uint32_t n_ent = 0;
    uint64_t occ_thr = 0;
    hg::DevBuf<ulonglong2> tab;
    hg::DevBuf<uint2> ent;
    hg::DevBuf<unsigned long long> rx, ry;
    uint32_t mask = 0;
};

extern "C" int hg_hits_create(const uint64_t* ref_x, const uint64_t* ref_y, int64_t n, const hg_params_t* params,
                              hg_hits_t** out)
{
    if (!out || n < 0 || (n > 0 && (!ref_x || !ref_y)) || n > 0x7fffffffLL)
        return fail(HG_ERR_ARG, "hg_hits_create: bad arguments");
    if (hg_device_count() <= 0) return fail(HG_ERR_CUDA, "hg_hits_create: no CUDA device");
    hg_params_t prm;
    if (params) prm = *params;
    else hg_default_params(&prm);
    auto h = std::make_unique<hg_hits>();
    HG_CUDA(cudaGetDevice(&h->device));
    h->n_ref = n;
    // MinimizerHit's operator< (include/seed.h:67-74): hash, rid, pos, strand;
    // stable, so equal keys keep their input order
    std::vector<uint32_t> idx((size_t)n);
    std::iota(idx.begin(), idx.end(), 0u);
    auto key = [&](uint32_t i, uint64_t& hh, uint32_t& rid, uint32_t& pos, uint32_t& strand) {
        hh = ref_x[i] >> 8, rid = (uint32_t)(ref_y[i] >> 32) & 0x7fffffffu, pos = (uint32_t)ref_y[i];
        strand = (uint32_t)(ref_y[i] >> 63);
    };
    std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) {
        uint64_t ha, hb;
        uint32_t ra, rb, pa, pb, sa, sb;
        key(a, ha, ra, pa, sa);
        key(b, hb, rb, pb, sb);
        if (ha != hb) return ha < hb;
        if (ra != rb) return ra < rb;
        if (pa != pb) return pa < pb;
        return sa < sb;
    });
    std::vector<unsigned long long> sx((size_t)n), sy((size_t)n);
    std::vector<uint64_t> ekey, occs;
    std::vector<uint32_t> est;
    for (int64_t i = 0; i < n; ++i) {
        sx[i] = ref_x[idx[i]], sy[i] = ref_y[idx[i]];
        const uint64_t hh = sx[i] >> 8;
        if (i == 0 || hh != ekey.back()) ekey.push_back(hh), est.push_back((uint32_t)i), occs.push_back(0);
        occs.back()++;
    }
    h->occ_thr = hg::occ_threshold(occs, prm);
    h->n_ent = (uint32_t)ekey.size();
    uint32_t tsize = 16;
    while (tsize < 2 * ekey.size() + 16) tsize <<= 1;
    std::vector<ulonglong2> tab(tsize);
    for (auto& t : tab) t.x = hg::kNoHash, t.y = 0;
    std::vector<uint2> ent(ekey.size());
    for (size_t e = 0; e < ekey.size(); ++e) {
        uint32_t s = (uint32_t)ekey[e] & (tsize - 1);
        while (tab[s].x != hg::kNoHash) s = (s + 1) & (tsize - 1);
        tab[s].x = ekey[e], tab[s].y = e;
        ent[e].x = est[e];
        ent[e].y = (uint32_t)occs[e] | (occs[e] > h->occ_thr ? 0x80000000u : 0u);
    }
    h->mask = tsize - 1;
    auto up = [&](auto& buf, const auto& v) -> cudaError_t {
        cudaError_t e = buf.alloc(std::max<size_t>(v.size(), 1));
        if (e != cudaSuccess || v.empty()) return e;
        return cudaMemcpy(buf.p, v.data(), sizeof(v[0]) * v.size(), cudaMemcpyHostToDevice);
    };
    cudaError_t e;
    if ((e = up(h->tab, tab)) != cudaSuccess || (e = up(h->ent, ent)) != cudaSuccess ||
        (e = up(h->rx, sx)) != cudaSuccess || (e = up(h->ry, sy)) != cudaSuccess)
        return hg::cuda_error(e, "hg_hits_create: upload");
    *out = h.release();
    return HG_OK;
}

extern "C" void hg_hits_destroy(hg_hits_t* h)
{
    if (!h) return;
    int cur = -1;
    cudaGetDevice(&cur);
    cudaSetDevice(h->device);
    delete h;
    if (cur >= 0) cudaSetDevice(cur);
}

extern "C" int64_t hg_collect_anchors(const hg_hits_t* h, const uint64_t* qry_x, const uint64_t* qry_y, int64_t n_qry,
                                      const hg_params_t* params, hg_anchor_t* out, int64_t cap, int64_t* needed)
{  // minimizer::collect_anchors (src/seed/minimizer.cpp:220-356)
    if (!h || n_qry < 0 || (n_qry > 0 && (!qry_x || !qry_y)) || cap < 0 || (cap > 0 && !out))
        return -fail(HG_ERR_ARG, "hg_collect_anchors: bad arguments");
    if (needed) *needed = 0;
    if (h->n_ref == 0 || n_qry == 0) return 0;
    hg_params_t prm;
    if (params) prm = *params;
    else hg_default_params(&prm);
    cudaSetDevice(h->device);
    Workspace* ws = nullptr;
    int r = hg::workspace(&ws);
    if (r) return -r;
    cudaStream_t st = ws->st;
    unsigned long long *d_q = nullptr, *d_cnt = nullptr, *d_off = nullptr;
    uint32_t *d_ent = nullptr, *d_occ = nullptr;
    hg_anchor_t* d_out = nullptr;
    unsigned long long* hbuf = nullptr;
    const size_t nq = (size_t)n_qry;
    auto cu = [&](cudaError_t ce, const char* where) -> int64_t { return -(int64_t)hg::cuda_error(ce, where); };
    cudaError_t ce;
    if ((ce = hg::ws_dev(ws, 0, 2 * nq, &d_q)) != cudaSuccess || (ce = hg::ws_dev(ws, 1, nq, &d_ent)) != cudaSuccess ||
        (ce = hg::ws_dev(ws, 2, h->n_ent, &d_occ)) != cudaSuccess ||
        (ce = hg::ws_dev(ws, 3, nq, &d_cnt)) != cudaSuccess || (ce = hg::ws_dev(ws, 4, nq + 1, &d_off)) != cudaSuccess)
        return cu(ce, "hg_collect_anchors: scratch");
    if ((ce = ws->host(16 * nq + 64, reinterpret_cast<void**>(&hbuf))) != cudaSuccess)
        return cu(ce, "hg_collect_anchors: staging");
    std::memcpy(hbuf, qry_x, 8 * nq);
    std::memcpy(hbuf + nq, qry_y, 8 * nq);
    hg::HitsDev hd{h->tab.p, h->mask, h->n_ent, h->ent.p, h->rx.p, h->ry.p};
    const int blocks = (int)std::min<int64_t>((n_qry + 255) / 256, 1184);
    if ((ce = cudaMemcpyAsync(d_q, hbuf, 16 * nq, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (ce = cudaMemsetAsync(d_occ, 0, 4 * (size_t)std::max<uint32_t>(h->n_ent, 1), st)) != cudaSuccess)
        return cu(ce, "hg_collect_anchors: upload");
    hg::collect_probe_kernel<<<blocks, 256, 0, st>>>(hd, d_q, n_qry, d_ent, d_occ);
    hg::collect_size_kernel<<<blocks, 256, 0, st>>>(hd, d_q + nq, n_qry, d_ent, d_occ, prm.q_occ_frac,
                                                    prm.sample_every_bp, d_cnt);
    hg::scan_counts_kernel<<<1, 1024, 0, st>>>(d_cnt, n_qry, d_off);
    unsigned long long* htot = hbuf + 2 * nq;
    if ((ce = cudaGetLastError()) != cudaSuccess ||
        (ce = cudaMemcpyAsync(htot, d_off + nq, 8, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (ce = cudaStreamSynchronize(st)) != cudaSuccess)
        return cu(ce, "hg_collect_anchors: count pass");
    const int64_t total = (int64_t)*htot;
    if (needed) *needed = total;
    if (total > cap) return -fail(HG_ERR_CAPACITY, "hg_collect_anchors: output capacity");
    if (total == 0) return 0;
    if ((ce = hg::ws_dev(ws, 5, (size_t)total, &d_out)) != cudaSuccess) return cu(ce, "hg_collect_anchors: output");
    hg::collect_emit_kernel<<<blocks, 256, 0, st>>>(hd, d_q, d_q + nq, n_qry, d_ent, d_cnt, d_off, d_out);
    hg_anchor_t* hout = nullptr;
    if ((ce = cudaGetLastError()) != cudaSuccess ||
        (ce = ws->host(sizeof(hg_anchor_t) * (size_t)total, reinterpret_cast<void**>(&hout))) != cudaSuccess ||
        (ce = cudaMemcpyAsync(hout, d_out, sizeof(hg_anchor_t) * (size_t)total, cudaMemcpyDeviceToHost, st)) !=
            cudaSuccess ||
        (ce = cudaStreamSynchronize(st)) != cudaSuccess)
        return cu(ce, "hg_collect_anchors: emit");
    std::memcpy(out, hout, sizeof(hg_anchor_t) * (size_t)total);
    return total;
}

// ---- chainAnchors

extern "C" int64_t hg_chain_anchors(hg_anchor_t* anchors, int64_t n, const hg_params_t* params, int64_t* chain,
                                    int64_t cap, int32_t* f, int64_t* p)
{  // anchor::chainAnchors (src/seed/anchor.cpp:332-461)
    if (n < 0 || n > (1LL << 30) || (n > 0 && !anchors) || cap < 0 || (cap > 0 && !chain))
        return -fail(HG_ERR_ARG, "hg_chain_anchors: bad arguments");
    if (n == 0) return 0;
    for (int64_t i = 0; i < n; ++i)
        if (anchors[i].rid_ref >= 0x80000000u) return -fail(HG_ERR_ARG, "hg_chain_anchors: rid_ref >= 2^31");
    hg_params_t prm;
    if (params) prm = *params;
    else hg_default_params(&prm);
    if (hg_device_count() <= 0) return -fail(HG_ERR_CUDA, "hg_chain_anchors: no CUDA device");
    Workspace* ws = nullptr;
    int r = hg::workspace(&ws);
    if (r) return -r;
    cudaStream_t st = ws->st;
    // log2f table over every dd + 1 a valid pair can reach: dd <= min(bw, max(max_dist_x, max_dist_y))
    const int64_t dd_max = std::max<int64_t>(0, std::min<int64_t>(prm.bw, std::max(prm.max_dist_x, prm.max_dist_y)));
    if (dd_max + 2 > (1 << 24)) return -fail(HG_ERR_ARG, "hg_chain_anchors: bw and max_dist above 2^24 are not supported");
    const int n_lg2 = (int)(dd_max + 2);
    const std::vector<float> lg = hg::log2_table(std::max(n_lg2, 2));
    const unsigned P = hg::sort_pad(n);
    const size_t nn = (size_t)n;
    hg_anchor_t *d_in = nullptr, *d_sorted = nullptr;
    hg::Key128* d_keys = nullptr;
    uint32_t* d_soa = nullptr;
    int32_t* d_dp = nullptr;
    float* d_lg = nullptr;
    auto cu = [&](cudaError_t ce, const char* where) -> int64_t { return -(int64_t)hg::cuda_error(ce, where); };
    cudaError_t ce;
    if ((ce = hg::ws_dev(ws, 0, nn, &d_in)) != cudaSuccess || (ce = hg::ws_dev(ws, 1, nn, &d_sorted)) != cudaSuccess ||
        (ce = hg::ws_dev(ws, 2, P, &d_keys)) != cudaSuccess || (ce = hg::ws_dev(ws, 3, 4 * nn, &d_soa)) != cudaSuccess ||
        (ce = hg::ws_dev(ws, 4, 4 * nn + 8, &d_dp)) != cudaSuccess ||
        (ce = hg::ws_dev(ws, 5, lg.size(), &d_lg)) != cudaSuccess)
        return cu(ce, "hg_chain_anchors: scratch");
    // pinned staging: anchors in and out at 0, the log2f table, then f, p,
    // the result words and the chain
    const size_t off_lg = 32 * nn;
    const size_t off_dp = (off_lg + 4 * lg.size() + 15) / 16 * 16;
    uint8_t* h = nullptr;
    if ((ce = ws->host(off_dp + 4 * (3 * nn + 4), reinterpret_cast<void**>(&h))) != cudaSuccess)
        return cu(ce, "hg_chain_anchors: staging");
    std::memcpy(h, anchors, 32 * nn);
    std::memcpy(h + off_lg, lg.data(), 4 * lg.size());
    if ((ce = cudaMemcpyAsync(d_in, h, 32 * nn, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (ce = cudaMemcpyAsync(d_lg, h + off_lg, 4 * lg.size(), cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return cu(ce, "hg_chain_anchors: upload");
    const int blocks = (int)std::min<int64_t>((P + 255) / 256, 1184);
    hg::chain_keys_kernel<<<blocks, 256, 0, st>>>(d_in, (int)n, P, d_keys);
    if ((ce = hg::sort_keys(d_keys, P, st)) != cudaSuccess) return cu(ce, "hg_chain_anchors: sort");
    // device DP words: f [0, n), p [n, 2n), t [2n, 3n), chain [3n, 4n), result [4n, 4n + 3)
    hg::ChainGen a{};
    a.n = (int)n;
    a.ref = d_soa, a.qry = d_soa + nn, a.span = d_soa + 2 * nn, a.grp = d_soa + 3 * nn;
    a.f = d_dp, a.p = d_dp + nn, a.t = d_dp + 2 * nn, a.chain = d_dp + 3 * nn, a.res = d_dp + 4 * nn;
    a.max_dist_x = prm.max_dist_x, a.max_dist_y = prm.max_dist_y, a.bw = prm.bw, a.max_skip = prm.max_skip;
    a.max_iter = prm.max_iter, a.min_cnt = prm.min_cnt, a.min_score = prm.min_score;
    a.gap_pen = prm.gap_penalty, a.skip_pen = prm.skip_penalty, a.lg2 = d_lg;
    hg::chain_gather_kernel<<<blocks, 256, 0, st>>>(d_in, d_keys, (int)n, d_sorted, d_soa, d_soa + nn,
                                                    d_soa + 2 * nn, d_soa + 3 * nn);
    hg::chain_general_kernel<<<1, 32, 0, st>>>(a);
    int32_t* hdp = reinterpret_cast<int32_t*>(h + off_dp);  // f, p, then the 3 result words, then the chain
    if ((ce = cudaGetLastError()) != cudaSuccess ||
        (ce = cudaMemcpyAsync(h, d_sorted, 32 * nn, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (ce = cudaMemcpyAsync(hdp, d_dp, 4 * (2 * nn), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (ce = cudaMemcpyAsync(hdp + 2 * nn, d_dp + 4 * nn, 12, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (ce = cudaStreamSynchronize(st)) != cudaSuccess)
        return cu(ce, "hg_chain_anchors: run");
    std::memcpy(anchors, h, 32 * nn);
    if (f) std::memcpy(f, hdp, 4 * nn);
    if (p)
        for (size_t i = 0; i < nn; ++i) p[i] = hdp[nn + i];
    const int32_t len = hdp[2 * nn];
    if (len > cap) return -fail(HG_ERR_CAPACITY, "hg_chain_anchors: chain capacity");
    if (len > 0) {
        int32_t* hc = hdp + 2 * nn + 4;
        if ((ce = cudaMemcpyAsync(hc, d_dp + 3 * nn, 4 * (size_t)len, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (ce = cudaStreamSynchronize(st)) != cudaSuccess)
            return cu(ce, "hg_chain_anchors: chain read-back");
        for (int32_t i = 0; i < len; ++i) chain[i] = hc[i];
    }
    return len;
}

// ---- row projection

extern "C" int64_t hg_project_row(const char* qry, int64_t qlen, const uint32_t* cigar, int64_t n_cigar, int pad,
                                  char* out, int64_t cap)
{  // cigar::delQueryToRefByCigar / padQueryToRefByCigar (src/align/cigar.cpp:150-299)
    if (qlen < 0 || (qlen > 0 && !qry) || n_cigar < 0 || (n_cigar > 0 && !cigar) || cap < 0 || (cap > 0 && !out))
        return -fail(HG_ERR_ARG, "hg_project_row: bad arguments");
    if (n_cigar == 0) {  // the reference returns the query unchanged
        if (qlen > cap) return -fail(HG_ERR_CAPACITY, "hg_project_row: output capacity");
        std::memcpy(out, qry, (size_t)qlen);
        return qlen;
    }
    // the sizes are checked on the host (n_cigar words the caller already holds)
    uint64_t qc_tot = 0, rc_tot = 0;
    for (int64_t i = 0; i < n_cigar; ++i) {
        const uint32_t op = cigar[i] & 0xfu;
        if (op > 8) return -fail(HG_ERR_ARG, "hg_project_row: unknown CIGAR op code");
        uint32_t qc, rc;
        int cp;
        hg::op_effect(op, cigar[i] >> 4, pad, qc, rc, cp);
        qc_tot += qc, rc_tot += rc;
    }
    if (qc_tot != (uint64_t)qlen)
        return -fail(HG_ERR_ARG, "hg_project_row: the CIGAR does not consume the query exactly");
    if ((int64_t)rc_tot > cap) return -fail(HG_ERR_CAPACITY, "hg_project_row: output capacity");
    if (hg_device_count() <= 0) return -fail(HG_ERR_CUDA, "hg_project_row: no CUDA device");
    Workspace* ws = nullptr;
    int r = hg::workspace(&ws);
    if (r) return -r;
    cudaStream_t st = ws->st;
    const size_t nc = (size_t)n_cigar;
    char *d_q = nullptr, *d_o = nullptr;
    uint32_t* d_c = nullptr;
    unsigned long long* d_off = nullptr;
    auto cu = [&](cudaError_t ce, const char* where) -> int64_t { return -(int64_t)hg::cuda_error(ce, where); };
    cudaError_t ce;
    if ((ce = hg::ws_dev(ws, 0, (size_t)qlen + 16, &d_q)) != cudaSuccess ||
        (ce = hg::ws_dev(ws, 1, rc_tot + 16, &d_o)) != cudaSuccess || (ce = hg::ws_dev(ws, 2, nc, &d_c)) != cudaSuccess ||
        (ce = hg::ws_dev(ws, 3, 2 * (nc + 1), &d_off)) != cudaSuccess)
        return cu(ce, "hg_project_row: scratch");
    uint8_t* h = nullptr;
    const size_t cbytes = 4 * nc;
    if ((ce = ws->host((size_t)qlen + cbytes + rc_tot + 64, reinterpret_cast<void**>(&h))) != cudaSuccess)
        return cu(ce, "hg_project_row: staging");
    std::memcpy(h, cigar, cbytes);
    std::memcpy(h + cbytes, qry, (size_t)qlen);
    if ((ce = cudaMemcpyAsync(d_c, h, cbytes, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (qlen && (ce = cudaMemcpyAsync(d_q, h + cbytes, (size_t)qlen, cudaMemcpyHostToDevice, st)) != cudaSuccess))
        return cu(ce, "hg_project_row: upload");
    hg::project_scan_kernel<<<1, 1024, 0, st>>>(d_c, n_cigar, pad, d_off, d_off + nc + 1);
    const int blocks = (int)std::min<int64_t>((n_cigar + 7) / 8, 1184);
    hg::project_fill_kernel<<<blocks, 256, 0, st>>>(d_q, d_c, n_cigar, pad, d_off, d_off + nc + 1, d_o);
    char* ho = reinterpret_cast<char*>(h + cbytes + (size_t)qlen);
    if ((ce = cudaGetLastError()) != cudaSuccess ||
        (rc_tot && (ce = cudaMemcpyAsync(ho, d_o, rc_tot, cudaMemcpyDeviceToHost, st)) != cudaSuccess) ||
        (ce = cudaStreamSynchronize(st)) != cudaSuccess)
        return cu(ce, "hg_project_row: run");
    std::memcpy(out, ho, rc_tot);
    return (int64_t)rc_tot;
}

// ---- SiteCount accumulation of caller rows

extern "C" int hg_count_rows(const char* rows, int64_t n_rows, int64_t L, int64_t row_stride, uint32_t* counts7,
                             int accumulate)
{  // consensus::processBatchParallelWithLocals (src/consensus/consensus.cpp:304-411)
    if (n_rows < 0 || L <= 0 || L > 0x7fffffffLL || row_stride < L || !counts7 || (n_rows > 0 && !rows))
        return fail(HG_ERR_ARG, "hg_count_rows: bad arguments");
    if (hg_device_count() <= 0) return fail(HG_ERR_CUDA, "hg_count_rows: no CUDA device");
    hg::Workspace* ws = nullptr;
    int r = hg::workspace(&ws);
    if (r) return r;
    cudaStream_t st = ws->st;
    const size_t cw = 7 * (size_t)L;
    const int64_t dstride = (L + 15) / 16 * 16;
    // rows go up in chunks of at most 256 MB of padded rows
    const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(n_rows, (256LL << 20) / dstride));
    uint32_t* d_cnt = nullptr;
    uint8_t* d_rows = nullptr;
    HG_CUDA(hg::ws_dev(ws, 0, cw, &d_cnt));
    HG_CUDA(hg::ws_dev(ws, 1, (size_t)(chunk * dstride), &d_rows));
    uint8_t* h = nullptr;
    HG_CUDA(ws->host(4 * cw, reinterpret_cast<void**>(&h)));
    if (accumulate) {
        std::memcpy(h, counts7, 4 * cw);
        HG_CUDA(cudaMemcpyAsync(d_cnt, h, 4 * cw, cudaMemcpyHostToDevice, st));
    } else {
        HG_CUDA(cudaMemsetAsync(d_cnt, 0, 4 * cw, st));
    }
    for (int64_t r0 = 0; r0 < n_rows; r0 += chunk) {
        const int64_t m = std::min(chunk, n_rows - r0);
        // padding columns past L are never counted (the kernel stops at L), but
        // the kernel reads whole 8-byte words: clear them once per chunk
        HG_CUDA(cudaMemsetAsync(d_rows, 0, (size_t)(m * dstride), st));
        HG_CUDA(cudaMemcpy2DAsync(d_rows, (size_t)dstride, rows + r0 * row_stride, (size_t)row_stride, (size_t)L,
                                  (size_t)m, cudaMemcpyHostToDevice, st));
        HG_CUDA(hg_launch_count(d_rows, dstride, (int)m, (int)L, d_cnt, st));
        HG_CUDA(cudaStreamSynchronize(st));  // the next chunk reuses the row buffer
    }
    HG_CUDA(cudaMemcpyAsync(h, d_cnt, 4 * cw, cudaMemcpyDeviceToHost, st));
    HG_CUDA(cudaStreamSynchronize(st));
    std::memcpy(counts7, h, 4 * cw);
    return HG_OK;
}
