// hg_anchor.cu - K2: anchor collection against the resident center index.
//
// Restates minimizer::collect_anchors (src/seed/minimizer.cpp:220-356) for a
// single center (rid 0, forward strand on both sides, so is_rev is false and
// span = min(k, k) = k):
//   * a query hit whose hash occurs more than q_occ_frac * |query hits| times
//     among the query's hits is dropped (:280-315);
//   * a hash whose center occurrence count exceeds the -f/-U threshold is only
//     expanded at query positions divisible by sample_every_bp (:325-330);
//   * surviving hits expand over the center occurrences in ascending position.
// The anchors are then ordered as chainAnchors sorts them (rid_ref, is_rev,
// pos_ref, pos_qry; src/seed/anchor.cpp:343-349).  Keys are unique on this
// path.  Near-colinear queries produce them already sorted, so the sort runs
// only when a block-wide check finds an inversion.
//
// One CTA owns one query (persistent).  Query-side counts per center entry
// live in shared memory when the center has <= kSmemEnt distinct hashes,
// otherwise in a per-CTA slice of global memory; both are cleared after use.
#include "hg_batch.cuh"

namespace hg {

constexpr int kAnchorThreads = 256;
constexpr int kSmemEnt = 8192;

__device__ void bitonic_sort_u64(unsigned long long* key, int N)
{
    for (int kk = 2; kk <= N; kk <<= 1) {
        for (int j = kk >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < N; i += blockDim.x) {
                const int l = i ^ j;
                if (l > i) {
                    const unsigned long long a = key[i], c = key[l];
                    const bool asc = (i & kk) == 0;
                    if ((a > c) == asc) key[i] = c, key[l] = a;
                }
            }
            __syncthreads();
        }
    }
}

__global__ void __launch_bounds__(kAnchorThreads) anchor_kernel(IndexDev ix, BatchDev b)
{
    extern __shared__ __align__(16) unsigned char dsm[];
    __shared__ int scan_s[33];
    __shared__ int s_q, s_flag;
    __shared__ unsigned long long s_base;
    uint32_t* cnt = (ix.n_ent <= (uint32_t)kSmemEnt) ? reinterpret_cast<uint32_t*>(dsm)
                                                     : b.ent_cnt + (size_t)blockIdx.x * ix.n_ent;
    const int tid = threadIdx.x;
    if (ix.n_ent <= (uint32_t)kSmemEnt)
        for (int i = tid; i < (int)ix.n_ent; i += kAnchorThreads) cnt[i] = 0;
    __syncthreads();

    for (;;) {
        if (tid == 0) s_q = (int)atomicAdd(&b.queues[1], 1u);
        __syncthreads();
        const int qi = s_q;
        __syncthreads();
        if (qi >= b.n) break;
        const int q = b.order ? b.order[qi] : qi;
        const int nm = b.n_matched[q], nh = b.n_hits[q];
        const int64_t hb = b.hoff[q];
        const uint32_t* hp = b.hit_pos + hb;
        const uint32_t* he = b.hit_ent + hb;
        for (int i = tid; i < nm; i += kAnchorThreads) atomicAdd(&cnt[he[i]], 1u);
        __syncthreads();
        const double limit = ix.q_occ_frac > 0.0 ? ix.q_occ_frac * (double)nh : 0.0;
        // anchors of hit i: its center occurrences if the hit survives the filters
        auto n_out = [&](int i) -> int {
            const uint32_t d = he[i];
            const uint32_t my = ix.ent_meta[d].y;
            bool keep = !(ix.q_occ_frac > 0.0 && (double)cnt[d] > limit);
            if (keep && (my >> 31)) keep = ix.sample_every != 0 && (hp[i] % ix.sample_every) == 0;
            return keep ? (int)(my & 0x7fffffffu) : 0;
        };
        // total (coalesced: thread t takes hits t, t+256, ...); the counts of the
        // first kKeep chunks stay in registers for the emission pass
        constexpr int kKeep = 16;
        int keepn[kKeep];
        int my = 0;
#pragma unroll
        for (int r = 0; r < kKeep; ++r) {
            const int i = tid + r * kAnchorThreads;
            keepn[r] = i < nm ? n_out(i) : 0;
            my += keepn[r];
        }
        for (int i = tid + kKeep * kAnchorThreads; i < nm; i += kAnchorThreads) my += n_out(i);
        int A;
        block_excl_sum(my, scan_s, &A);
        if (tid == 0) {
            unsigned long long base = atomicAdd(b.a_cursor, (unsigned long long)A);
            if ((int64_t)(base + A) > b.acap) {
                atomicOr(&b.status[q], kStArenaOverflow);
                base = ~0ull;
            }
            s_base = base;
        }
        __syncthreads();
        const unsigned long long base = s_base;
        if (base != ~0ull) {
            // hits in chunks of 256, a block scan per chunk keeps hit order
            int carry = 0;
            for (int c0 = 0, r = 0; c0 < nm; c0 += kAnchorThreads, ++r) {
                const int i = c0 + tid;
                int k = 0;
                if (r < kKeep) {
#pragma unroll
                    for (int rr = 0; rr < kKeep; ++rr)
                        if (rr == r) k = keepn[rr];
                } else {
                    k = i < nm ? n_out(i) : 0;
                }
                int tot;
                const int ex = block_excl_sum(k, scan_s, &tot);
                if (k) {
                    const uint2 m = ix.ent_meta[he[i]];
                    const uint32_t qp = hp[i];
                    const bool once = (m.y & 0x7fffffffu) == 1u;
                    for (int j = 0; j < k; ++j) {
                        b.a_ref[base + carry + ex + j] = once ? m.x : ix.cpos[m.x + j];
                        b.a_qry[base + carry + ex + j] = qp;
                    }
                }
                carry += tot;
            }
        }
        __syncthreads();
        for (int i = tid; i < nm; i += kAnchorThreads) cnt[he[i]] = 0;
        if (tid == 0) s_flag = 0;
        __syncthreads();
        if (base == ~0ull) {
            if (tid == 0) b.a_n[q] = 0, b.a_base[q] = 0;
            continue;
        }
        // order check, sort only on an inversion
        uint32_t* ar = b.a_ref + base;
        uint32_t* aq = b.a_qry + base;
        for (int i = tid; i + 1 < A; i += kAnchorThreads) {
            const unsigned long long k0 = (unsigned long long)ar[i] << 32 | aq[i];
            const unsigned long long k1 = (unsigned long long)ar[i + 1] << 32 | aq[i + 1];
            if (k0 > k1) s_flag = 1;
        }
        __syncthreads();
        if (s_flag) {
            int N = 1;
            while (N < A) N <<= 1;
            unsigned long long* key = b.a_tmp + 2 * base;  // rare: only when an inversion exists
            for (int i = tid; i < N; i += kAnchorThreads)
                key[i] = i < A ? ((unsigned long long)ar[i] << 32 | aq[i]) : ~0ull;
            __syncthreads();
            bitonic_sort_u64(key, N);
            for (int i = tid; i < A; i += kAnchorThreads) {
                ar[i] = (uint32_t)(key[i] >> 32);
                aq[i] = (uint32_t)key[i];
            }
            __syncthreads();
        }
        if (tid == 0) b.a_base[q] = (int64_t)base, b.a_n[q] = A;
    }
}

}  // namespace hg

static constexpr size_t kAnchorSmem = hg::kSmemEnt * 4;  // per-entry counters (at most kSmemEnt entries)

// Raises the dynamic shared-memory limit of the anchor kernel; called once
// per context before any launch or graph capture.
extern "C" cudaError_t hg_prepare_kernels(void)
{
    return cudaFuncSetAttribute(hg::anchor_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kAnchorSmem);
}

extern "C" cudaError_t hg_launch_anchor(const hg::IndexDev* ix, const hg::BatchDev* b, int grid, cudaStream_t st)
{
    // counters for the center's entries live in shared memory when they fit
    const size_t smem = ix->n_ent <= (uint32_t)hg::kSmemEnt ? ((size_t)ix->n_ent * 4 + 15) & ~(size_t)15 : 16;
    hg::anchor_kernel<<<grid, hg::kAnchorThreads, smem, st>>>(*ix, *b);
    return cudaGetLastError();
}
