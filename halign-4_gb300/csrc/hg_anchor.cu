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
constexpr int kSmemSort = 4096;

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
    unsigned long long* skey = reinterpret_cast<unsigned long long*>(dsm + kSmemEnt * 4);
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
        // each thread owns a contiguous run of hits so the scan keeps hit order
        const int per = (nm + kAnchorThreads - 1) / kAnchorThreads;
        const int i0 = min(tid * per, nm), i1 = min(i0 + per, nm);
        int my = 0;
        for (int i = i0; i < i1; ++i) {
            const uint32_t d = he[i];
            bool keep = !(ix.q_occ_frac > 0.0 && (double)cnt[d] > limit);
            if (keep && ix.ent_over[d]) keep = ix.sample_every != 0 && (hp[i] % ix.sample_every) == 0;
            if (keep) my += (int)ix.ent_count[d];
        }
        int A;
        const int ex = block_excl_sum(my, scan_s, &A);
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
            int o = ex;
            for (int i = i0; i < i1; ++i) {
                const uint32_t d = he[i];
                bool keep = !(ix.q_occ_frac > 0.0 && (double)cnt[d] > limit);
                if (keep && ix.ent_over[d]) keep = ix.sample_every != 0 && (hp[i] % ix.sample_every) == 0;
                if (!keep) continue;
                const uint32_t st = ix.ent_start[d], c = ix.ent_count[d];
                for (uint32_t j = 0; j < c; ++j, ++o) {
                    b.a_ref[base + o] = ix.cpos[st + j];
                    b.a_qry[base + o] = hp[i];
                }
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
            unsigned long long* key = (N <= kSmemSort) ? skey : b.a_tmp + 2 * base;
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

static constexpr size_t kAnchorSmem = hg::kSmemEnt * 4 + hg::kSmemSort * 8;

// Raises the dynamic shared-memory limit of the anchor kernel; called once
// per context before any launch or graph capture.
extern "C" cudaError_t hg_prepare_kernels(void)
{
    return cudaFuncSetAttribute(hg::anchor_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kAnchorSmem);
}

extern "C" cudaError_t hg_launch_anchor(const hg::IndexDev* ix, const hg::BatchDev* b, int grid, cudaStream_t st)
{
    hg::anchor_kernel<<<grid, hg::kAnchorThreads, kAnchorSmem, st>>>(*ix, *b);
    return cudaGetLastError();
}
