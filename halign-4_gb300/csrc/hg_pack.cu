// hg_pack.cu - device packing of ASCII queries into the input format of
// the batch path (the format hg_pack writes on the host): 2-bit codes
// A C G T = 0 1 2 3, four bases per byte (base j at bits 2j of byte j / 4),
// each query's bytes zero-padded to a multiple of 16; every byte that is
// not an upper-case A/C/G/T packs as 0 and is listed in an exception run
// (start, length, byte) of one repeated byte, in position order.
//
// Three launches per sub-batch, on the stream that then aligns it:
//   1. ascii_pack_kernel: one warp per query packs its bytes and counts the
//      exception runs (a run starts at an exception byte whose predecessor
//      is not the same exception byte);
//   2. exc_offsets_kernel: one CTA scans the counts into exc_off; when the
//      runs exceed the buffer it writes zero offsets (no query reads an
//      exception) and raises a flag the host turns into a capacity error;
//   3. ascii_runs_kernel: one warp per query with runs writes them; the
//      k-th run end pairs with the k-th run start.
#include "hg_batch.cuh"

namespace hg {

__device__ __forceinline__ uint32_t ascii_code(uint32_t ch)
{
    return ch == 'A' ? 0u : ch == 'C' ? 1u : ch == 'G' ? 2u : ch == 'T' ? 3u : 4u;
}

constexpr int kPackThreads = 256;

// One warp per query, 128 bases (32 output bytes) per step: lane l takes the
// 4 bases of output byte j = j0 + l from two 32-bit words of the query's
// bytes (one funnel shift for the query's alignment), packs them with the
// SWAR test of hg_pack (((c >> 1) ^ (c >> 2)) & 3 maps A C G T to 0 1 2 3;
// rebuilding the bytes from the codes confirms them) and only falls back to
// a byte loop where a word holds another byte or the query's end.  Run
// starts need the byte before each lane's first: the previous lane's last.
__global__ void __launch_bounds__(kPackThreads) ascii_pack_kernel(const uint8_t* ascii, const int64_t* aoff, int n,
                                                                  const int64_t* poff, uint8_t* packed, int32_t* nrun)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int64_t a0 = aoff[0];
    for (int q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < n; q += nw) {
        const uint8_t* s = ascii + (aoff[q] - a0);
        const int64_t len = aoff[q + 1] - aoff[q];
        uint8_t* out = packed + poff[q];
        const int64_t nb = (len + 3) / 4, pad = (nb + 15) / 16 * 16;
        // the query's bytes as aligned words (the buffer starts aligned and
        // keeps slack after the last query, so the word past a query's end is
        // readable; bytes past the end are masked below)
        const uint32_t mis = (uint32_t)((uintptr_t)s & 3u);
        const uint32_t* sw = reinterpret_cast<const uint32_t*>(s - mis);
        uint32_t carry = 0;  // the byte before this step's first base (0: none)
        int runs = 0;
        for (int64_t j0 = 0; j0 < pad; j0 += 32) {
            const int64_t j = j0 + lane;
            uint32_t v = 0;
            if (j < nb) {
                const uint32_t w0 = sw[j], w1 = sw[j + 1];
                v = __funnelshift_r(w0, w1, 8u * mis);
            }
            uint32_t prev = __shfl_up_sync(FULL, v, 1) >> 24;
            if (lane == 0) prev = carry;
            carry = __shfl_sync(FULL, v, 31) >> 24;
            const int64_t t0 = 4 * j;
            uint32_t byte = 0;
            if (j < nb) {
                const uint32_t cd = ((v >> 1) ^ (v >> 2)) & 0x03030303u;
                const uint32_t b0 = cd & 0x01010101u, b1 = (cd >> 1) & 0x01010101u;
                if (t0 + 4 <= len && 0x41414141u + 2u * b0 + 6u * b1 + 11u * (b0 & b1) == v) {
                    byte = (cd & 3u) | ((cd >> 6) & 0xCu) | ((cd >> 12) & 0x30u) | ((cd >> 18) & 0xC0u);
                } else {  // another byte, or the query's end, in this word
                    bool prevx = t0 > 0 && ascii_code(prev) > 3;
                    for (int u = 0; u < 4 && t0 + u < len; ++u) {
                        const uint32_t ch = (v >> (8 * u)) & 0xffu, c = ascii_code(ch);
                        if (c < 4) byte |= c << (2 * u);
                        else if (!prevx || ch != prev) ++runs;
                        prevx = c > 3, prev = ch;
                    }
                }
            }
            if (j < pad) out[j] = (uint8_t)byte;
        }
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) runs += __shfl_xor_sync(FULL, runs, d);
        if (lane == 0) nrun[q] = runs;
    }
}

// Exclusive scan of the run counts (one CTA); zero offsets and *flag = 1
// when the total exceeds cap.
__global__ void __launch_bounds__(1024) exc_offsets_kernel(const int32_t* nrun, int n, int64_t* off, int64_t cap,
                                                           int32_t* flag)
{
    __shared__ int64_t part[1024];
    const int tid = threadIdx.x;
    const int per = (n + 1023) / 1024;
    const int i0 = min(tid * per, n), i1 = min(i0 + per, n);
    int64_t s = 0;
    for (int i = i0; i < i1; ++i) s += nrun[i];
    part[tid] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const int64_t v = tid >= o ? part[tid - o] : 0;
        __syncthreads();
        part[tid] += v;
        __syncthreads();
    }
    const int64_t total = part[1023];
    const bool over = total > cap;
    int64_t run = part[tid] - s;
    for (int i = i0; i < i1; ++i) {
        off[i] = over ? 0 : run;
        run += nrun[i];
    }
    if (tid == 1023) off[n] = over ? 0 : total;
    if (tid == 0) *flag = over ? 1 : 0;
}

constexpr int kRunsWarps = kPackThreads / 32;

__global__ void __launch_bounds__(kPackThreads) ascii_runs_kernel(const uint8_t* ascii, const int64_t* aoff, int n,
                                                                  const int32_t* nrun, const int64_t* exc_off,
                                                                  int32_t* exc)
{
    __shared__ int64_t s_start[kRunsWarps][32];  // start positions of the current step's runs, by rank
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    const unsigned lt = (1u << lane) - 1u;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int64_t a0 = aoff[0];
    for (int q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < n; q += nw) {
        const int64_t e0 = exc_off[q], cnt = exc_off[q + 1] - e0;  // 0 after an overflow
        if (nrun[q] == 0 || cnt <= 0) continue;
        const uint8_t* s = ascii + (aoff[q] - a0);
        const int64_t len = aoff[q + 1] - aoff[q];
        int64_t starts = 0, ends = 0, open_start = 0;
        uint32_t carry_ch = 0;
        bool carry_x = false;
        for (int64_t c0 = 0; c0 < len; c0 += 32) {
            const int64_t t = c0 + lane;
            const bool in = t < len;
            const uint32_t ch = in ? s[t] : 0u;
            const bool x = in && ascii_code(ch) > 3;
            uint32_t pch = __shfl_up_sync(FULL, ch, 1);
            bool px = __shfl_up_sync(FULL, (int)x, 1) != 0;
            if (lane == 0) pch = carry_ch, px = carry_x;
            uint32_t nch = __shfl_down_sync(FULL, ch, 1);
            bool nx = __shfl_down_sync(FULL, (int)x, 1) != 0;
            if (lane == 31) {
                nch = t + 1 < len ? s[t + 1] : 0u;
                nx = t + 1 < len && ascii_code(nch) > 3;
            }
            const bool st = x && (!px || pch != ch);
            const bool en = x && (!nx || nch != ch);
            const unsigned sm = __ballot_sync(FULL, st), em = __ballot_sync(FULL, en);
            if (st) {
                const int r = __popc(sm & lt);
                s_start[wl][r] = t;
                if (starts + r < cnt) {
                    exc[(e0 + starts + r) * 3] = (int32_t)t;
                    exc[(e0 + starts + r) * 3 + 2] = (int32_t)ch;
                }
            }
            __syncwarp();
            if (en) {
                const int64_t r = ends + __popc(em & lt);  // pairs with start r
                const int64_t j = r - starts;               // < 0: the run opened in an earlier step
                const int64_t sp = j < 0 ? open_start : s_start[wl][j];
                if (r < cnt) exc[(e0 + r) * 3 + 1] = (int32_t)(t + 1 - sp);
            }
            const int ns = __popc(sm), ne = __popc(em);
            if (ns && starts + ns > ends + ne) open_start = s_start[wl][ns - 1];
            starts += ns, ends += ne;
            carry_ch = __shfl_sync(FULL, ch, 31);
            carry_x = __shfl_sync(FULL, (int)x, 31) != 0;
            __syncwarp();
        }
    }
}

}  // namespace hg

// ASCII bytes of queries [0, n) (query i at ascii + aoff[i] - aoff[0]) into
// packed + poff[i], exception runs into exc / exc_off (cap runs at most;
// *flag = 1 and zero offsets when they exceed it).  nrun: n int32 scratch.
extern "C" cudaError_t hg_launch_ascii_pack(const uint8_t* ascii, const int64_t* aoff, int n, const int64_t* poff,
                                            uint8_t* packed, int32_t* nrun, int64_t* exc_off, int32_t* exc, int64_t cap,
                                            int32_t* flag, int sms, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    const int warps = hg::kPackThreads / 32;
    const int grid = std::max(1, std::min((n + warps - 1) / warps, sms * 8));
    hg::ascii_pack_kernel<<<grid, hg::kPackThreads, 0, st>>>(ascii, aoff, n, poff, packed, nrun);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    hg::exc_offsets_kernel<<<1, 1024, 0, st>>>(nrun, n, exc_off, cap, flag);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    hg::ascii_runs_kernel<<<grid, hg::kPackThreads, 0, st>>>(ascii, aoff, n, nrun, exc_off, exc);
    return cudaGetLastError();
}
