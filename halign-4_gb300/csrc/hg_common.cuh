// hg_common.cuh - shared device definitions for the GB300 align-to-center path.
//
// Layout conventions (all device buffers live in HBM, owned by an hg_index
// or an hg_ctx handle):
//   * queries: 2-bit packed, A=0 C=1 G=2 T=3, base i of a query at bits
//     2*(i%4) of byte i/4; every query starts on a 16-byte boundary and keeps
//     64 bytes of slack, so kernels read its bases as 8-byte words (two
//     adjacent words funnel-shifted into a register window).  Bytes that are
//     not A/C/G/T are kept losslessly as exception runs {start, len, byte}.
//   * the center: one DNA5 code per base (ScoreChar2Idx, include/align.h:72-89)
//     for the gap-fill DP, plus a minimizer hash table (see hg_index).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace hg {

constexpr uint64_t kNoHash = ~0ull;  // invalid k-mer marker (hashes are < 2^56)
constexpr uint32_t kEmptyKey = 0xffffffffu;
constexpr int32_t kNegInf = -0x40000000;  // KSW_NEG_INF (include/ksw2.h:6)

// KSW_EZ_* flags (include/ksw2.h:8-18)
constexpr int kEzScoreOnly = 0x01, kEzRight = 0x02, kEzGenericSc = 0x04, kEzApproxMax = 0x08,
              kEzApproxDrop = 0x10, kEzExtzOnly = 0x40, kEzRevCigar = 0x80;

// Status bits reported per query / per call.
enum : uint32_t {
    kStOk = 0,
    kStArenaOverflow = 1u << 0,   // a dynamic arena was too small; retried by the host
    kStPartialCigar = 1u << 1,    // chainless global alignment stopped at the band edge
    kStBadInput = 1u << 2,
    kStCigarOverflow = 1u << 3,
    kStLengthMismatch = 1u << 4,
};

// splitmix64 (src/seed/minimizer.cpp:16-22)
__device__ __forceinline__ uint64_t splitmix64(uint64_t x)
{
    x += 0x9e3779b97f4a7c15ULL;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
    return x ^ (x >> 31);
}

// nt4_table (include/seed.h:157-190)
__host__ __device__ __forceinline__ uint8_t nt4_of(uint8_t c)
{
    switch (c) {
    case 'A': case 'a': return 0;
    case 'C': case 'c': return 1;
    case 'G': case 'g': return 2;
    case 'T': case 't': case 'U': case 'u': return 3;
    default: return 4;
    }
}

// ScoreChar2Idx (include/align.h:72-89)
__host__ __device__ __forceinline__ uint8_t dna5_of(uint8_t c)
{
    switch (c) {
    case 'A': case 'a': return 0;
    case 'C': case 'c': return 1;
    case 'G': case 'g': return 2;
    case 'T': case 't': return 3;
    default: return 4;
    }
}

// k_base_map (include/consensus.h:126-145): A C G T U N(default) gap
__host__ __device__ __forceinline__ uint32_t site_of(uint8_t c)
{
    switch (c) {
    case 'A': case 'a': return 0;
    case 'C': case 'c': return 1;
    case 'G': case 'g': return 2;
    case 'T': case 't': return 3;
    case 'U': case 'u': return 4;
    case '-': case '.': return 6;
    default: return 5;
    }
}

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

template <typename T>
__device__ __forceinline__ T warp_incl_sum(T v)
{
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T n = __shfl_up_sync(0xffffffffu, v, o);
        if ((int)lane_id() >= o) v += n;
    }
    return v;
}

__device__ __forceinline__ int warp_incl_max(int v)
{
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int n = __shfl_up_sync(0xffffffffu, v, o);
        if ((int)lane_id() >= o) v = max(v, n);
    }
    return v;
}

__device__ __forceinline__ int warp_incl_min(int v)
{
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int n = __shfl_up_sync(0xffffffffu, v, o);
        if ((int)lane_id() >= o) v = min(v, n);
    }
    return v;
}

// Block-wide exclusive sum for blockDim.x <= 1024 (multiple of 32).
// `scratch` needs 33 ints.  Returns the exclusive prefix; *total gets the sum.
__device__ __forceinline__ int block_excl_sum(int v, int* scratch, int* total)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int inc = warp_incl_sum(v);
    if (lane == 31) scratch[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        int s = lane < nw ? scratch[lane] : 0;
        const int si = warp_incl_sum(s);
        if (lane < nw) scratch[lane] = si - s;
        if (lane == 31) scratch[32] = si;
    }
    __syncthreads();
    const int r = scratch[wid] + inc - v;
    *total = scratch[32];
    __syncthreads();
    return r;
}

// One byte lane of ksw_extz2_sse's inner loop as compiled for plain SSE2
// (src/align/ksw2_extz2_sse.c:26-47, 150-223): 8-bit wrapping add/sub,
// unsigned max/min, signed compares.  mode: 0 score-only, 1 left-aligned
// gaps, 2 right-aligned gaps (KSW_EZ_RIGHT).
struct LaneOut {
    uint8_t u, v, x, y, d;
};

__device__ __forceinline__ int8_t s8(uint32_t v) { return (int8_t)(uint8_t)v; }

__device__ __forceinline__ LaneOut ksw_lane(uint32_t s, uint32_t xt1, uint32_t vt1, uint32_t ut, uint32_t yt,
                                           uint32_t qe2, uint32_t max_sc, uint32_t q, int mode)
{
    uint32_t z = (s + qe2) & 0xffu;
    uint32_t a = (xt1 + vt1) & 0xffu;
    uint32_t b = (yt + ut) & 0xffu;
    uint32_t d = 0;
    if (mode == 0) {
        z = s8(z) > 0 ? z : 0u;
        z = max(z, a);
    } else if (mode == 1) {
        d = s8(a) > s8(z) ? 1u : 0u;
        z = s8(z) > 0 ? z : 0u;
        z = max(z, a);
        if (s8(b) > s8(z)) d = 2u;
    } else {
        d = s8(z) > s8(a) ? 0u : 1u;
        z = s8(z) > 0 ? z : 0u;
        z = max(z, a);
        if (!(s8(z) > s8(b))) d = 2u;
    }
    z = max(z, b);
    z = min(z, max_sc);
    LaneOut o;
    o.u = (uint8_t)(z - vt1);
    o.v = (uint8_t)(z - ut);
    z = (z - q) & 0xffu;
    a = (a - z) & 0xffu;
    b = (b - z) & 0xffu;
    if (mode != 2) {
        o.x = s8(a) > 0 ? (uint8_t)a : 0;
        o.y = s8(b) > 0 ? (uint8_t)b : 0;
        if (mode == 1) {
            if (s8(a) > 0) d |= 0x08u;
            if (s8(b) > 0) d |= 0x10u;
        }
    } else {
        o.x = s8(a) < 0 ? 0 : (uint8_t)a;
        o.y = s8(b) < 0 ? 0 : (uint8_t)b;
        if (!(s8(a) < 0)) d |= 0x08u;
        if (!(s8(b) < 0)) d |= 0x10u;
    }
    o.d = (uint8_t)d;
    return o;
}

// auto_band (include/align.h:159-172): qlen is the reference length here,
// exactly as globalAlignKSW2 passes it (src/align/align.cpp:45).
__host__ __device__ __forceinline__ int auto_band(int qlen, int tlen)
{
    const int d = qlen > tlen ? qlen - tlen : tlen - qlen;
    const int mx = qlen > tlen ? qlen : tlen;
    if ((double)d / (double)mx > 0.5) return -1;
    return 200 + (int)(0.1 * (double)(qlen + tlen / 2));
}

// Base code of query position i from a packed query (+ exception runs).
__device__ __forceinline__ uint32_t packed_code(const uint8_t* packed, uint32_t i)
{
    return (packed[i >> 2] >> ((i & 3u) * 2u)) & 3u;
}

}  // namespace hg
