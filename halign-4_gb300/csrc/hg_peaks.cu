// hg_peaks.cu - integer and DPX throughput ceilings of this GPU, measured.
//
// The align-to-center path is integer work bound by instruction issue, so its
// roofline is an integer one, not the HBM copy rate or the tensor rate.  Each
// kernel below runs one instruction class in 8 independent chains per
// thread over a full grid (every SM, 2048 threads each) and reports element
// operations per second:
//   [0] int32 max(a + b, c) written as plain add and max, ops = 2
//   [1] DPX __viaddmax_s32 (max(a + b, c) in one instruction), ops = 2
//   [2] DPX __viaddmax_s16x2 (two 16-bit lanes), ops = 4
//   [3] DPX __vimax3_s16x2 (three-way max of two 16-bit lanes), ops = 4
//   [4] 64-bit multiply-add (splitmix64's multiplies), ops = 1
//   [5] integer-pipe warp instructions per second: [1]'s kernel issues one
//       instruction per step and chain
//   [6] __vsub2 (16x2 subtract, plus one xor per step), lane ops = 2
//   [7] __vcmpgts2 (16x2 signed compare to masks, plus one add), lane ops = 2
// The chains feed on values loaded at run time and the results are stored,
// so nothing folds away.  Measured on GB300 (ncu instruction counts): the
// compiler fuses [0]'s add and max into one integer-pipe instruction, so [0]
// and [1] run at the same rate, two warp instructions per clock per SM; the
// 16x2 forms issue at that rate too and do twice the element operations.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/halign_gb300.h"
#include "hg_internal.h"

namespace hg {

constexpr int kPeakChains = 8;
constexpr int kPeakIters = 4096;

__global__ void __launch_bounds__(256) peak_add_max(const int32_t* in, int32_t* out)
{
    int32_t x[kPeakChains];
    const int32_t k = in[threadIdx.x & 7];
#pragma unroll
    for (int i = 0; i < kPeakChains; ++i) x[i] = in[16 + i] + (int32_t)threadIdx.x;
    for (int it = 0; it < kPeakIters; ++it) {
#pragma unroll
        for (int i = 0; i < kPeakChains; ++i) x[i] = max(x[i] + k, x[(i + 1) & 7]);
    }
    int32_t s = 0;
#pragma unroll
    for (int i = 0; i < kPeakChains; ++i) s ^= x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void __launch_bounds__(256) peak_dpx_s32(const int32_t* in, int32_t* out)
{
    int32_t x[kPeakChains];
    const int32_t k = in[threadIdx.x & 7];
#pragma unroll
    for (int i = 0; i < kPeakChains; ++i) x[i] = in[16 + i] + (int32_t)threadIdx.x;
    for (int it = 0; it < kPeakIters; ++it) {
#pragma unroll
        for (int i = 0; i < kPeakChains; ++i) x[i] = __viaddmax_s32(x[i], k, x[(i + 1) & 7]);
    }
    int32_t s = 0;
#pragma unroll
    for (int i = 0; i < kPeakChains; ++i) s ^= x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void __launch_bounds__(256) peak_dpx_s16x2(const int32_t* in, int32_t* out)
{
    unsigned x[kPeakChains];
    const unsigned k = (unsigned)in[threadIdx.x & 7];
#pragma unroll
    for (int i = 0; i < kPeakChains; ++i) x[i] = (unsigned)in[16 + i] + threadIdx.x;
    for (int it = 0; it < kPeakIters; ++it) {
#pragma unroll
        for (int i = 0; i < kPeakChains; ++i) x[i] = __viaddmax_s16x2(x[i], k, x[(i + 1) & 7]);
    }
    unsigned s = 0;
#pragma unroll
    for (int i = 0; i < kPeakChains; ++i) s ^= x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = (int32_t)s;
}

__global__ void __launch_bounds__(256) peak_max3_s16x2(const int32_t* in, int32_t* out)
{
    unsigned x[kPeakChains];
    const unsigned k = (unsigned)in[threadIdx.x & 7];
#pragma unroll
    for (int i = 0; i < kPeakChains; ++i) x[i] = (unsigned)in[16 + i] + threadIdx.x;
    for (int it = 0; it < kPeakIters; ++it) {
#pragma unroll
        for (int i = 0; i < kPeakChains; ++i) x[i] = __vimax3_s16x2(x[i], k, x[(i + 1) & 7]);
    }
    unsigned s = 0;
#pragma unroll
    for (int i = 0; i < kPeakChains; ++i) s ^= x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = (int32_t)s;
}

__global__ void __launch_bounds__(256) peak_mul64(const int32_t* in, int32_t* out)
{
    unsigned long long x[kPeakChains];
    const unsigned long long m = 0xbf58476d1ce4e5b9ULL ^ (unsigned)in[threadIdx.x & 7];
#pragma unroll
    for (int i = 0; i < kPeakChains; ++i) x[i] = (unsigned long long)in[16 + i] + threadIdx.x;
    for (int it = 0; it < kPeakIters / 4; ++it) {
#pragma unroll
        for (int i = 0; i < kPeakChains; ++i) x[i] = x[i] * m + x[(i + 1) & 7];
    }
    unsigned long long s = 0;
#pragma unroll
    for (int i = 0; i < kPeakChains; ++i) s ^= x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = (int32_t)(s ^ (s >> 32));
}

// 16x2 SIMD add / subtract / compare without DPX: the other operations a
// packed DP cell needs.
__global__ void __launch_bounds__(256) peak_vsub2(const int32_t* in, int32_t* out)
{
    unsigned x[kPeakChains];
    const unsigned k = (unsigned)in[threadIdx.x & 7];
#pragma unroll
    for (int i = 0; i < kPeakChains; ++i) x[i] = (unsigned)in[16 + i] + threadIdx.x;
    for (int it = 0; it < kPeakIters; ++it) {
#pragma unroll
        for (int i = 0; i < kPeakChains; ++i) x[i] = __vsub2(x[(i + 1) & 7], x[i] ^ k);
    }
    unsigned s = 0;
#pragma unroll
    for (int i = 0; i < kPeakChains; ++i) s ^= x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = (int32_t)s;
}

__global__ void __launch_bounds__(256) peak_vcmpgt2(const int32_t* in, int32_t* out)
{
    unsigned x[kPeakChains];
    const unsigned k = (unsigned)in[threadIdx.x & 7];
#pragma unroll
    for (int i = 0; i < kPeakChains; ++i) x[i] = (unsigned)in[16 + i] + threadIdx.x;
    for (int it = 0; it < kPeakIters; ++it) {
#pragma unroll
        for (int i = 0; i < kPeakChains; ++i) x[i] = __vcmpgts2(x[(i + 1) & 7], x[i]) + k;
    }
    unsigned s = 0;
#pragma unroll
    for (int i = 0; i < kPeakChains; ++i) s ^= x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = (int32_t)s;
}

}  // namespace hg

extern "C" int hg_int_peaks(double* out, int n)
{
    if (!out || n <= 0) return hg::set_error(HG_ERR_ARG, "hg_int_peaks: bad arguments");
    int dev = 0, sms = 0;
    HG_CUDA(cudaGetDevice(&dev));
    HG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = sms * 8, threads = 256;  // 2048 threads per SM
    int32_t *d_in = nullptr, *d_out = nullptr;
    HG_CUDA(cudaMalloc(&d_in, 64 * sizeof(int32_t)));
    HG_CUDA(cudaMalloc(&d_out, (size_t)blocks * threads * sizeof(int32_t)));
    int32_t h[64];
    for (int i = 0; i < 64; ++i) h[i] = (i * 2654435761u) & 0x3ff;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int rc = HG_OK;
    auto cleanup = [&]() {
        cudaFree(d_in), cudaFree(d_out);
        cudaEventDestroy(e0), cudaEventDestroy(e1);
    };
    if (cudaMemcpy(d_in, h, sizeof(h), cudaMemcpyHostToDevice) != cudaSuccess) {
        cleanup();
        return hg::set_error(HG_ERR_CUDA, "hg_int_peaks: upload");
    }
    using K = void (*)(const int32_t*, int32_t*);
    const K kernels[7] = {hg::peak_add_max, hg::peak_dpx_s32, hg::peak_dpx_s16x2, hg::peak_max3_s16x2,
                          hg::peak_mul64, hg::peak_vsub2, hg::peak_vcmpgt2};
    // element operations per inner step per chain (the last two: one xor or
    // add each, counted as the 16x2 operation's two lanes only)
    const double ops[7] = {2.0, 2.0, 4.0, 4.0, 1.0, 2.0, 2.0};
    const double iters[7] = {hg::kPeakIters, hg::kPeakIters, hg::kPeakIters, hg::kPeakIters, hg::kPeakIters / 4,
                             hg::kPeakIters, hg::kPeakIters};
    double res[9] = {};
    const int slot[7] = {0, 1, 2, 3, 4, 6, 7};
    for (int k = 0; k < 7 && rc == HG_OK; ++k) {
        kernels[k]<<<blocks, threads>>>(d_in, d_out);  // warm-up
        float best = 1e30f;
        for (int rep = 0; rep < 3; ++rep) {
            cudaEventRecord(e0);
            kernels[k]<<<blocks, threads>>>(d_in, d_out);
            cudaEventRecord(e1);
            if (cudaEventSynchronize(e1) != cudaSuccess) {
                rc = hg::set_error(HG_ERR_CUDA, "hg_int_peaks: kernel");
                break;
            }
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            best = ms < best ? ms : best;
        }
        res[slot[k]] = (double)blocks * threads * hg::kPeakChains * iters[k] * ops[k] / (best * 1e-3);
    }
    res[5] = res[1] / 2.0 / 32.0;  // one instruction (two element ops) per lane and step, 32 lanes per warp
    cleanup();
    for (int i = 0; i < n && i < 8; ++i) out[i] = res[i];
    return rc;
}
