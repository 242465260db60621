// Device peaks that bound the fused sequence kernels, measured on the GPU at
// hand: the FP32 fused-multiply-add (and so the instruction issue) rate and
// the shared-memory load bandwidth of all SMs.  The fused kernels keep their
// fields on chip, so these, not HBM, are the denominators of their roofline.
// Test and measurement hook (include/wavetorch_gb300_testing.h); the product
// kernels do not call it.
#include <cstdint>

#include "internal.cuh"
#include "../../include/wavetorch_gb300_testing.h"

namespace {

constexpr int PEAK_THREADS = 1024;
constexpr int PEAK_BLOCKS_PER_SM = 2;
constexpr int FFMA_CHAINS = 8;
constexpr int FFMA_UNROLL = 16;
constexpr int SMEM_FLOAT4 = 4096;          // 64 KB of float4 per block
constexpr int SMEM_UNROLL = 16;

// FFMA_CHAINS independent chains per thread: every instruction of the inner
// loop is an FFMA whose operands are ready (8 chains x 4-cycle latency per
// warp, 32 warps per SM), so the loop runs at the issue rate.  SM 0's first
// thread records the clock and the global timer around its loop.
__global__ void __launch_bounds__(PEAK_THREADS) peak_ffma_kernel(int iters, float a, float b,
                                                                 float* out,
                                                                 unsigned long long* clk) {
    float x[FFMA_CHAINS];
#pragma unroll
    for (int k = 0; k < FFMA_CHAINS; ++k) x[k] = (float)(threadIdx.x + k) * 1e-3f;
    long long c0 = clock64();
    uint64_t g0 = global_ns();
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < FFMA_UNROLL; ++u) {
#pragma unroll
            for (int k = 0; k < FFMA_CHAINS; ++k) x[k] = __fmaf_rn(x[k], a, b);
        }
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < FFMA_CHAINS; ++k) s += x[k];
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        clk[0] = (unsigned long long)(clock64() - c0);
        clk[1] = global_ns() - g0;
    }
}

// Conflict-free 16-byte shared-memory loads: a warp reads 512 contiguous
// bytes per instruction; four adds per load keep the values live.
__global__ void __launch_bounds__(PEAK_THREADS) peak_smem_kernel(int iters, float* out) {
    extern __shared__ float4 buf[];
    for (int i = threadIdx.x; i < SMEM_FLOAT4; i += blockDim.x)
        buf[i] = make_float4((float)i, 1.f, 2.f, 3.f);
    __syncthreads();
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    int idx = threadIdx.x;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < SMEM_UNROLL; ++u) {
            const float4 v = buf[(idx + u * 32) & (SMEM_FLOAT4 - 1)];
            acc.x += v.x; acc.y += v.y; acc.z += v.z; acc.w += v.w;
        }
        idx = (idx + SMEM_UNROLL * 32) & (SMEM_FLOAT4 - 1);
    }
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = acc.x + acc.y + acc.z + acc.w;
}

}  // namespace

extern "C" int wt_test_device_peaks_scratch_floats(size_t* n) {
    if (!n) return WT_ERR_INVALID;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return wt_cuda_status(e);
    *n = (size_t)sms * PEAK_BLOCKS_PER_SM * PEAK_THREADS + 4;
    return WT_OK;
}

extern "C" int wt_test_device_peaks(wt_device_peaks* out, float* scratch, size_t scratch_floats,
                                    wt_stream_t stream) {
    if (!out || !scratch) return WT_ERR_INVALID;
    size_t need = 0;
    int rc = wt_test_device_peaks_scratch_floats(&need);
    if (rc) return rc;
    if (scratch_floats < need) return WT_ERR_INVALID;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaStream_t st = (cudaStream_t)stream;
    const int blocks = sms * PEAK_BLOCKS_PER_SM;
    // the clock words sit after the per-thread outputs (8-byte aligned)
    size_t off = ((size_t)blocks * PEAK_THREADS + 1) & ~(size_t)1;
    unsigned long long* clk = reinterpret_cast<unsigned long long*>(scratch + off);
    cudaEvent_t e0, e1;
    cudaError_t e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e != cudaSuccess) return wt_cuda_status(e);
    auto timed = [&](auto launch, float* ms) -> cudaError_t {
        launch();                                   // warm-up
        cudaEventRecord(e0, st);
        launch();
        cudaEventRecord(e1, st);
        cudaError_t r = cudaEventSynchronize(e1);
        if (r == cudaSuccess) r = cudaEventElapsedTime(ms, e0, e1);
        return r == cudaSuccess ? cudaGetLastError() : r;
    };
    const int fiters = 4096;
    float ms_f = 0.f, ms_s = 0.f;
    e = timed([&] {
        peak_ffma_kernel<<<blocks, PEAK_THREADS, 0, st>>>(fiters, 0.999f, 1e-3f, scratch, clk);
    }, &ms_f);
    const size_t smem = SMEM_FLOAT4 * sizeof(float4);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(peak_smem_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
    const int siters = 2048;
    if (e == cudaSuccess)
        e = timed([&] { peak_smem_kernel<<<blocks, PEAK_THREADS, smem, st>>>(siters, scratch); },
                  &ms_s);
    unsigned long long hclk[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpy(hclk, clk, sizeof(hclk), cudaMemcpyDeviceToHost);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    wt_count_launches(4);
    if (e != cudaSuccess) return wt_cuda_status(e);
    const double threads = (double)blocks * PEAK_THREADS;
    const double ffma = threads * fiters * FFMA_UNROLL * FFMA_CHAINS;
    out->ffma_per_s = ffma / (ms_f * 1e-3);
    out->warp_inst_per_s = out->ffma_per_s / 32.0;
    out->smem_bytes_per_s = threads * siters * SMEM_UNROLL * sizeof(float4) / (ms_s * 1e-3);
    out->sm_mhz = hclk[1] ? (double)hclk[0] / (double)hclk[1] * 1e3 : 0.0;
    out->sm_count = sms;
    return WT_OK;
}
