// kd_probe.cu -- the FP32 fused multiply-add rate of the current GPU, measured: the peak the
// mixed walk's force sums are held against (MEASURED_PEAKS-style figures exist for HBM and
// bf16 tensor work only).
//
// Every thread runs kChains independent multiply-add chains (enough to cover the pipe's
// latency at full occupancy) for `iters` rounds; the grid fills every SM.  The scalar kernel
// issues fma.rn.f32, the packed one fma.rn.f32x2 (two lanes per instruction), the form the
// walk's pair sums use.  Flops = 2 per multiply-add.
#include <cuda_runtime.h>

#include "../../include/kdnbody.h"
#include "kd_internal.cuh"

namespace kd {

void set_thread_error(const char *msg);

namespace {

constexpr int kChains = 8;
constexpr int kProbeThreads = 256;

__global__ __launch_bounds__(kProbeThreads) void k_fma_scalar(float *out, int iters, float s) {
    float a[kChains];
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = s * (float)(threadIdx.x + k);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < kChains; ++k) a[k] = fmaf(a[k], 0.999999f, 1e-7f);
    }
    float t = 0.f;
#pragma unroll
    for (int k = 0; k < kChains; ++k) t += a[k];
    if (t == 12345.678f) out[blockIdx.x] = t;  // keeps the chains alive; never true in practice
}

__global__ __launch_bounds__(kProbeThreads) void k_fma_packed(float *out, int iters, float s) {
    unsigned long long a[kChains];
    unsigned long long m, c;
    asm("mov.b64 %0, {%1, %2};" : "=l"(m) : "f"(0.999999f), "f"(0.999998f));
    asm("mov.b64 %0, {%1, %2};" : "=l"(c) : "f"(1e-7f), "f"(2e-7f));
#pragma unroll
    for (int k = 0; k < kChains; ++k) {
        const float v = s * (float)(threadIdx.x + k);
        asm("mov.b64 %0, {%1, %2};" : "=l"(a[k]) : "f"(v), "f"(v + 1.f));
    }
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < kChains; ++k)
            asm volatile("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(a[k]) : "l"(m), "l"(c));
    }
    float t = 0.f;
#pragma unroll
    for (int k = 0; k < kChains; ++k) {
        float x, y;
        asm("mov.b64 {%0, %1}, %2;" : "=f"(x), "=f"(y) : "l"(a[k]));
        t += x + y;
    }
    if (t == 12345.678f) out[blockIdx.x] = t;
}

}  // namespace
}  // namespace kd

extern "C" int kd_fp32_peak(int32_t device, double out[2]) {
    using namespace kd;
    if (!out) {
        set_thread_error("kd_fp32_peak: out is NULL");
        return KD_EINVAL;
    }
    cudaError_t e = cudaSetDevice(device);
    int blocks_per_sm = 0;
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_fma_scalar,
                                                          kProbeThreads, 0);
    const int blocks = sm_count() * (blocks_per_sm > 0 ? blocks_per_sm : 1);
    constexpr int kIters = 1 << 15;
    float *sink = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    if (e == cudaSuccess) e = cudaMalloc((void **)&sink, sizeof(float) * (size_t)blocks);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&ev[0]);
    if (e == cudaSuccess) e = cudaEventCreate(&ev[1]);
    const double fmas = (double)blocks * kProbeThreads * kChains * (double)kIters;
    for (int packed = 0; packed < 2 && e == cudaSuccess; ++packed) {
        float best = 1e30f;
        for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {  // first launch warms up
            cudaEventRecord(ev[0], st);
            if (packed)
                k_fma_packed<<<blocks, kProbeThreads, 0, st>>>(sink, kIters, 1e-3f);
            else
                k_fma_scalar<<<blocks, kProbeThreads, 0, st>>>(sink, kIters, 1e-3f);
            cudaEventRecord(ev[1], st);
            e = cudaEventSynchronize(ev[1]);
            float ms = 0.f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev[0], ev[1]);
            if (rep > 0 && ms < best) best = ms;
        }
        // flops: 2 per multiply-add, two multiply-adds per packed instruction
        out[packed] = (packed ? 2.0 : 1.0) * 2.0 * fmas / (best * 1e-3) / 1e12;
    }
    for (auto &x : ev)
        if (x) cudaEventDestroy(x);
    if (st) cudaStreamDestroy(st);
    if (sink) cudaFree(sink);
    if (e != cudaSuccess) {
        set_thread_error(cudaGetErrorString(e));
        return KD_ECUDA;
    }
    return KD_OK;
}
