// kd_noalloc.cu -- FP64 direct-sum accelerations for sampled bodies without allocating any
// device memory.
//
// Who needs this: a host that has committed the GPU's memory to its own simulation state
// (at tens of millions of bodies with checkpoints, a caller may reserve nearly all HBM up
// front and must not let a library take more), and a host that measures its accuracy
// inside its step loop, where the device-wide synchronisation of cudaMalloc/cudaFree would
// stall every other stream.  kd_direct_accel (which needs a context and allocates its
// buffers per call) serves everyone else.
//
// The scratch of the chunked sum -- one partial acceleration per (source chunk, sink) -- lives
// in a file-scope __device__ array of kNoAllocScratchDoubles doubles (1 MiB) that every GPU
// loading the library holds until exit.  Host code cannot use that array's name as a device
// address, so the first call on each device, with that device current, looks the address up
// with cudaGetSymbolAddress and keeps it for later calls.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/kdnbody.h"

namespace kd {
// records the message kd_last_error(NULL) reports for the calling thread (kd_api.cu)
void set_thread_error(const char *msg);
}  // namespace kd

namespace {

constexpr size_t kNoAllocScratchDoubles = size_t(1) << 17;  // 1 MiB
constexpr size_t kNoAllocMaxSinks = kNoAllocScratchDoubles / 3;
constexpr uint32_t kMinChunk = 4096;  // smallest source chunk worth one grid column
constexpr int kThreads = 128;
constexpr int kMaxDevices = 64;

__device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

std::mutex g_setup_mutex;
double *g_scratch_addr[kMaxDevices] = {};

// Every (sink, chunk) partial is written, so the scratch needs no clearing between calls.
__global__ __launch_bounds__(kThreads) void k_noalloc_partial(
    const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ z,
    const double *__restrict__ m, uint32_t n, const uint64_t *__restrict__ sinks, uint32_t ns,
    uint32_t chunk, double *partial) {
    __shared__ double sx[kThreads], sy[kThreads], sz[kThreads], sm[kThreads];
    const uint32_t k = blockIdx.x * kThreads + threadIdx.x;
    const uint32_t c = blockIdx.y;
    const uint32_t j0 = c * chunk;
    const uint32_t j1 = min(n, j0 + chunk);
    const uint64_t si = k < ns ? sinks[k] : 0ull;
    const bool valid = k < ns && si < n;  // an out-of-range sink reads nothing
    const uint32_t i = valid ? (uint32_t)si : 0u;
    const double px = valid ? x[i] : 0.0, py = valid ? y[i] : 0.0, pz = valid ? z[i] : 0.0;
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (uint32_t base = j0; base < j1; base += kThreads) {
        const uint32_t j = base + threadIdx.x;
        __syncthreads();
        if (j < j1) {
            sx[threadIdx.x] = x[j];
            sy[threadIdx.x] = y[j];
            sz[threadIdx.x] = z[j];
            sm[threadIdx.x] = m[j];
        }
        __syncthreads();
        const uint32_t cnt = min((uint32_t)kThreads, j1 - base);
        for (uint32_t q = 0; q < cnt; ++q) {
            if (base + q == i) continue;
            // pair kernel of array_particle.rs:67-76 in its IEEE operation order
            const double dx = __dsub_rn(px, sx[q]);
            const double dy = __dsub_rn(py, sy[q]);
            const double dz = __dsub_rn(pz, sz[q]);
            const double dp2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)),
                                         __dmul_rn(dz, dz));
            const double dist = __dsqrt_rn(dp2);
            const double magi = __ddiv_rn(-sm[q], __dmul_rn(__dmul_rn(dist, dist), dist));
            ax = __dadd_rn(ax, __dmul_rn(magi, dx));
            ay = __dadd_rn(ay, __dmul_rn(magi, dy));
            az = __dadd_rn(az, __dmul_rn(magi, dz));
        }
    }
    if (k < ns) {
        double *o = partial + 3 * ((size_t)c * ns + k);
        o[0] = ax;
        o[1] = ay;
        o[2] = az;
    }
}

__global__ void k_noalloc_sum(const double *partial, const uint64_t *sinks, uint32_t n,
                              uint32_t ns, uint32_t chunks, double *acc) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ns) return;
    double ax = 0.0, ay = 0.0, az = 0.0;
    if (sinks[k] < n) {
        for (uint32_t c = 0; c < chunks; ++c) {
            const double *o = partial + 3 * ((size_t)c * ns + k);
            ax += o[0];
            ay += o[1];
            az += o[2];
        }
    } else {
        ax = ay = az = __longlong_as_double(0x7ff8000000000000ll);  // NaN
    }
    acc[3 * (size_t)k] = ax;
    acc[3 * (size_t)k + 1] = ay;
    acc[3 * (size_t)k + 2] = az;
}

}  // namespace

extern "C" int kd_direct_accel_noalloc(const double *x, const double *y, const double *z,
                                       const double *m, size_t n, const uint64_t *sinks,
                                       size_t ns, double *acc, void *stream) {
    if (!x || !y || !z || !m || !sinks || !acc) {
        kd::set_thread_error("kd_direct_accel_noalloc: NULL device pointer");
        return KD_EINVAL;
    }
    if (n < 1 || n >= (size_t(1) << 31)) {
        kd::set_thread_error("kd_direct_accel_noalloc: n must be in [1, 2^31)");
        return KD_EINVAL;
    }
    if (ns < 1 || ns > kNoAllocMaxSinks) {
        kd::set_thread_error("kd_direct_accel_noalloc: ns must be in [1, 43690] "
                             "(its scratch holds 131072 doubles, 3 per sink and chunk)");
        return KD_EINVAL;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        kd::set_thread_error("kd_direct_accel_noalloc: no usable current device");
        return KD_ECUDA;
    }
    double *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_scratch_addr[dev]) {
            double *p = nullptr;
            e = cudaGetSymbolAddress((void **)&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) {
                kd::set_thread_error("kd_direct_accel_noalloc: cudaGetSymbolAddress failed");
                return KD_ECUDA;
            }
            g_scratch_addr[dev] = p;
        }
        scratch = g_scratch_addr[dev];
    }
    // as many source chunks as the scratch holds for ns sinks, none smaller than kMinChunk
    const size_t max_chunks = kNoAllocScratchDoubles / (3 * ns);
    const size_t want = (n + kMinChunk - 1) / kMinChunk;
    const uint32_t chunks = (uint32_t)(want < max_chunks ? want : max_chunks);
    const uint32_t chunk = (uint32_t)((n + chunks - 1) / chunks);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    dim3 grid((uint32_t)((ns + kThreads - 1) / kThreads), chunks);
    k_noalloc_partial<<<grid, kThreads, 0, st>>>(x, y, z, m, (uint32_t)n, sinks, (uint32_t)ns,
                                                 chunk, scratch);
    k_noalloc_sum<<<(uint32_t)((ns + 255) / 256), 256, 0, st>>>(scratch, sinks, (uint32_t)n,
                                                                (uint32_t)ns, chunks, acc);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        kd::set_thread_error(cudaGetErrorString(e));
        return KD_ECUDA;
    }
    return KD_OK;
}
