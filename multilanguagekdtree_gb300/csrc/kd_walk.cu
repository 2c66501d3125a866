// kd_walk.cu -- multipole upward pass, theta-opening traversal and kick-drift.
//
// FP64 path: every body gets exactly the interaction set of the reference's recursive walk
// (MarkCLewis/MultiLanguageKDTree Parallel/RustVersion/src/array_kd_tree.rs:585-621): a
// warp walks the union of its 32 bodies' walks with a shared stack, and a per-lane mask
// records which bodies still descend.  The opening test and both force kernels use the
// reference's IEEE operation order (array_kd_tree.rs:601-609, array_particle.rs:67-76),
// written with explicit round-to-nearest intrinsics so no multiply-add is fused.
//
// The mixed-precision path walks the tree per group of sinks (kd_group.cu).
#include "kd_internal.cuh"

namespace kd {

static constexpr uint32_t kFull = 0xffffffffu;

// ------------------------------------------------------------------ FP64 walk

__device__ __forceinline__ void load_noded(const NodeD *rec, uint32_t node, double &cx,
                                           double &cy, double &cz, double &m, double &s2,
                                           uint32_t &a, uint32_t &b) {
    const double2 *p = reinterpret_cast<const double2 *>(rec + node);
    const double2 v0 = __ldg(p), v1 = __ldg(p + 1), v2 = __ldg(p + 2);
    cx = v0.x; cy = v0.y; cz = v1.x; m = v1.y; s2 = v2.x;
    const uint2 ab = __ldg(reinterpret_cast<const uint2 *>(p + 2) + 1);
    a = ab.x;
    b = ab.y;
}

// (rsqrt64, in kd_internal.cuh, stands in for the reference's sqrt and division: the
// interaction magnitude m / (d^2 sqrt(d^2)) = m r^3 differs from the IEEE-rounded one by a
// few ulp.)
// m / |d|^3 as the reference forms it (array_kd_tree.rs:607, array_particle.rs:72-73), or
// by rsqrt64 when d2 is in its range; d2 = 0 keeps the reference's inf.
__device__ __forceinline__ double inv_cube(double d2) {
    if (d2 >= 1e-30 && d2 <= 1e30) {
        const double r = rsqrt64(d2);
        return (r * r) * r;
    }
    return __ddiv_rn(1.0, __dmul_rn(d2, __dsqrt_rn(d2)));
}

// FP32 pre-test of the opening decision size^2 < theta^2 d^2 (array_kd_tree.rs:606): on the
// split (hi + lo) coordinates d^2 carries a relative error below 1e-6 once |d| exceeds
// 1e-5 of the coordinates' magnitude, so a decision outside a 4e-6 relative margin is the
// FP64 decision.  Returns 1 (accept), 0 (open) or -1 (undecided: test in FP64).
__device__ __forceinline__ int pretest(const float4 &mh, const float4 &ml, float p2,
                                       const NodeP &q, float theta2f) {
    const float ex = (mh.x - q.hi.x) + (ml.x - q.lo.x);
    const float ey = (mh.y - q.hi.y) + (ml.y - q.lo.y);
    const float ez = (mh.z - q.hi.z) + (ml.z - q.lo.z);
    const float e2 = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
    const float scale = p2 + fmaf(q.hi.x, q.hi.x, fmaf(q.hi.y, q.hi.y, q.hi.z * q.hi.z));
    const float rhs = theta2f * e2, lhs = q.hi.w;
    const float margin = 4e-6f * (lhs + rhs);
    const bool sure = e2 >= 1e-30f && e2 > 1e-10f * scale && scale < 1e37f && rhs < 1e37f;
    if (sure && lhs < rhs - margin) return 1;
    if (sure && lhs > rhs + margin) return 0;
    return -1;
}

template <bool kCount>
__global__ __launch_bounds__(kWalkWarps * 32) void k_walk_fp64(
    const NodeD *__restrict__ rec, const NodeP *__restrict__ recp,
    const float4 *__restrict__ thi, const float4 *__restrict__ tlo,
    const dbl4 *__restrict__ tpos, const uint32_t *__restrict__ tid, uint32_t n,
    double theta2, float theta2f, double *__restrict__ acc, uint32_t *err,
    unsigned long long *counts, uint32_t stack_cap) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t s = (blockIdx.x * kWalkWarps + warp) * 32 + lane;
    const bool valid = s < n;
    uint32_t mask = __ballot_sync(kFull, valid);
    if (mask == 0) return;
    const uint32_t bit = 1u << lane;
    // traversal stack: entry k (pending right child, lanes still descending) lives in lane k
    uint32_t st_node = 0, st_mask = 0;
    dbl4 me = valid ? tpos[s] : make_double4_32a(0.0, 0.0, 0.0, 0.0);
    const float4 mh = valid ? thi[s] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 ml = valid ? tlo[s] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float p2 = fmaf(mh.x, mh.x, fmaf(mh.y, mh.y, mh.z * mh.z));
    double ax = 0.0, ay = 0.0, az = 0.0;
    unsigned long long c_p2p = 0, c_open = 0, c_m2p = 0, c_vis = 0;
    uint32_t node = 0;
    int sp = 0;
    while (true) {
        double cx, cy, cz, m, s2;
        uint32_t a, b;
        load_noded(rec, node, cx, cy, cz, m, s2, a, b);
        if (kCount) c_vis += (mask & bit) ? 1 : 0;
        bool descend = false;
        if (b != 0u) {
            // leaf: sequential pair sum, self excluded by identity (array_kd_tree.rs:588-598)
            if (mask & bit) {
                for (uint32_t k = 0; k < b; ++k) {
                    const uint32_t j = a + k;
                    if (j == s) continue;
                    const dbl4 q = ldg_dbl4(&tpos[j]);
                    const double dx = me.x - q.x, dy = me.y - q.y, dz = me.z - q.z;
                    const double dp2 = fma(dx, dx, fma(dy, dy, dz * dz));
                    const double magi = -q.w * inv_cube(dp2);
                    ax = fma(magi, dx, ax);
                    ay = fma(magi, dy, ay);
                    az = fma(magi, dz, az);
                    if (kCount) ++c_p2p;
                }
            }
        } else {
            bool take = false;
            if (mask & bit) {
                if (kCount) ++c_open;
                const NodeP q = recp[node];
                const int pre = pretest(mh, ml, p2, q, theta2f);
                if (pre != 0) {
                    // the reference's d and d^2 (exact FP64 order): the test when the FP32
                    // estimate is undecided, and the force either way
                    const double dx = __dsub_rn(me.x, cx);
                    const double dy = __dsub_rn(me.y, cy);
                    const double dz = __dsub_rn(me.z, cz);
                    const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)),
                                                __dmul_rn(dz, dz));
                    take = pre == 1 || s2 < __dmul_rn(theta2, d2);
                    if (take) {
                        const double magi = -m * inv_cube(d2);
                        ax = fma(dx, magi, ax);
                        ay = fma(dy, magi, ay);
                        az = fma(dz, magi, az);
                        if (kCount) ++c_m2p;
                    }
                }
            }
            const uint32_t open = mask & ~__ballot_sync(kFull, take);
            if (open) {
                if (sp >= (int)stack_cap) {
                    if (lane == 0) atomicOr(err, kErrStack);
                    break;
                }
                if (lane == sp) {
                    st_node = a;
                    st_mask = open;
                }
                ++sp;
                node = node + 1;
                mask = open;
                descend = true;
            }
        }
        if (descend) continue;
        if (sp == 0) break;
        --sp;
        node = __shfl_sync(kFull, st_node, sp);
        mask = __shfl_sync(kFull, st_mask, sp);
    }
    if (valid) {
        const uint32_t o = tid[s];
        acc[3 * (size_t)o] = ax;
        acc[3 * (size_t)o + 1] = ay;
        acc[3 * (size_t)o + 2] = az;
    }
    if (kCount) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            c_p2p += __shfl_xor_sync(kFull, c_p2p, o);
            c_open += __shfl_xor_sync(kFull, c_open, o);
            c_m2p += __shfl_xor_sync(kFull, c_m2p, o);
            c_vis += __shfl_xor_sync(kFull, c_vis, o);
        }
        if (lane == 0) {
            atomicAdd(&counts[0], c_p2p);
            atomicAdd(&counts[1], c_open);
            atomicAdd(&counts[2], c_m2p);
            atomicAdd(&counts[3], c_vis);
        }
    }
}

void launch_walk_fp64(const NodeD *rec, const NodeP *recp, const float4 *thi,
                      const float4 *tlo, const dbl4 *tpos, const uint32_t *tid, uint32_t n,
                      double theta, double *acc, uint32_t *err, unsigned long long *counts,
                      cudaStream_t st, uint32_t stack_cap) {
    const uint32_t threads = kWalkWarps * 32;
    const uint32_t blocks = (n + threads - 1) / threads;
    const double theta2 = theta * theta;  // THETA * THETA is formed first (array_kd_tree.rs:606)
    const float theta2f = (float)theta2;
    // the stack lives in the lanes' registers: one entry per lane at most
    stack_cap = stack_cap < (uint32_t)kStackMax ? stack_cap : (uint32_t)kStackMax;
    if (counts)
        k_walk_fp64<true><<<blocks, threads, 0, st>>>(rec, recp, thi, tlo, tpos, tid, n, theta2,
                                                      theta2f, acc, err, counts, stack_cap);
    else
        k_walk_fp64<false><<<blocks, threads, 0, st>>>(rec, recp, thi, tlo, tpos, tid, n, theta2,
                                                       theta2f, acc, err, nullptr, stack_cap);
}

// 0.5 m v^2 and 0.5 m phi summed per block in a fixed order (then on the host, in order).
__global__ void k_energy_partial(Bodies b, const double *phi, uint32_t n, double *part) {
    __shared__ double rk[256], rp[256];
    double k = 0.0, p = 0.0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double m = b.m[i];
        k += 0.5 * m * (b.vx[i] * b.vx[i] + b.vy[i] * b.vy[i] + b.vz[i] * b.vz[i]);
        p += 0.5 * m * phi[i];
    }
    rk[threadIdx.x] = k;
    rp[threadIdx.x] = p;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) {
            rk[threadIdx.x] += rk[threadIdx.x + h];
            rp[threadIdx.x] += rp[threadIdx.x + h];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = rk[0];
        part[2 * blockIdx.x + 1] = rp[0];
    }
}

void launch_energy_partial(const Bodies &b, const double *phi, uint32_t n, double *part,
                           int blocks, cudaStream_t st) {
    k_energy_partial<<<blocks, 256, 0, st>>>(b, phi, n, part);
}

// ------------------------------------------------------------------ kick-drift

// v += dt*a; p += dt*v (array_kd_tree.rs:649-658), IEEE order without fused multiply-add.
// After a failed device check of this step (or an earlier one) the state is left as it is,
// so a call that returns KD_EDEVICE leaves the bodies at the start of the failed step.
__global__ void k_kick_drift(Bodies b, const double *__restrict__ acc, uint32_t n, double dt,
                             const uint32_t *err) {
    if (*(volatile const uint32_t *)err) return;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x) {
        // every load first: the state arrays may alias as far as the compiler knows
        const double ax = acc[3 * (size_t)i], ay = acc[3 * (size_t)i + 1],
                     az = acc[3 * (size_t)i + 2];
        const double vx0 = b.vx[i], vy0 = b.vy[i], vz0 = b.vz[i];
        const double x0 = b.x[i], y0 = b.y[i], z0 = b.z[i];
        const double vx = __dadd_rn(vx0, __dmul_rn(dt, ax));
        const double vy = __dadd_rn(vy0, __dmul_rn(dt, ay));
        const double vz = __dadd_rn(vz0, __dmul_rn(dt, az));
        b.vx[i] = vx;
        b.vy[i] = vy;
        b.vz[i] = vz;
        b.x[i] = __dadd_rn(x0, __dmul_rn(dt, vx));
        b.y[i] = __dadd_rn(y0, __dmul_rn(dt, vy));
        b.z[i] = __dadd_rn(z0, __dmul_rn(dt, vz));
    }
}

void launch_kick_drift(Bodies &b, double *acc, uint32_t n, double dt, const uint32_t *err,
                       cudaStream_t st) {
    int blocks = (int)((n + 255) / 256);
    if (blocks > sm_count() * 16) blocks = sm_count() * 16;
    k_kick_drift<<<blocks, 256, 0, st>>>(b, acc, n, dt, err);
}

// ------------------------------------------------------------------ body transfer

__global__ void k_aos_to_soa(const double *__restrict__ aos, Bodies b, uint32_t n,
                             uint32_t *err) {
    bool bad = false;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x) {
        const double2 *p = reinterpret_cast<const double2 *>(aos + 8 * (size_t)i);
        const double2 a0 = p[0], a1 = p[1], a2 = p[2], a3 = p[3];
        b.x[i] = a0.x; b.y[i] = a0.y; b.z[i] = a1.x;
        b.vx[i] = a1.y; b.vy[i] = a2.x; b.vz[i] = a2.y;
        b.r[i] = a3.x; b.m[i] = a3.y;
        bad |= !(isfinite(a0.x) && isfinite(a0.y) && isfinite(a1.x) && isfinite(a1.y) &&
                 isfinite(a2.x) && isfinite(a2.y) && isfinite(a3.y) && a3.y >= 0.0);
    }
    if (__any_sync(__activemask(), bad) && bad) atomicOr(err, kErrNumeric);
}

void launch_aos_to_soa(const void *aos, Bodies &b, uint32_t n, uint32_t *err, cudaStream_t st) {
    int blocks = (int)((n + 255) / 256);
    if (blocks > sm_count() * 16) blocks = sm_count() * 16;
    k_aos_to_soa<<<blocks, 256, 0, st>>>(static_cast<const double *>(aos), b, n, err);
}

__global__ void k_soa_to_aos(Bodies b, double *__restrict__ aos, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x) {
        double2 *p = reinterpret_cast<double2 *>(aos + 8 * (size_t)i);
        p[0] = make_double2(b.x[i], b.y[i]);
        p[1] = make_double2(b.z[i], b.vx[i]);
        p[2] = make_double2(b.vy[i], b.vz[i]);
        p[3] = make_double2(b.r[i], b.m[i]);
    }
}

void launch_soa_to_aos(const Bodies &b, void *aos, uint32_t n, cudaStream_t st) {
    int blocks = (int)((n + 255) / 256);
    if (blocks > sm_count() * 16) blocks = sm_count() * 16;
    k_soa_to_aos<<<blocks, 256, 0, st>>>(b, static_cast<double *>(aos), n);
}

// Direct transfers between pinned host records and the device's SoA state: a block moves 256
// records (16 KB) through shared memory, so the host side is read or written as consecutive
// 16-byte chunks by consecutive threads, and the conversion costs no pass of its own.
constexpr int kXferRecords = 256;

__global__ __launch_bounds__(kXferRecords) void k_host_to_soa(const float4 *__restrict__ host,
                                                              Bodies b, uint32_t n,
                                                              uint32_t *err) {
    __shared__ float4 buf[4 * kXferRecords];
    bool bad = false;
    for (uint32_t r0 = blockIdx.x * kXferRecords; r0 < n; r0 += gridDim.x * kXferRecords) {
        const uint32_t cnt = min((uint32_t)kXferRecords, n - r0);
        const float4 *src = host + 4 * (size_t)r0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint32_t q = threadIdx.x + k * kXferRecords;
            if (q < 4 * cnt) buf[q] = src[q];
        }
        __syncthreads();
        if (threadIdx.x < cnt) {
            const double2 *p = reinterpret_cast<const double2 *>(buf + 4 * threadIdx.x);
            const double2 a0 = p[0], a1 = p[1], a2 = p[2], a3 = p[3];
            const uint32_t i = r0 + threadIdx.x;
            b.x[i] = a0.x; b.y[i] = a0.y; b.z[i] = a1.x;
            b.vx[i] = a1.y; b.vy[i] = a2.x; b.vz[i] = a2.y;
            b.r[i] = a3.x; b.m[i] = a3.y;
            bad |= !(isfinite(a0.x) && isfinite(a0.y) && isfinite(a1.x) && isfinite(a1.y) &&
                     isfinite(a2.x) && isfinite(a2.y) && isfinite(a3.y) && a3.y >= 0.0);
        }
        __syncthreads();
    }
    if (bad) atomicOr(err, kErrNumeric);
}

__global__ __launch_bounds__(kXferRecords) void k_soa_to_host(Bodies b, float4 *__restrict__ host,
                                                              uint32_t n) {
    __shared__ float4 buf[4 * kXferRecords];
    for (uint32_t r0 = blockIdx.x * kXferRecords; r0 < n; r0 += gridDim.x * kXferRecords) {
        const uint32_t cnt = min((uint32_t)kXferRecords, n - r0);
        if (threadIdx.x < cnt) {
            const uint32_t i = r0 + threadIdx.x;
            double2 *p = reinterpret_cast<double2 *>(buf + 4 * threadIdx.x);
            p[0] = make_double2(b.x[i], b.y[i]);
            p[1] = make_double2(b.z[i], b.vx[i]);
            p[2] = make_double2(b.vy[i], b.vz[i]);
            p[3] = make_double2(b.r[i], b.m[i]);
        }
        __syncthreads();
        float4 *dst = host + 4 * (size_t)r0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint32_t q = threadIdx.x + k * kXferRecords;
            if (q < 4 * cnt) dst[q] = buf[q];
        }
        __syncthreads();
    }
}

void launch_host_to_soa(const void *host, Bodies &b, uint32_t n, uint32_t *err,
                        cudaStream_t st) {
    int blocks = (int)((n + kXferRecords - 1) / kXferRecords);
    if (blocks > sm_count() * 8) blocks = sm_count() * 8;
    k_host_to_soa<<<blocks, kXferRecords, 0, st>>>(static_cast<const float4 *>(host), b, n, err);
}

void launch_soa_to_host(const Bodies &b, void *host, uint32_t n, cudaStream_t st) {
    int blocks = (int)((n + kXferRecords - 1) / kXferRecords);
    if (blocks > sm_count() * 8) blocks = sm_count() * 8;
    k_soa_to_host<<<blocks, kXferRecords, 0, st>>>(b, static_cast<float4 *>(host), n);
}

// ------------------------------------------------------------------ direct sum

// Sinks are spread one per thread; sources are swept in chunks of kDirectChunk bodies, one
// chunk per grid column, staged through shared memory.  Each (sink, chunk) partial is
// summed in source order; the chunks are then added in chunk order (deterministic).
__global__ __launch_bounds__(kDirectThreads) void k_direct(Bodies b, uint32_t n,
                                                          const uint64_t *__restrict__ sinks,
                                                          uint32_t ns, double *partial) {
    __shared__ double sx[kDirectThreads], sy[kDirectThreads], sz[kDirectThreads],
        sm[kDirectThreads];
    const uint32_t k = blockIdx.x * kDirectThreads + threadIdx.x;
    const uint32_t chunk = blockIdx.y;
    const uint32_t j0 = chunk * kDirectChunk, j1 = min(n, j0 + kDirectChunk);
    const bool valid = k < ns;
    const uint32_t i = valid ? (uint32_t)sinks[k] : 0u;
    const double px = valid ? b.x[i] : 0.0, py = valid ? b.y[i] : 0.0, pz = valid ? b.z[i] : 0.0;
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (uint32_t base = j0; base < j1; base += kDirectThreads) {
        const uint32_t j = base + threadIdx.x;
        __syncthreads();
        if (j < j1) {
            sx[threadIdx.x] = b.x[j];
            sy[threadIdx.x] = b.y[j];
            sz[threadIdx.x] = b.z[j];
            sm[threadIdx.x] = b.m[j];
        }
        __syncthreads();
        const uint32_t cnt = min((uint32_t)kDirectThreads, j1 - base);
        for (uint32_t q = 0; q < cnt; ++q) {
            if (base + q == i) continue;
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
    if (valid) {
        double *o = partial + 3 * ((size_t)chunk * ns + k);
        o[0] = ax;
        o[1] = ay;
        o[2] = az;
    }
}

__global__ void k_direct_sum(const double *partial, uint32_t ns, uint32_t chunks, double *acc) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ns) return;
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (uint32_t c = 0; c < chunks; ++c) {
        const double *o = partial + 3 * ((size_t)c * ns + k);
        ax += o[0];
        ay += o[1];
        az += o[2];
    }
    acc[3 * (size_t)k] = ax;
    acc[3 * (size_t)k + 1] = ay;
    acc[3 * (size_t)k + 2] = az;
}

void launch_direct(const Bodies &b, uint32_t n, const uint64_t *sinks, uint32_t ns,
                   double *partial, double *acc, cudaStream_t st) {
    const uint32_t chunks = (n + kDirectChunk - 1) / kDirectChunk;
    dim3 grid((ns + kDirectThreads - 1) / kDirectThreads, chunks);
    k_direct<<<grid, kDirectThreads, 0, st>>>(b, n, sinks, ns, partial);
    k_direct_sum<<<(ns + 255) / 256, 256, 0, st>>>(partial, ns, chunks, acc);
}

// ------------------------------------------------------------------ heavy bodies

// Total mass in a fixed reduction order (one block), then every body at or above
// frac * total is listed (unordered; the host sorts the short list).
// Total mass in a fixed order: per-block partial sums over a fixed grid, then one block
// adds the partials in block order (deterministic for a given n).
constexpr int kMassBlocks = 304;

__global__ __launch_bounds__(256) void k_mass_partial(const double *m, uint32_t n,
                                                      double *part) {
    __shared__ double red[8];
    double s = 0.0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        s += m[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(kFull, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < 8; ++w) t += red[w];
        part[blockIdx.x] = t;
    }
}

__global__ void k_mass_total(const double *part, int nblk, double *out) {
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int q = 0; q < nblk; ++q) t += part[q];
        *out = t;
    }
}

__global__ void k_heavy(const double *m, uint32_t n, double frac, const double *total,
                        uint32_t *heavy_ids, uint32_t *n_heavy) {
    const double thr = frac * (*total);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x) {
        if (m[i] > 0.0 && m[i] >= thr) {
            const uint32_t k = atomicAdd(n_heavy, 1u);
            if (k < (uint32_t)kMaxHeavy) heavy_ids[k] = i;
        }
    }
}

void launch_find_heavy(const Bodies &b, uint32_t n, double frac, double *scratch_total,
                       uint32_t *heavy_ids, uint32_t *n_heavy, uint32_t *err, cudaStream_t st) {
    (void)err;
    cudaMemsetAsync(n_heavy, 0, sizeof(uint32_t), st);
    k_mass_partial<<<kMassBlocks, 256, 0, st>>>(b.m, n, scratch_total + 1);
    k_mass_total<<<1, 32, 0, st>>>(scratch_total + 1, kMassBlocks, scratch_total);
    int blocks = (int)((n + 255) / 256);
    if (blocks > sm_count() * 8) blocks = sm_count() * 8;
    k_heavy<<<blocks, 256, 0, st>>>(b.m, n, frac, scratch_total, heavy_ids, n_heavy);
}

}  // namespace kd
