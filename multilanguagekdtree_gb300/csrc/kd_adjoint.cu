// kd_adjoint.cu -- reverse-mode (adjoint) step of the mixed-precision Barnes-Hut step.
//
// Forward step (array_kd_tree.rs:649-658, semi-implicit Euler):  v' = v + dt a(x),
// x' = x + dt v'.  For a loss L of the final state, with lx = dL/dx and lv = dL/dv, one
// backward step over step n is
//     mu = lv' + dt lx'          lv = mu          lx = lx' + dt J(x_n)^T mu
// where J = da/dx over the interaction set the forward walk used at x_n (tree membership
// and opening decisions are piecewise constant, so they are frozen).
//
// Every interaction of sink s with a source at c of mass m (a body of a leaf, or the
// centre of mass of an accepted node) has d = x_s - c and contributes, with the unit tidal
// product w = |d|^-3 (mu_s - 3 (d . mu_s) |d|^-2 d):
//     to the sink:                            -m w
//     to a pair source j:                     +m_j w
//     to each body i of an accepted node:     +m_i w      (dc/dx_i = m_i / M)
// The walk below repeats the forward mixed walk's traversal and decisions bit for bit
// (same data, same FP32 test), accumulates the sink terms per lane (compensated), reduces
// the source terms over the warp and adds them with one atomic per (warp, source): pair
// sources per tree position (U), node sources per node (G).  Heavy bodies (left out of the
// FP32 masses) contribute in FP64 on both sides.
#include "kd_internal.cuh"

namespace kd {

static constexpr uint32_t kFull = 0xffffffffu;

__device__ __forceinline__ void kahan_add3(float &sum, float &comp, float x) {
    const float y = x - comp;
    const float t = sum + y;
    comp = (t - sum) - y;
    sum = t;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

// mu = lv + dt lx  (original order)
__global__ void k_adj_mu(const double *lx, const double *lv, double *mu, uint32_t n3, double dt) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += gridDim.x * blockDim.x)
        mu[i] = lv[i] + dt * lx[i];
}

// lx += dt y ; lv = mu
__global__ void k_adj_update(double *lx, double *lv, const double *mu, const double *y,
                             uint32_t n3, double dt) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += gridDim.x * blockDim.x) {
        lx[i] += dt * y[i];
        lv[i] = mu[i];
    }
}

struct HeavyB {
    double x, y, z, m;
};

template <int kWarps>
__global__ __launch_bounds__(kWarps * 32) void k_adj_walk(
    const NodeF *__restrict__ rec, const float4 *__restrict__ thi,
    const float4 *__restrict__ tlo, const float4 *__restrict__ trel,
    const uint32_t *__restrict__ tid, uint32_t n, float theta2, Bodies b,
    const uint32_t *__restrict__ heavy_ids, int n_heavy, const double *__restrict__ mu,
    double *__restrict__ ysink, float *__restrict__ U, float *__restrict__ G,
    double *__restrict__ yheavy, uint32_t *err) {
    __shared__ HeavyB heavy[kMaxHeavy];
    __shared__ double hred[kWarps][kMaxHeavy][3];
    if (threadIdx.x < n_heavy) {
        const uint32_t h = heavy_ids[threadIdx.x];
        heavy[threadIdx.x] = HeavyB{b.x[h], b.y[h], b.z[h], b.m[h]};
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t s = (blockIdx.x * kWarps + warp) * 32 + lane;
    const bool valid = s < n;
    uint32_t mask = __ballot_sync(kFull, valid);
    const uint32_t bit = 1u << lane;
    const float4 mh = valid ? thi[s] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 ml = valid ? tlo[s] : make_float4(0.f, 0.f, 0.f, 0.f);
    const uint32_t o = valid ? tid[s] : 0u;
    double mux = 0.0, muy = 0.0, muz = 0.0;
    if (valid) {
        mux = mu[3 * (size_t)o];
        muy = mu[3 * (size_t)o + 1];
        muz = mu[3 * (size_t)o + 2];
    }
    const float fmx = (float)mux, fmy = (float)muy, fmz = (float)muz;
    float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
    float px = 0.f, py = 0.f, pz = 0.f;
    uint32_t st_node = 0, st_mask = 0;
    uint32_t node = 0;
    int sp = 0;
    while (mask) {
        const float4 nh = __ldg(&rec[node].hi);
        const uint2 ab = __ldg(reinterpret_cast<const uint2 *>(&rec[node].a));
        bool descend = false;
        if (ab.y != 0u) {
            const bool act = (mask & bit) != 0;
            const float4 ol = __ldg(&rec[node].lo);
            const float qx = (mh.x - nh.x) + (ml.x - ol.x);
            const float qy = (mh.y - nh.y) + (ml.y - ol.y);
            const float qz = (mh.z - nh.z) + (ml.z - ol.z);
            for (uint32_t k = 0; k < ab.y; ++k) {
                const uint32_t j = ab.x + k;
                float wx = 0.f, wy = 0.f, wz = 0.f;
                const float4 r = __ldg(&trel[j]);
                if (act && j != s) {
                    const float dx = qx - r.x, dy = qy - r.y, dz = qz - r.z;
                    const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                    const float inv = rsqrtf(d2);
                    const float inv2 = inv * inv, inv3 = inv2 * inv;
                    const float dm = fmaf(dx, fmx, fmaf(dy, fmy, dz * fmz));
                    const float c3 = 3.0f * dm * inv2;
                    wx = inv3 * fmaf(-c3, dx, fmx);
                    wy = inv3 * fmaf(-c3, dy, fmy);
                    wz = inv3 * fmaf(-c3, dz, fmz);
                    px = fmaf(-r.w, wx, px);
                    py = fmaf(-r.w, wy, py);
                    pz = fmaf(-r.w, wz, pz);
                }
                // source side of member j, summed over the warp's sinks
                wx = warp_sum(wx);
                wy = warp_sum(wy);
                wz = warp_sum(wz);
                if (lane == 0 && r.w != 0.0f) {
                    atomicAdd(&U[3 * (size_t)j], wx);
                    atomicAdd(&U[3 * (size_t)j + 1], wy);
                    atomicAdd(&U[3 * (size_t)j + 2], wz);
                }
            }
            if (act) {
                kahan_add3(sx, cx, px);
                kahan_add3(sy, cy, py);
                kahan_add3(sz, cz, pz);
                px = py = pz = 0.f;
            }
        } else {
            bool take = false;
            if (mask & bit) {
                const float ex = mh.x - nh.x, ey = mh.y - nh.y, ez = mh.z - nh.z;
                const float e2 = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
                take = nh.w < theta2 * e2;
            }
            const uint32_t tk = __ballot_sync(kFull, take);
            if (tk) {
                const float4 nl = __ldg(&rec[node].lo);
                float wx = 0.f, wy = 0.f, wz = 0.f;
                if (take) {
                    const float dx = (mh.x - nh.x) + (ml.x - nl.x);
                    const float dy = (mh.y - nh.y) + (ml.y - nl.y);
                    const float dz = (mh.z - nh.z) + (ml.z - nl.z);
                    const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                    const float inv = rsqrtf(d2);
                    const float inv2 = inv * inv, inv3 = inv2 * inv;
                    const float dm = fmaf(dx, fmx, fmaf(dy, fmy, dz * fmz));
                    const float c3 = 3.0f * dm * inv2;
                    wx = inv3 * fmaf(-c3, dx, fmx);
                    wy = inv3 * fmaf(-c3, dy, fmy);
                    wz = inv3 * fmaf(-c3, dz, fmz);
                    px = fmaf(-nl.w, wx, px);
                    py = fmaf(-nl.w, wy, py);
                    pz = fmaf(-nl.w, wz, pz);
                }
                wx = warp_sum(wx);
                wy = warp_sum(wy);
                wz = warp_sum(wz);
                if (lane == 0) {
                    atomicAdd(&G[3 * (size_t)node], wx);
                    atomicAdd(&G[3 * (size_t)node + 1], wy);
                    atomicAdd(&G[3 * (size_t)node + 2], wz);
                }
            }
            const uint32_t open = mask & ~tk;
            if (open) {
                if (sp >= kStackMax) {
                    if (lane == 0) atomicOr(err, kErrStack);
                    break;
                }
                if (lane == sp) {
                    st_node = ab.x;
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
    kahan_add3(sx, cx, px);
    kahan_add3(sy, cy, py);
    kahan_add3(sz, cz, pz);
    // heavy bodies in FP64: sink side here, source side reduced over the block
    double hx[kMaxHeavy][3];
#pragma unroll
    for (int h = 0; h < kMaxHeavy; ++h) hx[h][0] = hx[h][1] = hx[h][2] = 0.0;
    double ysx = (double)sx - (double)cx, ysy = (double)sy - (double)cy,
           ysz = (double)sz - (double)cz;
    if (valid) {
        const double X = b.x[o], Y = b.y[o], Z = b.z[o];
#pragma unroll
        for (int h = 0; h < kMaxHeavy; ++h) {
            if (h >= n_heavy || heavy_ids[h] == o) continue;
            const HeavyB q = heavy[h];
            const double dx = X - q.x, dy = Y - q.y, dz = Z - q.z;
            const double d2 = dx * dx + dy * dy + dz * dz;
            const double inv2 = 1.0 / d2;
            const double inv3 = inv2 * sqrt(inv2);
            const double dm = dx * mux + dy * muy + dz * muz;
            const double c3 = 3.0 * dm * inv2;
            const double wx = inv3 * (mux - c3 * dx), wy = inv3 * (muy - c3 * dy),
                         wz = inv3 * (muz - c3 * dz);
            ysx -= q.m * wx;
            ysy -= q.m * wy;
            ysz -= q.m * wz;
            hx[h][0] = q.m * wx;
            hx[h][1] = q.m * wy;
            hx[h][2] = q.m * wz;
        }
        ysink[3 * (size_t)s] = ysx;
        ysink[3 * (size_t)s + 1] = ysy;
        ysink[3 * (size_t)s + 2] = ysz;
    }
    if (n_heavy > 0) {
#pragma unroll
        for (int h = 0; h < kMaxHeavy; ++h)
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                double v = hx[h][d];
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(kFull, v, off);
                if (lane == 0) hred[warp][h][d] = v;
            }
        __syncthreads();
        if (threadIdx.x < (unsigned)(3 * n_heavy)) {
            const int h = threadIdx.x / 3, d = threadIdx.x % 3;
            double v = 0.0;
            for (int w = 0; w < kWarps; ++w) v += hred[w][h][d];
            atomicAdd(&yheavy[3 * h + d], v);
        }
    }
}

// Per leaf: H = sum of the node-source sums G over the leaf's ancestors; every body i of the
// leaf gets y_i = ysink_i + m_i (U_i + H) (+ the heavy-source sum for a heavy body), written
// in original order.
__global__ void k_adj_combine(Topology t, const NodeF *__restrict__ rec,
                              const float4 *__restrict__ trel, const uint32_t *__restrict__ tid,
                              const double *__restrict__ ysink, const float *__restrict__ U,
                              const float *__restrict__ G, const uint32_t *heavy_ids,
                              int n_heavy, const double *yheavy, double *__restrict__ y) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= t.n_leaves) return;
    const uint32_t leaf = t.leaves[i];
    double hx = 0.0, hy = 0.0, hz = 0.0;
    for (uint32_t a = t.parent[leaf]; a != 0xffffffffu; a = t.parent[a]) {
        hx += (double)G[3 * (size_t)a];
        hy += (double)G[3 * (size_t)a + 1];
        hz += (double)G[3 * (size_t)a + 2];
    }
    const uint32_t st = rec[leaf].a, cn = rec[leaf].b;
    for (uint32_t k = st; k < st + cn; ++k) {
        const double m = (double)trel[k].w;
        const uint32_t o = tid[k];
        double vx = ysink[3 * (size_t)k] + m * ((double)U[3 * (size_t)k] + hx);
        double vy = ysink[3 * (size_t)k + 1] + m * ((double)U[3 * (size_t)k + 1] + hy);
        double vz = ysink[3 * (size_t)k + 2] + m * ((double)U[3 * (size_t)k + 2] + hz);
        for (int h = 0; h < n_heavy; ++h)
            if (heavy_ids[h] == o) {
                vx += yheavy[3 * h];
                vy += yheavy[3 * h + 1];
                vz += yheavy[3 * h + 2];
            }
        y[3 * (size_t)o] = vx;
        y[3 * (size_t)o + 1] = vy;
        y[3 * (size_t)o + 2] = vz;
    }
}

int launch_adjoint_step(const AdjArgs &a, cudaStream_t st) {
    const uint32_t n3 = 3 * a.n;
    int grid = (int)((n3 + 255) / 256);
    if (grid > 152 * 16) grid = 152 * 16;
    k_adj_mu<<<grid, 256, 0, st>>>(a.lx, a.lv, a.mu, n3, a.dt);
    cudaMemsetAsync(a.U, 0, sizeof(float) * 3 * (size_t)a.n, st);
    cudaMemsetAsync(a.G, 0, sizeof(float) * 3 * (size_t)a.topo.n_nodes, st);
    cudaMemsetAsync(a.yheavy, 0, sizeof(double) * 3 * kMaxHeavy, st);
    constexpr int kW = 4;
    const uint32_t threads = kW * 32;
    const uint32_t blocks = (a.n + threads - 1) / threads;
    k_adj_walk<kW><<<blocks, threads, 0, st>>>(a.recf, a.thi, a.tlo, a.trel, a.tid, a.n,
                                               (float)(a.theta * a.theta), a.bodies, a.heavy,
                                               a.n_heavy, a.mu, a.ysink, a.U, a.G, a.yheavy,
                                               a.err);
    k_adj_combine<<<(a.topo.n_leaves + 127) / 128, 128, 0, st>>>(
        a.topo, a.recf, a.trel, a.tid, a.ysink, a.U, a.G, a.heavy, a.n_heavy, a.yheavy, a.y);
    k_adj_update<<<grid, 256, 0, st>>>(a.lx, a.lv, a.mu, a.y, n3, a.dt);
    return 4;
}

}  // namespace kd
