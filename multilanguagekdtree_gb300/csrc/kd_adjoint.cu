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
// the source terms over the warp with reduce-scatter butterflies and adds them with one
// atomic per (warp, source): pair sources per tree position (U), node sources per node (G).  Heavy bodies (left out of the
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

// Reduce-scatter over the warp of V values per lane (V = 3 * 2^k, value v[3q + c] belongs
// to source q, component c): halving steps while more than 3 values remain, then a full
// reduction of the last 3.  Afterwards the lanes whose bits above the finished ones equal q
// hold the warp sums of source q in v[0..2].
template <int V>
__device__ __forceinline__ void butterfly(float (&v)[V], int lane) {
    int cnt = V;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        if (cnt > 3) {
            const bool upper = (lane & o) != 0;
            const int h = cnt / 2;
#pragma unroll
            for (int i = 0; i < V / 2; ++i) {
                if (i < h) {
                    const float send = upper ? v[i] : v[i + h];
                    const float keep = upper ? v[i + h] : v[i];
                    v[i] = keep + __shfl_xor_sync(kFull, send, o);
                }
            }
            cnt = h;
        } else {
#pragma unroll
            for (int i = 0; i < 3; ++i) v[i] += __shfl_xor_sync(kFull, v[i], o);
        }
    }
}

struct AdjSink {
    float4 mh, ml;             // split coordinates of the sink
    float mx, my, mz;          // mu of the sink (FP32)
    float px, py, pz;          // partial sink-side sum
    float sx, sy, sz, cx, cy, cz;  // compensated sink-side sum
};

// Sink-side term and unit tidal product w for a source at displacement d, mass m.
__device__ __forceinline__ void tidal(const AdjSink &k, float dx, float dy, float dz, float &wx,
                                      float &wy, float &wz) {
    const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    const float inv = rsqrtf(d2);
    const float inv2 = inv * inv, inv3 = inv2 * inv;
    const float dm = fmaf(dx, k.mx, fmaf(dy, k.my, dz * k.mz));
    const float c3 = 3.0f * dm * inv2;
    wx = inv3 * fmaf(-c3, dx, k.mx);
    wy = inv3 * fmaf(-c3, dy, k.my);
    wz = inv3 * fmaf(-c3, dz, k.mz);
}

// Pair sources of one leaf for the lanes in `act`: sink terms into the partial, source terms
// reduced over the warp and added to U (tree order) by one lane per member.
template <int M>
__device__ __forceinline__ void adj_leaf(const NodeF *__restrict__ rec,
                                         const float4 *__restrict__ trel, uint32_t node,
                                         const float4 &nh, const uint2 &ab, bool act, uint32_t s,
                                         AdjSink &k, float *__restrict__ U, int lane) {
    float v[3 * M];
#pragma unroll
    for (int i = 0; i < 3 * M; ++i) v[i] = 0.f;
    float mass[M];
    const float4 ol = __ldg(&rec[node].lo);
    const float qx = (k.mh.x - nh.x) + (k.ml.x - ol.x);
    const float qy = (k.mh.y - nh.y) + (k.ml.y - ol.y);
    const float qz = (k.mh.z - nh.z) + (k.ml.z - ol.z);
#pragma unroll
    for (int q = 0; q < M; ++q) {
        mass[q] = 0.f;
        if ((uint32_t)q < ab.y) {
            const uint32_t j = ab.x + q;
            const float4 r = __ldg(&trel[j]);
            mass[q] = r.w;
            if (act && j != s) {
                float wx, wy, wz;
                tidal(k, qx - r.x, qy - r.y, qz - r.z, wx, wy, wz);
                k.px = fmaf(-r.w, wx, k.px);
                k.py = fmaf(-r.w, wy, k.py);
                k.pz = fmaf(-r.w, wz, k.pz);
                v[3 * q] = wx;
                v[3 * q + 1] = wy;
                v[3 * q + 2] = wz;
            }
        }
    }
    if (act) {
        kahan_add3(k.sx, k.cx, k.px);
        kahan_add3(k.sy, k.cy, k.py);
        kahan_add3(k.sz, k.cz, k.pz);
        k.px = k.py = k.pz = 0.f;
    }
    butterfly<3 * M>(v, lane);
    // after the halving steps lane bits 4..(5-log2 M) name the member it holds
    constexpr int kShift = 5 - (M == 8 ? 3 : (M == 4 ? 2 : (M == 2 ? 1 : 0)));
    const int q = lane >> kShift;
    if ((lane & ((1 << kShift) - 1)) == 0 && (uint32_t)q < ab.y) {
        float m = 0.f;
#pragma unroll
        for (int t = 0; t < M; ++t)
            if (t == q) m = mass[t];
        if (m != 0.0f) {
            const uint32_t j = ab.x + q;
            atomicAdd(&U[3 * (size_t)j], v[0]);
            atomicAdd(&U[3 * (size_t)j + 1], v[1]);
            atomicAdd(&U[3 * (size_t)j + 2], v[2]);
        }
    }
}

// One child of an opened node.  Leaf: pair terms (sink and source side).  Internal node:
// opening test, multipole sink term; w is returned for the caller's source-side reduction.
__device__ __forceinline__ uint32_t adj_visit(const NodeF *__restrict__ rec,
                                              const float4 *__restrict__ trel, uint32_t node,
                                              const float4 &nh, const uint2 &ab, uint32_t mask,
                                              uint32_t bit, uint32_t s, float theta2,
                                              AdjSink &k, float *__restrict__ U, int lane,
                                              bool &took, float &wx, float &wy, float &wz) {
    const bool act = (mask & bit) != 0;
    took = false;
    wx = wy = wz = 0.f;
    if (ab.y != 0u) {
        if (ab.y <= 4u)
            adj_leaf<4>(rec, trel, node, nh, ab, act, s, k, U, lane);
        else
            adj_leaf<8>(rec, trel, node, nh, ab, act, s, k, U, lane);
        return 0u;
    }
    const float ex = k.mh.x - nh.x, ey = k.mh.y - nh.y, ez = k.mh.z - nh.z;
    const float e2 = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
    const bool take = act && nh.w < theta2 * e2;
    const uint32_t tk = __ballot_sync(kFull, take);
    if (tk) {
        const float4 nl = __ldg(&rec[node].lo);
        if (take) {
            tidal(k, ex + (k.ml.x - nl.x), ey + (k.ml.y - nl.y), ez + (k.ml.z - nl.z), wx, wy,
                  wz);
            k.px = fmaf(-nl.w, wx, k.px);
            k.py = fmaf(-nl.w, wy, k.py);
            k.pz = fmaf(-nl.w, wz, k.pz);
            took = true;
        }
    }
    return mask & ~tk;
}

// The traversal of k_walk_mixed (both children of an opened node per iteration, the same
// per-lane decisions), with the transpose-Jacobian terms in place of the forces.
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
    AdjSink k;
    k.mh = valid ? thi[s] : make_float4(0.f, 0.f, 0.f, 0.f);
    k.ml = valid ? tlo[s] : make_float4(0.f, 0.f, 0.f, 0.f);
    const uint32_t o = valid ? tid[s] : 0u;
    double mux = 0.0, muy = 0.0, muz = 0.0;
    if (valid) {
        mux = mu[3 * (size_t)o];
        muy = mu[3 * (size_t)o + 1];
        muz = mu[3 * (size_t)o + 2];
    }
    k.mx = (float)mux;
    k.my = (float)muy;
    k.mz = (float)muz;
    k.px = k.py = k.pz = 0.f;
    k.sx = k.sy = k.sz = k.cx = k.cy = k.cz = 0.f;
    uint32_t st_node = 0, st_right = 0, st_mask = 0;
    int sp = 0;
    uint32_t cur = 0, cur_right = 0;
    if (mask) {
        const float4 nh = __ldg(&rec[0].hi);
        const uint2 ab = __ldg(reinterpret_cast<const uint2 *>(&rec[0].a));
        bool took;
        float wx, wy, wz;
        mask = adj_visit(rec, trel, 0u, nh, ab, mask, bit, s, theta2, k, U, lane, took, wx, wy,
                         wz);
        if (__any_sync(kFull, took)) {
            float v[3] = {wx, wy, wz};
            butterfly<3>(v, lane);
            if (lane == 0) {
                atomicAdd(&G[0], v[0]);
                atomicAdd(&G[1], v[1]);
                atomicAdd(&G[2], v[2]);
            }
        }
        cur_right = ab.x;
    }
    while (mask) {
        const uint32_t L = cur + 1, R = cur_right;
        const float4 hL = __ldg(&rec[L].hi);
        const uint2 aL = __ldg(reinterpret_cast<const uint2 *>(&rec[L].a));
        const float4 hR = __ldg(&rec[R].hi);
        const uint2 aR = __ldg(reinterpret_cast<const uint2 *>(&rec[R].a));
        bool tL, tR;
        float v[6];
        const uint32_t oL = adj_visit(rec, trel, L, hL, aL, mask, bit, s, theta2, k, U, lane, tL,
                                      v[0], v[1], v[2]);
        const uint32_t oR = adj_visit(rec, trel, R, hR, aR, mask, bit, s, theta2, k, U, lane, tR,
                                      v[3], v[4], v[5]);
        const bool anyL = __any_sync(kFull, tL), anyR = __any_sync(kFull, tR);
        if (anyL || anyR) {
            // node sources of both children at once: lanes 0-15 end with L's sums, 16-31 R's
            butterfly<6>(v, lane);
            if ((lane & 15) == 0 && (lane ? anyR : anyL)) {
                const uint32_t nd = lane ? R : L;
                atomicAdd(&G[3 * (size_t)nd], v[0]);
                atomicAdd(&G[3 * (size_t)nd + 1], v[1]);
                atomicAdd(&G[3 * (size_t)nd + 2], v[2]);
            }
        }
        if (oL) {
            if (oR) {
                if (sp >= kStackMax) {
                    if (lane == 0) atomicOr(err, kErrStack);
                    break;
                }
                if (lane == sp) {
                    st_node = R;
                    st_right = aR.x;
                    st_mask = oR;
                }
                ++sp;
            }
            cur = L;
            cur_right = aL.x;
            mask = oL;
        } else if (oR) {
            cur = R;
            cur_right = aR.x;
            mask = oR;
        } else {
            if (sp == 0) break;
            --sp;
            cur = __shfl_sync(kFull, st_node, sp);
            cur_right = __shfl_sync(kFull, st_right, sp);
            mask = __shfl_sync(kFull, st_mask, sp);
        }
    }
    kahan_add3(k.sx, k.cx, k.px);
    kahan_add3(k.sy, k.cy, k.py);
    kahan_add3(k.sz, k.cz, k.pz);
    // heavy bodies in FP64: sink side here, source side reduced over the block
    double hx[kMaxHeavy][3];
#pragma unroll
    for (int h = 0; h < kMaxHeavy; ++h) hx[h][0] = hx[h][1] = hx[h][2] = 0.0;
    double ysx = (double)k.sx - (double)k.cx, ysy = (double)k.sy - (double)k.cy,
           ysz = (double)k.sz - (double)k.cz;
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
                double val = hx[h][d];
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) val += __shfl_xor_sync(kFull, val, off);
                if (lane == 0) hred[warp][h][d] = val;
            }
        __syncthreads();
        if (threadIdx.x < (unsigned)(3 * n_heavy)) {
            const int h = threadIdx.x / 3, d = threadIdx.x % 3;
            double val = 0.0;
            for (int w = 0; w < kWarps; ++w) val += hred[w][h][d];
            atomicAdd(&yheavy[3 * h + d], val);
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
