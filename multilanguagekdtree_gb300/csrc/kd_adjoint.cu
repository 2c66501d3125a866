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
// The walk (k_adj_group, kd_group.cu) repeats the forward grouped walk's traversal and
// decisions (the same code and data), accumulates the sink terms per lane (compensated) and
// the source terms per list entry: pair sources per tree position (U), node sources per node
// (G).  Heavy bodies (left out of the FP32 masses) contribute in FP64 on both sides.
#include "kd_internal.cuh"

namespace kd {

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

// Per leaf: H = sum of the node-source sums G over the leaf's ancestors; every body i of the
// leaf gets y_i = ysink_i + m_i (U_i + H) (+ the heavy-source sum for a heavy body), written
// in original order.
__global__ void k_adj_combine(Topology t, const NodeF *__restrict__ rec,
                              const float4 *__restrict__ trel, const uint32_t *__restrict__ tid,
                              const double *__restrict__ ysink, const double *__restrict__ U,
                              const double *__restrict__ G, const uint32_t *heavy_ids,
                              int n_heavy, const double *yheavy, double *__restrict__ y) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= t.n_leaves) return;
    const uint32_t leaf = t.leaves[i];
    double hx = 0.0, hy = 0.0, hz = 0.0;
    for (uint32_t a = t.parent[leaf]; a != 0xffffffffu; a = t.parent[a]) {
        hx += G[3 * (size_t)a];
        hy += G[3 * (size_t)a + 1];
        hz += G[3 * (size_t)a + 2];
    }
    const uint32_t st = rec[leaf].a, cn = rec[leaf].b;
    for (uint32_t k = st; k < st + cn; ++k) {
        const double m = (double)trel[k].w;
        const uint32_t o = tid[k];
        double vx = ysink[3 * (size_t)k] + m * (U[3 * (size_t)k] + hx);
        double vy = ysink[3 * (size_t)k + 1] + m * (U[3 * (size_t)k + 1] + hy);
        double vz = ysink[3 * (size_t)k + 2] + m * (U[3 * (size_t)k + 2] + hz);
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
    if (grid > sm_count() * 16) grid = sm_count() * 16;
    k_adj_mu<<<grid, 256, 0, st>>>(a.lx, a.lv, a.mu, n3, a.dt);
    cudaMemsetAsync(a.U, 0, sizeof(double) * 3 * (size_t)a.n, st);
    cudaMemsetAsync(a.G, 0, sizeof(double) * 3 * (size_t)a.topo.n_nodes, st);
    cudaMemsetAsync(a.yheavy, 0, sizeof(double) * 3 * kMaxHeavy, st);
    launch_adj_group(a, st);  // the walk and, with heavy bodies, their source sums
    k_adj_combine<<<(a.topo.n_leaves + 127) / 128, 128, 0, st>>>(
        a.topo, a.recf, a.trel, a.tid, a.ysink, a.U, a.G, a.heavy, a.n_heavy, a.yheavy, a.y);
    k_adj_update<<<grid, 256, 0, st>>>(a.lx, a.lv, a.mu, a.y, n3, a.dt);
    return a.n_heavy > 0 ? 5 : 4;
}

}  // namespace kd
