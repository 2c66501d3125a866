// kd_group.cu -- grouped theta-opening walk of the mixed-precision path.
//
// The sinks are cut into groups of whole leaves, consecutive in tree order, at most 32
// bodies each (one per lane).  A warp walks the tree once for its group: the 32 lanes test
// 32 stack nodes at a time against the group's bounding box with the opening test
// size^2 < theta^2 dmin^2, dmin the distance from the node's centre of mass to the box
// (Barnes 1990, "A modified tree code: don't laugh; it runs", J. Comput. Phys. 87:161).
// The group's bodies are boxed in two parts, split where the deepest node holding the whole
// group splits: a run of leaves that crosses a high-level split joins two far-apart corners
// of the tree, and one box around both would open nearly every node for that group.
// Accepted nodes and the bodies of reached leaves go to an interaction list in shared
// memory; whenever the list holds kFlush entries every lane sums it for its own body, so the
// force loop runs without divergence and without per-lane traversal state.
//
// A node the group accepts passes the reference's per-body test (array_kd_tree.rs:600-609)
// for every body of the group, because dmin is at most each body's distance: every body's
// force is a sum over a partition of the other bodies into nodes that each pass its own
// opening test -- a refinement of the reference walk's partition, never a coarser one.
//
// Coordinates are relative to the group's first body (split hi + lo to FP32), forces are
// FP32 with compensated (Kahan) sums per block of 32 list entries, and the heavy bodies are
// summed in FP64 at the end, as in the per-body mixed walk.
#include "kd_internal.cuh"

namespace kd {

namespace {

constexpr uint32_t kFull = 0xffffffffu;

__device__ __forceinline__ float rsqrt_ftz(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ void kahan(float &sum, float &comp, float x) {
    const float y = x - comp;
    const float t = sum + y;
    comp = (t - sum) - y;
    sum = t;
}

struct Heavy {
    double x, y, z, m;
};

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(kFull, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

__device__ __forceinline__ float warp_min(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(kFull, v, o));
    return v;
}

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(kFull, v, o));
    return v;
}

// Sum of the list entries [0, nl) on the lane's body at (qx, qy, qz): plain FP32 partial
// sums over 32 entries, each folded into the compensated sums.
template <bool kPot>
__device__ __forceinline__ void sum_list(const float4 *list, uint32_t nl, float qx, float qy,
                                         float qz, float (&s)[4], float (&c)[4]) {
    for (uint32_t k0 = 0; k0 < nl; k0 += 32) {
        const uint32_t k1 = min(nl, k0 + 32u);
        float px = 0.f, py = 0.f, pz = 0.f, pp = 0.f;
#pragma unroll 8
        for (uint32_t k = k0; k < k1; ++k) {
            const float4 e = list[k];
            const float dx = e.x - qx, dy = e.y - qy, dz = e.z - qz;
            const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            const float inv = rsqrt_ftz(d2);
            const float mi = e.w * inv;
            const float f = mi * (inv * inv);
            px = fmaf(f, dx, px);
            py = fmaf(f, dy, py);
            pz = fmaf(f, dz, pz);
            if (kPot) pp += mi;
        }
        kahan(s[0], c[0], px);
        kahan(s[1], c[1], py);
        kahan(s[2], c[2], pz);
        if (kPot) kahan(s[3], c[3], -pp);
    }
}

}  // namespace

template <bool kCount, bool kPot>
__global__ __launch_bounds__(kGroupWarps * 32, 4) void k_walk_group(
    const NodeF *__restrict__ rec, const float4 *__restrict__ thi,
    const float4 *__restrict__ tlo, const float4 *__restrict__ trel,
    const uint32_t *__restrict__ tid, const uint32_t *__restrict__ gstart,
    const uint32_t *__restrict__ gsplit, uint32_t n_groups, uint32_t stk_cap, float theta2, Bodies b, const uint32_t *__restrict__ heavy_ids,
    int n_heavy, double *__restrict__ acc, double *__restrict__ phi, uint32_t *err,
    unsigned long long *counts) {
    extern __shared__ float4 smem[];
    __shared__ Heavy heavy[kMaxHeavy];
    if (threadIdx.x < n_heavy) {
        const uint32_t h = heavy_ids[threadIdx.x];
        heavy[threadIdx.x] = Heavy{b.x[h], b.y[h], b.z[h], b.m[h]};
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t g = blockIdx.x * kGroupWarps + warp;
    if (g >= n_groups) return;  // no block-wide barrier follows
    const uint32_t wbytes = group_warp_bytes(stk_cap);
    float4 *list = reinterpret_cast<float4 *>(reinterpret_cast<char *>(smem) + warp * wbytes);
    float4 *own = list + kGroupListCap;
    uint32_t *own_pos = reinterpret_cast<uint32_t *>(own + 32);
    uint32_t *stk = own_pos + 32;
    const uint32_t lt = (1u << lane) - 1u;

    const uint32_t g0 = gstart[g], g1 = gstart[g + 1], gs = gsplit[g];
    const bool valid = lane < (int)(g1 - g0);
    const uint32_t s = valid ? g0 + lane : g0;
    const float4 mh = thi[s], ml = tlo[s];
    // the group's frame: origin at its first body, split precision
    const float ohx = __shfl_sync(kFull, mh.x, 0), ohy = __shfl_sync(kFull, mh.y, 0),
                ohz = __shfl_sync(kFull, mh.z, 0);
    const float olx = __shfl_sync(kFull, ml.x, 0), oly = __shfl_sync(kFull, ml.y, 0),
                olz = __shfl_sync(kFull, ml.z, 0);
    const float qx = (mh.x - ohx) + (ml.x - olx);
    const float qy = (mh.y - ohy) + (ml.y - oly);
    const float qz = (mh.z - ohz) + (ml.z - olz);
    // two boxes: the group's bodies before and after the split of the deepest node holding
    // the whole group (an empty box gives an infinite distance)
    const bool inA = valid && s < gs, inB = valid && s >= gs;
    const float alx = warp_min(inA ? qx : INFINITY), ahx = warp_max(inA ? qx : -INFINITY);
    const float aly = warp_min(inA ? qy : INFINITY), ahy = warp_max(inA ? qy : -INFINITY);
    const float alz = warp_min(inA ? qz : INFINITY), ahz = warp_max(inA ? qz : -INFINITY);
    const float blx = warp_min(inB ? qx : INFINITY), bhx = warp_max(inB ? qx : -INFINITY);
    const float bly = warp_min(inB ? qy : INFINITY), bhy = warp_max(inB ? qy : -INFINITY);
    const float blz = warp_min(inB ? qz : INFINITY), bhz = warp_max(inB ? qz : -INFINITY);

    float sum[4] = {0.f, 0.f, 0.f, 0.f}, comp[4] = {0.f, 0.f, 0.f, 0.f};
    uint32_t nl = 0, nown = 0, top = 1;
    unsigned long long n_m2p = 0, n_p2p = 0, n_test = 0;
    if (lane == 0) stk[0] = 0u;
    __syncwarp();
    while (top > 0) {
        const uint32_t take = min(top, 32u);
        const bool has = (uint32_t)lane < take;
        const uint32_t node = has ? stk[top - 1 - lane] : 0u;
        top -= take;
        __syncwarp();
        if (kCount) n_test += take;
        float4 h = make_float4(0.f, 0.f, 0.f, 0.f), l = h;
        uint2 ab = make_uint2(0u, 0u);
        if (has) {
            h = __ldg(&rec[node].hi);
            l = __ldg(&rec[node].lo);
            ab = __ldg(reinterpret_cast<const uint2 *>(&rec[node].a));
        }
        const bool leaf = ab.y != 0u;
        // centre of mass (leaf: its first body) in the group frame
        const float cx = (h.x - ohx) + (l.x - olx);
        const float cy = (h.y - ohy) + (l.y - oly);
        const float cz = (h.z - ohz) + (l.z - olz);
        const float ex = fmaxf(fmaxf(alx - cx, cx - ahx), 0.f);
        const float ey = fmaxf(fmaxf(aly - cy, cy - ahy), 0.f);
        const float ez = fmaxf(fmaxf(alz - cz, cz - ahz), 0.f);
        const float fx = fmaxf(fmaxf(blx - cx, cx - bhx), 0.f);
        const float fy = fmaxf(fmaxf(bly - cy, cy - bhy), 0.f);
        const float fz = fmaxf(fmaxf(blz - cz, cz - bhz), 0.f);
        const float dmin2 = fminf(fmaf(ex, ex, fmaf(ey, ey, ez * ez)),
                                  fmaf(fx, fx, fmaf(fy, fy, fz * fz)));
        const bool take_m = has && !leaf && h.w < theta2 * dmin2;
        const bool open = has && !leaf && !take_m;
        const bool mine = has && leaf && ab.x >= g0 && ab.x < g1;
        const bool far = has && leaf && !mine;

        // accepted nodes: one entry each
        const uint32_t am = __ballot_sync(kFull, take_m);
        if (take_m) list[nl + __popc(am & lt)] = make_float4(cx, cy, cz, l.w);
        nl += __popc(am);
        if (kCount) n_m2p += __popc(am);
        // reached leaves: their bodies, the group's own leaves into their own list
        const uint32_t fc = far ? ab.y : 0u, oc = mine ? ab.y : 0u;
        const uint32_t fi = warp_incl_scan(fc, lane), oi = warp_incl_scan(oc, lane);
        const uint32_t ft = __shfl_sync(kFull, fi, 31), ot = __shfl_sync(kFull, oi, 31);
        if (leaf && has) {
            // all member loads of the leaf in flight at once (leaf size <= 8)
            float4 t[8];
#pragma unroll
            for (uint32_t k = 0; k < 8; ++k)
                if (k < ab.y) t[k] = __ldg(&trel[ab.x + k]);
            if (far) {
                float4 *dst = list + nl + fi - fc;
#pragma unroll
                for (uint32_t k = 0; k < 8; ++k)
                    if (k < ab.y) dst[k] = make_float4(cx + t[k].x, cy + t[k].y, cz + t[k].z, t[k].w);
            } else {
                const uint32_t o0 = nown + oi - oc;
#pragma unroll
                for (uint32_t k = 0; k < 8; ++k)
                    if (k < ab.y && o0 + k < 32u) {
                        own[o0 + k] = make_float4(cx + t[k].x, cy + t[k].y, cz + t[k].z, t[k].w);
                        own_pos[o0 + k] = ab.x + k;
                    }
            }
        }
        nl += ft;
        nown = min(nown + ot, 32u);
        if (kCount) n_p2p += ft;
        // opened nodes: both children
        const uint32_t om = __ballot_sync(kFull, open);
        if (top + 2u * __popc(om) > stk_cap) {
            if (lane == 0) atomicOr(err, kErrStack);
            break;
        }
        if (open) {
            const uint32_t slot = top + 2u * __popc(om & lt);
            stk[slot] = ab.x;      // right child
            stk[slot + 1] = node + 1u;  // left child
        }
        top += 2u * __popc(om);
        __syncwarp();
        if (nl >= (uint32_t)kGroupFlush) {
            sum_list<kPot>(list, nl, qx, qy, qz, sum, comp);
            nl = 0;
            __syncwarp();
        }
    }
    __syncwarp();
    if (nl) sum_list<kPot>(list, nl, qx, qy, qz, sum, comp);
    // the group's own leaves, self excluded by tree position
    {
        float px = 0.f, py = 0.f, pz = 0.f, pp = 0.f;
        for (uint32_t k = 0; k < nown; ++k) {
            if (own_pos[k] == s) continue;
            const float4 e = own[k];
            const float dx = e.x - qx, dy = e.y - qy, dz = e.z - qz;
            const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            const float inv = rsqrt_ftz(d2);
            const float mi = e.w * inv;
            const float f = mi * (inv * inv);
            px = fmaf(f, dx, px);
            py = fmaf(f, dy, py);
            pz = fmaf(f, dz, pz);
            if (kPot) pp += mi;
        }
        kahan(sum[0], comp[0], px);
        kahan(sum[1], comp[1], py);
        kahan(sum[2], comp[2], pz);
        if (kPot) kahan(sum[3], comp[3], -pp);
    }
    if (valid) {
        const uint32_t o = tid[s];
        double ax = (double)sum[0] - (double)comp[0];
        double ay = (double)sum[1] - (double)comp[1];
        double az = (double)sum[2] - (double)comp[2];
        double ph = (double)sum[3] - (double)comp[3];
        // heavy bodies in FP64, pair kernel of array_particle.rs:67-76
        const double px64 = b.x[o], py64 = b.y[o], pz64 = b.z[o];
        for (int hh = 0; hh < n_heavy; ++hh) {
            if (heavy_ids[hh] == o) continue;
            const Heavy q = heavy[hh];
            const double dx = px64 - q.x, dy = py64 - q.y, dz = pz64 - q.z;
            const double dp2 = dx * dx + dy * dy + dz * dz;
            const double dist = sqrt(dp2);
            const double magi = -q.m / (dist * dist * dist);
            ax += magi * dx;
            ay += magi * dy;
            az += magi * dz;
            if (kPot) ph -= q.m / dist;
        }
        acc[3 * (size_t)o] = ax;
        acc[3 * (size_t)o + 1] = ay;
        acc[3 * (size_t)o + 2] = az;
        if (kPot) phi[o] = ph;
    }
    if (kCount && lane == 0) {
        const unsigned long long nv = g1 - g0;
        // the own leaves hold every body of the group (each reached once)
        const unsigned long long own_pairs = nown >= nv ? nv * (nown - 1) : nv * nown;
        atomicAdd(&counts[0], nv * n_p2p + own_pairs);
        atomicAdd(&counts[1], n_test);
        atomicAdd(&counts[2], nv * n_m2p);
        atomicAdd(&counts[3], nv * n_test);
    }
}

void launch_walk_group(const NodeF *rec, const float4 *thi, const float4 *tlo,
                       const float4 *trel, const uint32_t *tid, const uint32_t *gstart,
                       const uint32_t *gsplit, uint32_t n_groups, uint32_t stk_cap, double theta, const Bodies &b,
                       const uint32_t *heavy_ids, int n_heavy, double *acc, uint32_t *err,
                       unsigned long long *counts, cudaStream_t st, double *phi) {
    const uint32_t threads = kGroupWarps * 32;
    const uint32_t blocks = (n_groups + kGroupWarps - 1) / kGroupWarps;
    const size_t smem = (size_t)kGroupWarps * group_warp_bytes(stk_cap);
    const float theta2 = (float)(theta * theta);
    if (phi) {
        auto k = k_walk_group<false, true>;
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k<<<blocks, threads, smem, st>>>(rec, thi, tlo, trel, tid, gstart, gsplit, n_groups, stk_cap,
                                         theta2, b, heavy_ids, n_heavy, acc, phi, err, nullptr);
    } else if (counts) {
        auto k = k_walk_group<true, false>;
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k<<<blocks, threads, smem, st>>>(rec, thi, tlo, trel, tid, gstart, gsplit, n_groups, stk_cap,
                                         theta2, b, heavy_ids, n_heavy, acc, nullptr, err, counts);
    } else {
        auto k = k_walk_group<false, false>;
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k<<<blocks, threads, smem, st>>>(rec, thi, tlo, trel, tid, gstart, gsplit, n_groups, stk_cap,
                                         theta2, b, heavy_ids, n_heavy, acc, nullptr, err, nullptr);
    }
}

}  // namespace kd
