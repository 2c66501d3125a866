// kd_group.cu -- grouped theta-opening walk of the mixed-precision path, and its adjoint.
//
// The sinks are cut into groups of whole leaves, consecutive in tree order, at most 64
// bodies each (two per lane).  A warp walks the tree once for its group: the 32 lanes test
// 32 stack nodes at a time against the group's bounding box with the opening test
// size^2 < theta^2 dmin^2, dmin the distance from the node's centre of mass to the box
// (Barnes 1990, "A modified tree code: don't laugh; it runs", J. Comput. Phys. 87:161).
// The group's bodies are boxed in two parts, split where the deepest node holding the whole
// group splits: a run of leaves that crosses a high-level split joins two far-apart corners
// of the tree, and one box around both would open nearly every node for that group.
// Accepted nodes and the bodies of reached leaves go to an interaction list in shared
// memory; whenever the list holds kGroupFlush entries every lane sums it for its two bodies,
// so the force loop runs without divergence and without per-lane traversal state.  Two
// sinks per lane halve the traversal per body against 32-body groups, for a group box that
// accepts somewhat fewer nodes.
//
// A node the group accepts passes the reference's per-body test (array_kd_tree.rs:600-609)
// for every body of the group, because dmin is at most each body's distance: every body's
// force is a sum over a partition of the other bodies into nodes that each pass its own
// opening test -- a refinement of the reference walk's partition, never a coarser one.
//
// Coordinates are relative to the group's first body (split hi + lo to FP32), forces are
// FP32, two list entries per packed f32x2 instruction, with compensated (Kahan) sums per
// block of 64 list entries, and the heavy bodies are summed in FP64 at the end.
//
// The adjoint walk runs the same traversal (the same code, so the same decisions) and
// evaluates each block of 32 list entries against the 64 sinks with a rotation: at step k
// lane l pairs its two sinks with entry (l + k) mod 32 and passes the entry's source-side
// accumulator one lane down, so after 32 steps lane l holds the sum over all sinks for
// entry l -- both sides of J^T mu from one tidal product per pair, one FP64 atomic per entry
// and component (the sums over groups then carry no FP32 rounding).
#include "kd_internal.cuh"

namespace kd {

namespace {

constexpr uint32_t kFull = 0xffffffffu;
constexpr uint32_t kNodeTarget = 0x80000000u;  // adjoint list target: node id (else body)
constexpr uint32_t kNoTarget = 0xffffffffu;
constexpr float kFar = 1e15f;  // position of padding entries: contributes exactly nothing

__device__ __forceinline__ float rsqrt_ftz(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Two FP32 values in one 64-bit register, for the packed f32x2 arithmetic of sm_100 and
// later (one instruction, two IEEE round-to-nearest results).
typedef unsigned long long f2;

__device__ __forceinline__ f2 pk(float a, float b) {
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}

__device__ __forceinline__ void upk(f2 v, float &a, float &b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}

__device__ __forceinline__ f2 add2(f2 a, f2 b) {
    f2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}

__device__ __forceinline__ f2 sub2(f2 a, f2 b) {
    f2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}

__device__ __forceinline__ f2 mul2(f2 a, f2 b) {
    f2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}

__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
    f2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
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

// Per-warp shared memory: interaction list, own-leaf list, stack, and (adjoint) the list's
// source targets.  An own-list entry k is own[2k] = (hi xyz, light mass) and
// own[2k+1] = (lo xyz, tree position as bits): pairs inside the group are formed from the
// split absolute positions, so a close pair's separation keeps its relative precision.
struct WarpMem {
    float4 *list, *own;
    uint32_t *stk, *tgt;
};

__device__ __forceinline__ WarpMem warp_mem(float4 *smem, int warp, uint32_t stk_cap,
                                            bool with_tgt) {
    const uint32_t wbytes =
        group_warp_bytes(stk_cap) + (with_tgt ? kGroupListCap * (uint32_t)sizeof(uint32_t) : 0u);
    WarpMem w;
    w.list = reinterpret_cast<float4 *>(reinterpret_cast<char *>(smem) + warp * wbytes);
    w.own = w.list + kGroupListCap;
    w.stk = reinterpret_cast<uint32_t *>(w.own + 2 * kGroupSinks);
    w.tgt = w.stk + stk_cap;
    return w;
}

// List entry k.  The adjoint keeps one float4 per entry; the force walk keeps four component
// arrays X, Y, Z, M of kGroupListCap floats each in the same space, so that four
// consecutive entries of a component are one aligned float4 and two of them fill one packed
// register.
static_assert(kGroupListCap % 4 == 0, "component arrays must stay 16-byte aligned");

template <bool kSoA>
__device__ __forceinline__ void put_entry(const WarpMem &W, uint32_t k, float x, float y,
                                          float z, float m) {
    if (kSoA) {
        float *L = reinterpret_cast<float *>(W.list);
        L[k] = x;
        L[kGroupListCap + k] = y;
        L[2 * kGroupListCap + k] = z;
        L[3 * kGroupListCap + k] = m;
    } else {
        W.list[k] = make_float4(x, y, z, m);
    }
}

// One lane's view of its group: tree positions, frame origin, the lane's two sinks (bodies
// lane and lane + 32 of the group), the two boxes.
struct Group {
    uint32_t g0, g1;
    uint32_t s[2];                       // the sinks' tree positions (g0 when absent)
    bool valid[2];
    float ohx, ohy, ohz, olx, oly, olz;  // origin: the group's first body, hi + lo
    float qx[2], qy[2], qz[2];           // the sinks in the group frame
    float a[6], b[6];                    // boxes (lo xyz, hi xyz) before / after the split
};

__device__ __forceinline__ Group make_group(const float4 *__restrict__ thi,
                                            const float4 *__restrict__ tlo, uint32_t g0,
                                            uint32_t g1, uint32_t gs, int lane) {
    Group G;
    G.g0 = g0;
    G.g1 = g1;
    float4 mh[2], ml[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
        G.valid[u] = lane + 32 * u < (int)(g1 - g0);
        G.s[u] = G.valid[u] ? g0 + lane + 32 * u : g0;
        mh[u] = thi[G.s[u]];
        ml[u] = tlo[G.s[u]];
    }
    G.ohx = __shfl_sync(kFull, mh[0].x, 0);
    G.ohy = __shfl_sync(kFull, mh[0].y, 0);
    G.ohz = __shfl_sync(kFull, mh[0].z, 0);
    G.olx = __shfl_sync(kFull, ml[0].x, 0);
    G.oly = __shfl_sync(kFull, ml[0].y, 0);
    G.olz = __shfl_sync(kFull, ml[0].z, 0);
#pragma unroll
    for (int u = 0; u < 2; ++u) {
        G.qx[u] = (mh[u].x - G.ohx) + (ml[u].x - G.olx);
        G.qy[u] = (mh[u].y - G.ohy) + (ml[u].y - G.oly);
        G.qz[u] = (mh[u].z - G.ohz) + (ml[u].z - G.olz);
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        float alo = INFINITY, ahi = -INFINITY, blo = INFINITY, bhi = -INFINITY;
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const float q = d == 0 ? G.qx[u] : d == 1 ? G.qy[u] : G.qz[u];
            const bool inA = G.valid[u] && G.s[u] < gs, inB = G.valid[u] && G.s[u] >= gs;
            alo = fminf(alo, inA ? q : INFINITY);
            ahi = fmaxf(ahi, inA ? q : -INFINITY);
            blo = fminf(blo, inB ? q : INFINITY);
            bhi = fmaxf(bhi, inB ? q : -INFINITY);
        }
        G.a[d] = warp_min(alo);
        G.a[d + 3] = warp_max(ahi);
        G.b[d] = warp_min(blo);
        G.b[d + 3] = warp_max(bhi);
    }
    return G;
}

// Walk of one group.  Accepted nodes and far leaves' bodies are appended to W.list (with
// their source targets when kTgt, as float4 entries; else in component arrays); the group's
// own leaves go to W.own.  flush(nl) is called whenever the list holds kGroupFlush entries
// or more, and at the end.
template <bool kTgt, bool kCount, typename Flush>
__device__ __forceinline__ void traverse(const NodeF *__restrict__ rec,
                                         const float4 *__restrict__ trel,
                                         const float4 *__restrict__ thi,
                                         const float4 *__restrict__ tlo, const Group &G,
                                         const WarpMem &W, uint32_t stk_cap, float theta2,
                                         int lane, uint32_t *err, uint32_t &nown,
                                         unsigned long long (&cnt)[3], Flush &&flush) {
    const uint32_t lt = (1u << lane) - 1u;
    uint32_t nl = 0, top = 1;
    nown = 0;
    if (lane == 0) W.stk[0] = 0u;
    __syncwarp();
    // Software-pipelined: a wave's children are pushed as soon as its tests are done, and
    // the next wave's records are requested before this wave's list entries are written and
    // the list is flushed, so their latency overlaps that work.  The order of tests and of
    // list entries is the same as popping and loading at the top of each wave.
    uint32_t take = 1u;
    bool has = lane == 0;
    uint32_t node = 0u;
    top = 0u;
    float4 h = make_float4(0.f, 0.f, 0.f, 0.f), l = h;
    uint2 ab = make_uint2(0u, 0u);
    if (has) {
        h = __ldg(&rec[0].hi);
        l = __ldg(&rec[0].lo);
        ab = __ldg(reinterpret_cast<const uint2 *>(&rec[0].a));
    }
    while (take > 0) {
        if (kCount) cnt[2] += take;
        const bool leaf = ab.y != 0u;
        // centre of mass (leaf: its first body) in the group frame
        const float cx = (h.x - G.ohx) + (l.x - G.olx);
        const float cy = (h.y - G.ohy) + (l.y - G.oly);
        const float cz = (h.z - G.ohz) + (l.z - G.olz);
        const float ex = fmaxf(fmaxf(G.a[0] - cx, cx - G.a[3]), 0.f);
        const float ey = fmaxf(fmaxf(G.a[1] - cy, cy - G.a[4]), 0.f);
        const float ez = fmaxf(fmaxf(G.a[2] - cz, cz - G.a[5]), 0.f);
        const float fx = fmaxf(fmaxf(G.b[0] - cx, cx - G.b[3]), 0.f);
        const float fy = fmaxf(fmaxf(G.b[1] - cy, cy - G.b[4]), 0.f);
        const float fz = fmaxf(fmaxf(G.b[2] - cz, cz - G.b[5]), 0.f);
        const float dmin2 = fminf(fmaf(ex, ex, fmaf(ey, ey, ez * ez)),
                                  fmaf(fx, fx, fmaf(fy, fy, fz * fz)));
        const bool take_m = has && !leaf && h.w < theta2 * dmin2;
        const bool open = has && !leaf && !take_m;
        const bool mine = has && leaf && ab.x >= G.g0 && ab.x < G.g1;
        const bool far = has && leaf && !mine;

        // opened nodes: both children, then the next wave's nodes and their records
        const uint32_t om = __ballot_sync(kFull, open);
        if (top + 2u * __popc(om) > stk_cap) {
            if (lane == 0) atomicOr(err, kErrStack);
            break;
        }
        if (open) {
            const uint32_t slot = top + 2u * __popc(om & lt);
            W.stk[slot] = ab.x;           // right child
            W.stk[slot + 1] = node + 1u;  // left child
        }
        top += 2u * __popc(om);
        __syncwarp();
        const uint32_t ntake = min(top, 32u);
        const bool nhas = (uint32_t)lane < ntake;
        const uint32_t nnode = nhas ? W.stk[top - 1 - lane] : 0u;
        top -= ntake;
        __syncwarp();
        float4 nh = make_float4(0.f, 0.f, 0.f, 0.f), nlo = nh;
        uint2 nab = make_uint2(0u, 0u);
        if (nhas) {
            nh = __ldg(&rec[nnode].hi);
            nlo = __ldg(&rec[nnode].lo);
            nab = __ldg(reinterpret_cast<const uint2 *>(&rec[nnode].a));
        }

        // accepted nodes: one entry each
        const uint32_t am = __ballot_sync(kFull, take_m);
        if (take_m) {
            const uint32_t k = nl + __popc(am & lt);
            put_entry<!kTgt>(W, k, cx, cy, cz, l.w);
            if (kTgt) W.tgt[k] = node | kNodeTarget;
        }
        nl += __popc(am);
        if (kCount) cnt[1] += __popc(am);
        // reached leaves: their bodies, the group's own leaves into their own list.  One
        // scan for both counts: far-leaf bodies in the low half, own in the high half (each
        // total is at most 32 * 8)
        const uint32_t fc = far ? ab.y : 0u, oc = mine ? ab.y : 0u;
        const uint32_t pi = warp_incl_scan(fc | (oc << 16), lane);
        const uint32_t pt = __shfl_sync(kFull, pi, 31);
        const uint32_t fi = pi & 0xffffu, oi = pi >> 16, ft = pt & 0xffffu, ot = pt >> 16;
        // the far leaves' bodies, written cooperatively: lane j of a round takes body j of
        // the wave, finds its leaf (the first lane whose inclusive count exceeds j) by binary
        // search, and writes the same entry, at the same place, the leaf's lane would
        for (uint32_t j0 = 0; j0 < ft; j0 += 32) {
            const uint32_t j = j0 + (uint32_t)lane;
            int q = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1) {
                const uint32_t v = __shfl_sync(kFull, fi, q + step - 1);
                if (v <= j) q += step;
            }
            const uint32_t first = __shfl_sync(kFull, ab.x, q);
            const uint32_t before = __shfl_sync(kFull, fi - fc, q);
            const float ox = __shfl_sync(kFull, cx, q), oy = __shfl_sync(kFull, cy, q),
                        oz = __shfl_sync(kFull, cz, q);
            if (j < ft) {
                const uint32_t body = first + (j - before);
                const float4 t = __ldg(&trel[body]);
                put_entry<!kTgt>(W, nl + j, ox + t.x, oy + t.y, oz + t.z, t.w);
                if (kTgt) W.tgt[nl + j] = body;
            }
        }
        if (mine) {
            const uint32_t o0 = nown + oi - oc;
            for (uint32_t k = 0; k < ab.y && o0 + k < (uint32_t)kGroupSinks; ++k) {
                const float4 hi = __ldg(&thi[ab.x + k]), lo = __ldg(&tlo[ab.x + k]);
                W.own[2 * (o0 + k)] = hi;
                W.own[2 * (o0 + k) + 1] = make_float4(lo.x, lo.y, lo.z, __uint_as_float(ab.x + k));
            }
        }
        nl += ft;
        nown = min(nown + ot, (uint32_t)kGroupSinks);
        if (kCount) cnt[0] += ft;
        __syncwarp();
        if (nl >= (uint32_t)kGroupFlush) {
            flush(nl);
            nl = 0;
            __syncwarp();
        }
        take = ntake;
        has = nhas;
        node = nnode;
        h = nh;
        l = nlo;
        ab = nab;
    }
    __syncwarp();
    if (nl) flush(nl);
    __syncwarp();
}

// Two list entries (packed source coordinates and masses) on one sink (q, packed
// twice): the pair kernel of one entry per half.
template <bool kPot>
__device__ __forceinline__ void pair_term2(f2 ex, f2 ey, f2 ez, f2 em, f2 qx, f2 qy, f2 qz,
                                           f2 &px, f2 &py, f2 &pz, f2 &pp) {
    const f2 dx = sub2(ex, qx), dy = sub2(ey, qy), dz = sub2(ez, qz);
    const f2 d2 = fma2(dx, dx, fma2(dy, dy, mul2(dz, dz)));
    float da, db;
    upk(d2, da, db);
    const f2 inv = pk(rsqrt_ftz(da), rsqrt_ftz(db));
    const f2 mi = mul2(em, inv);
    const f2 f = mul2(mi, mul2(inv, inv));
    px = fma2(f, dx, px);
    py = fma2(f, dy, py);
    pz = fma2(f, dz, pz);
    if (kPot) pp = add2(pp, mi);
}

// Sum of the entries [0, nl) (nl a multiple of 4) of the component arrays L on the lane's
// two sinks, two entries per packed instruction: plain FP32 partial sums over 64 entries
// (even entries in one half, odd in the other), each folded into the compensated sums.
template <bool kPot>
__device__ __forceinline__ void sum_list(const float *L, uint32_t nl, const Group &G,
                                         float (&s)[2][4], float (&c)[2][4]) {
    f2 qx[2], qy[2], qz[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
        qx[u] = pk(G.qx[u], G.qx[u]);
        qy[u] = pk(G.qy[u], G.qy[u]);
        qz[u] = pk(G.qz[u], G.qz[u]);
    }
    for (uint32_t k0 = 0; k0 < nl; k0 += 64) {
        const uint32_t k1 = min(nl, k0 + 64u);
        f2 px[2] = {0ull, 0ull}, py[2] = {0ull, 0ull}, pz[2] = {0ull, 0ull},
           pp[2] = {0ull, 0ull};  // 0 bits: +0.0f in both halves
#pragma unroll 2
        for (uint32_t k = k0; k < k1; k += 4) {
            const float4 x = *reinterpret_cast<const float4 *>(L + k);
            const float4 y = *reinterpret_cast<const float4 *>(L + kGroupListCap + k);
            const float4 z = *reinterpret_cast<const float4 *>(L + 2 * kGroupListCap + k);
            const float4 m = *reinterpret_cast<const float4 *>(L + 3 * kGroupListCap + k);
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                pair_term2<kPot>(pk(x.x, x.y), pk(y.x, y.y), pk(z.x, z.y), pk(m.x, m.y), qx[u],
                                 qy[u], qz[u], px[u], py[u], pz[u], pp[u]);
                pair_term2<kPot>(pk(x.z, x.w), pk(y.z, y.w), pk(z.z, z.w), pk(m.z, m.w), qx[u],
                                 qy[u], qz[u], px[u], py[u], pz[u], pp[u]);
            }
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            float a, b;
            upk(px[u], a, b);
            kahan(s[u][0], c[u][0], a + b);
            upk(py[u], a, b);
            kahan(s[u][1], c[u][1], a + b);
            upk(pz[u], a, b);
            kahan(s[u][2], c[u][2], a + b);
            if (kPot) {
                upk(pp[u], a, b);
                kahan(s[u][3], c[u][3], -(a + b));
            }
        }
    }
}

// w = |d|^-3 (mu - 3 (d . mu) |d|^-2 d), d = sink - source: the tidal tensor times mu,
// returned as the factor inv3 = |d|^-3 and the vector v = w / inv3.
__device__ __forceinline__ void tidal_v(float dx, float dy, float dz, float mx, float my,
                                        float mz, float &inv3, float &vx, float &vy,
                                        float &vz) {
    const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    const float inv = rsqrt_ftz(d2);
    const float inv2 = inv * inv;
    inv3 = inv2 * inv;
    const float dm = fmaf(dx, mx, fmaf(dy, my, dz * mz));
    const float c3 = 3.0f * dm * inv2;
    vx = fmaf(-c3, dx, mx);
    vy = fmaf(-c3, dy, my);
    vz = fmaf(-c3, dz, mz);
}

// Adjoint terms of 32 sources (padding sources far away with zero mass) against the warp's
// 64 sinks by rotation: the sink terms -m w into the compensated sums (sum, comp), folded
// every 8 steps, and lane l returns the sum over the sinks of w for source l.
// `pair(slot, dx, dy, dz, m)` gives, for both of the lane's sinks, the separation
// sink - source and the source mass (zero where the pair does not exist).
template <typename Pair>
__device__ __forceinline__ void rotate32(int lane, const float (&mx)[2], const float (&my)[2],
                                         const float (&mz)[2], float (&sum)[2][3],
                                         float (&comp)[2][3], float &ax, float &ay, float &az,
                                         Pair &&pair) {
    ax = ay = az = 0.f;
    const int up = (lane + 1) & 31;
#pragma unroll 1
    for (int k0 = 0; k0 < 32; k0 += 8) {
        float px[2] = {0.f, 0.f}, py[2] = {0.f, 0.f}, pz[2] = {0.f, 0.f};
#pragma unroll
        for (int k = k0; k < k0 + 8; ++k) {
            float dx[2], dy[2], dz[2], m[2];
            pair((lane + k) & 31, dx, dy, dz, m);
            float bx = ax, by = ay, bz = az;
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                float inv3, vx, vy, vz;
                tidal_v(dx[u], dy[u], dz[u], mx[u], my[u], mz[u], inv3, vx, vy, vz);
                const float sm = -m[u] * inv3;
                px[u] = fmaf(sm, vx, px[u]);
                py[u] = fmaf(sm, vy, py[u]);
                pz[u] = fmaf(sm, vz, pz[u]);
                bx = fmaf(inv3, vx, bx);
                by = fmaf(inv3, vy, by);
                bz = fmaf(inv3, vz, bz);
            }
            ax = __shfl_sync(kFull, bx, up);
            ay = __shfl_sync(kFull, by, up);
            az = __shfl_sync(kFull, bz, up);
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            kahan(sum[u][0], comp[u][0], px[u]);
            kahan(sum[u][1], comp[u][1], py[u]);
            kahan(sum[u][2], comp[u][2], pz[u]);
        }
    }
}

}  // namespace

// FP64 mass of the body at tree position s: the light mass as split hi + lo, or, for a heavy
// body (light mass 0), its own mass.
__device__ __forceinline__ double body_mass(const float4 &mh, const float4 &ml, uint32_t o,
                                            const uint32_t *heavy_ids, const Heavy *heavy,
                                            int n_heavy) {
    double m = (double)mh.w + (double)ml.w;
    for (int hh = 0; hh < n_heavy; ++hh)
        if (heavy_ids[hh] == o) m = heavy[hh].m;
    return m;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

constexpr uint32_t kNoBody = 0xffffffffu;

// 1/sqrt(x) from the FP32 hardware estimate and one FP64 Newton step (relative error about
// 1.5 * (2^-22.9)^2, ~3e-14): the mixed path's heavy-body terms, which the FP32 pair sums
// around them bound far more loosely.  Outside [1e-30, 1e30] by square root and division.
__device__ __forceinline__ double inv_dist1(double x) {
    if (!(x >= 1e-30 && x <= 1e30)) return __ddiv_rn(1.0, __dsqrt_rn(x));
    float f;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(f) : "f"((float)x));
    const double y = (double)f;
    return y * fma(-0.5 * x * y, y, 1.5);
}

// The end of a group's walk for the lane's two sinks (body o0 / o1 at tree positions s0 / s1,
// kNoBody when the lane has none): the heavy bodies in FP64, both ways of every (sink,
// heavy) pair -- the heavy body's pull on the sink (the pair kernel of array_particle.rs:67-76
// with 1/|d| from inv_dist1 in place of the square root and division), and the sink's pull on
// the heavy body, whose sum over all bodies is the heavy body's own direct-sum acceleration
// (its grouped-walk value, a residual of cancelling FP32 terms, is replaced by
// k_heavy_finish) -- the warp's share of those sums into its own slot of hpart, and the
// accelerations (and potentials) out.
template <bool kPot>
__device__ __noinline__ void heavy_tail(uint32_t o0, uint32_t o1, uint32_t s0, uint32_t s1,
                                        double ax0, double ay0, double az0, double ph0,
                                        double ax1, double ay1, double az1, double ph1,
                                        const float4 *__restrict__ thi,
                                        const float4 *__restrict__ tlo,
                                        const double *__restrict__ bx,
                                        const double *__restrict__ by,
                                        const double *__restrict__ bz,
                                        const uint32_t *__restrict__ heavy_ids,
                                        const Heavy *heavy, int n_heavy, double *__restrict__ acc,
                                        double *__restrict__ phi, double *__restrict__ hpart,
                                        uint32_t g, uint32_t n_groups, int lane) {
    const uint32_t o[2] = {o0, o1}, sp[2] = {s0, s1};
    double ax[2] = {ax0, ax1}, ay[2] = {ay0, ay1}, az[2] = {az0, az1}, ph[2] = {ph0, ph1};
    double px[2], py[2], pz[2], ms[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
        px[u] = py[u] = pz[u] = ms[u] = 0.0;
        if (o[u] != kNoBody && n_heavy > 0) {
            px[u] = bx[o[u]];
            py[u] = by[o[u]];
            pz[u] = bz[o[u]];
            ms[u] = body_mass(thi[sp[u]], tlo[sp[u]], o[u], heavy_ids, heavy, n_heavy);
        }
    }
    for (int hh = 0; hh < n_heavy; ++hh) {  // warp-uniform
        const Heavy q = heavy[hh];
        double rx = 0.0, ry = 0.0, rz = 0.0, rp = 0.0;
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            if (o[u] == kNoBody || heavy_ids[hh] == o[u]) continue;
            const double dx = px[u] - q.x, dy = py[u] - q.y, dz = pz[u] - q.z;
            const double ri = inv_dist1(fma(dx, dx, fma(dy, dy, dz * dz)));
            const double ri3 = ri * ri * ri;
            const double magi = -q.m * ri3;
            ax[u] = fma(magi, dx, ax[u]);
            ay[u] = fma(magi, dy, ay[u]);
            az[u] = fma(magi, dz, az[u]);
            if (kPot) ph[u] -= q.m * ri;
            const double mr = ms[u] * ri3;
            rx = fma(mr, dx, rx);
            ry = fma(mr, dy, ry);
            rz = fma(mr, dz, rz);
            if (kPot) rp -= ms[u] * ri;
        }
        rx = warp_sum(rx);
        ry = warp_sum(ry);
        rz = warp_sum(rz);
        if (kPot) rp = warp_sum(rp);
        if (lane == 0) {
            double *slot = hpart + ((size_t)hh * n_groups + g) * 4;
            slot[0] = rx;
            slot[1] = ry;
            slot[2] = rz;
            slot[3] = rp;
        }
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
        if (o[u] == kNoBody) continue;
        acc[3 * (size_t)o[u]] = ax[u];
        acc[3 * (size_t)o[u] + 1] = ay[u];
        acc[3 * (size_t)o[u] + 2] = az[u];
        if (kPot) phi[o[u]] = ph[u];
    }
}

// One warp's group: the walk, the group's own leaves, the heavy bodies' FP64 terms on the
// group's sinks, and the group's share (hpart[heavy][group][x, y, z, potential]) of the
// heavy bodies' own direct sums.
template <bool kCount, bool kPot>
__device__ __forceinline__ void walk_group_warp(
    const NodeF *__restrict__ rec, const float4 *__restrict__ thi,
    const float4 *__restrict__ tlo, const float4 *__restrict__ trel,
    const uint32_t *__restrict__ tid, const uint32_t *__restrict__ gstart,
    const uint32_t *__restrict__ gsplit, uint32_t g, uint32_t stk_cap, float theta2,
    const Bodies &b, const uint32_t *__restrict__ heavy_ids, const Heavy *heavy, int n_heavy,
    double *__restrict__ acc, double *__restrict__ phi, uint32_t *err,
    unsigned long long *counts, float4 *smem, double *__restrict__ hpart, uint32_t n_groups,
    int lane, int warp) {
    const WarpMem W = warp_mem(smem, warp, stk_cap, false);
    const Group G = make_group(thi, tlo, gstart[g], gstart[g + 1], gsplit[g], lane);

    float sum[2][4] = {}, comp[2][4] = {};
    uint32_t nown = 0;
    unsigned long long cnt[3] = {0, 0, 0};  // pair entries, node entries, node tests
    traverse<false, kCount>(rec, trel, thi, tlo, G, W, stk_cap, theta2, lane, err, nown, cnt,
                            [&](uint32_t nl) {
                                // padded to a multiple of 4 with entries that add nothing
                                // (nl < kGroupFlush + 32 * 8, so the padding stays inside)
                                const uint32_t n4 = (nl + 3u) & ~3u;
                                if ((uint32_t)lane < n4 - nl)
                                    put_entry<true>(W, nl + lane, kFar, kFar, kFar, 0.f);
                                __syncwarp();
                                sum_list<kPot>(reinterpret_cast<const float *>(W.list), n4, G,
                                               sum, comp);
                            });
    // the group's own leaves, self excluded by tree position, separations from the split
    // absolute positions
#pragma unroll
    for (int u = 0; u < 2; ++u) {
        const float4 mh = thi[G.s[u]], ml = tlo[G.s[u]];
        float px = 0.f, py = 0.f, pz = 0.f, pp = 0.f;
        for (uint32_t k = 0; k < nown; ++k) {
            const float4 eh = W.own[2 * k], el = W.own[2 * k + 1];
            if (__float_as_uint(el.w) == G.s[u]) continue;
            const float dx = (eh.x - mh.x) + (el.x - ml.x);
            const float dy = (eh.y - mh.y) + (el.y - ml.y);
            const float dz = (eh.z - mh.z) + (el.z - ml.z);
            const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            const float inv = rsqrt_ftz(d2);
            const float mi = eh.w * inv;
            const float f = mi * (inv * inv);
            px = fmaf(f, dx, px);
            py = fmaf(f, dy, py);
            pz = fmaf(f, dz, pz);
            if (kPot) pp += mi;
        }
        kahan(sum[u][0], comp[u][0], px);
        kahan(sum[u][1], comp[u][1], py);
        kahan(sum[u][2], comp[u][2], pz);
        if (kPot) kahan(sum[u][3], comp[u][3], -pp);
    }
    // the heavy-body terms and the result, in a separate (not inlined) function so that the
    // walk's hot loops above are allocated registers without them
    heavy_tail<kPot>(G.valid[0] ? tid[G.s[0]] : kNoBody, G.valid[1] ? tid[G.s[1]] : kNoBody,
                     G.s[0], G.s[1], (double)sum[0][0] - (double)comp[0][0],
                     (double)sum[0][1] - (double)comp[0][1],
                     (double)sum[0][2] - (double)comp[0][2],
                     (double)sum[0][3] - (double)comp[0][3],
                     (double)sum[1][0] - (double)comp[1][0],
                     (double)sum[1][1] - (double)comp[1][1],
                     (double)sum[1][2] - (double)comp[1][2],
                     (double)sum[1][3] - (double)comp[1][3], thi, tlo, b.x, b.y, b.z,
                     heavy_ids, heavy, n_heavy, acc, phi, hpart, g, n_groups, lane);
    if (kCount && lane == 0) {
        const unsigned long long nv = G.g1 - G.g0;
        // the own leaves hold every body of the group (each reached once)
        const unsigned long long own_pairs = nown >= nv ? nv * (nown - 1) : nv * nown;
        atomicAdd(&counts[0], nv * cnt[0] + own_pairs);
        atomicAdd(&counts[1], cnt[2]);
        atomicAdd(&counts[2], nv * cnt[1]);
        atomicAdd(&counts[3], nv * cnt[2]);
    }
}

static_assert(kGroupWarps * 32 >= kMaxHeavy, "a block loads the heavy bodies");
// 16 warps per SM (128 registers)
template <bool kCount, bool kPot>
__global__ __launch_bounds__(kGroupWarps * 32, 16 / kGroupWarps) void k_walk_group(
    const NodeF *__restrict__ rec, const float4 *__restrict__ thi,
    const float4 *__restrict__ tlo, const float4 *__restrict__ trel,
    const uint32_t *__restrict__ tid, const uint32_t *__restrict__ gstart,
    const uint32_t *__restrict__ gsplit, uint32_t n_groups, uint32_t stk_cap, float theta2,
    Bodies b, const uint32_t *__restrict__ heavy_ids, int n_heavy, double *__restrict__ acc,
    double *__restrict__ phi, double *__restrict__ hpart, uint32_t *err,
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
    // no block barrier follows: a warp whose group is done exits (a trailing barrier, which
    // held finished warps until the block's slowest, cost 7% of the walk)
    if (g >= n_groups) return;
    walk_group_warp<kCount, kPot>(rec, thi, tlo, trel, tid, gstart, gsplit, g, stk_cap, theta2,
                                  b, heavy_ids, heavy, n_heavy, acc, phi, err, counts, smem,
                                  hpart, n_groups, lane, warp);
}

// The heavy bodies' accelerations (and potentials) as FP64 direct sums over every other
// body, from the groups' partial sums (hpart[heavy][group][4]): block q of heavy body h adds
// groups [q * chunk, (q + 1) * chunk) in a fixed order (strided per thread, then the warps'
// butterflies, then the warps in order) into hpart's block area; the last block of h to
// finish adds the kFinishBlocks block sums in order.  Deterministic for a given n; overwrites
// what the grouped walk wrote for the heavy body.  `count` (kMaxHeavy words, zero between
// launches) counts the finished blocks of each heavy body.
__global__ __launch_bounds__(kFinishThreads) void k_heavy_finish(
    double *__restrict__ hpart, uint32_t n_groups, const uint32_t *__restrict__ heavy_ids,
    uint32_t *count, double *__restrict__ acc, double *__restrict__ phi,
    double *__restrict__ out3) {
    __shared__ double red[4][kFinishThreads / 32];
    __shared__ bool last;
    const int hh = blockIdx.y, q = blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const double *src = hpart + (size_t)hh * n_groups * 4;
    double *blk = hpart + (size_t)kMaxHeavy * n_groups * 4 + ((size_t)hh * kFinishBlocks) * 4;
    const uint32_t chunk = (n_groups + kFinishBlocks - 1) / kFinishBlocks;
    const uint32_t g0 = min(n_groups, (uint32_t)q * chunk), g1 = min(n_groups, g0 + chunk);
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for (uint32_t g = g0 + threadIdx.x; g < g1; g += kFinishThreads) {
        const dbl4 t = *reinterpret_cast<const dbl4 *>(src + (size_t)g * 4);
        v[0] += t.x;
        v[1] += t.y;
        v[2] += t.z;
        v[3] += t.w;
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        v[c] = warp_sum(v[c]);
        if (lane == 0) red[c][warp] = v[c];
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double t = 0.0;
        for (int w = 0; w < kFinishThreads / 32; ++w) t += red[threadIdx.x][w];
        blk[(size_t)q * 4 + threadIdx.x] = t;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(&count[hh], 1u) == kFinishBlocks - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    if (threadIdx.x < 4) {
        double t = 0.0;
        for (int k = 0; k < kFinishBlocks; ++k) t += __ldcg(&blk[(size_t)k * 4 + threadIdx.x]);
        const size_t o = heavy_ids[hh];
        if (out3) {  // the adjoint's heavy source sums
            if (threadIdx.x < 3) out3[3 * hh + threadIdx.x] = t;
        } else if (threadIdx.x < 3) {
            acc[3 * o + threadIdx.x] = t;
        } else if (phi) {
            phi[o] = t;
        }
        if (threadIdx.x == 0) count[hh] = 0u;
    }
}

// Transpose-Jacobian product of one step over the grouped interaction set.  Per sink s:
// ysink_s (tree order) = -sum m w + the FP64 heavy-body terms; per list entry the sum over
// the group's sinks of w goes to U (a body, tree order) or G (a node); the heavy bodies'
// source sums go to yheavy.
// 12 warps per SM
__global__ __launch_bounds__(kGroupWarps * 32, 12 / kGroupWarps) void k_adj_group(
    const NodeF *__restrict__ rec, const float4 *__restrict__ thi,
    const float4 *__restrict__ tlo, const float4 *__restrict__ trel,
    const uint32_t *__restrict__ tid, const uint32_t *__restrict__ gstart,
    const uint32_t *__restrict__ gsplit, uint32_t n_groups, uint32_t stk_cap, float theta2,
    Bodies b, const uint32_t *__restrict__ heavy_ids, int n_heavy,
    const double *__restrict__ mu, double *__restrict__ ysink, double *__restrict__ U,
    double *__restrict__ Gn, double *__restrict__ hpart, uint32_t *err) {
    extern __shared__ float4 smem[];
    __shared__ Heavy heavy[kMaxHeavy];
    __shared__ double hmu[kMaxHeavy][3];
    if (threadIdx.x < n_heavy) {
        const uint32_t h = heavy_ids[threadIdx.x];
        heavy[threadIdx.x] = Heavy{b.x[h], b.y[h], b.z[h], b.m[h]};
        hmu[threadIdx.x][0] = mu[3 * (size_t)h];
        hmu[threadIdx.x][1] = mu[3 * (size_t)h + 1];
        hmu[threadIdx.x][2] = mu[3 * (size_t)h + 2];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t g = blockIdx.x * kGroupWarps + warp;
    double hx[kMaxHeavy][3];
#pragma unroll
    for (int h = 0; h < kMaxHeavy; ++h) hx[h][0] = hx[h][1] = hx[h][2] = 0.0;
    if (g >= n_groups) return;  // warp-uniform; no block barrier follows
    {
        const WarpMem W = warp_mem(smem, warp, stk_cap, true);
        const Group G = make_group(thi, tlo, gstart[g], gstart[g + 1], gsplit[g], lane);
        // sinks without a body sit far away with mu = 0: every term they make is zero.  A
        // heavy sink's row is its direct sum (below), so it takes no part in the rotation.
        float mx[2], my[2], mz[2], qx[2], qy[2], qz[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            mx[u] = my[u] = mz[u] = 0.f;
            if (G.valid[u] && !is_heavy(tid[G.s[u]], heavy_ids, n_heavy)) {
                const size_t o = tid[G.s[u]];
                mx[u] = (float)mu[3 * o];
                my[u] = (float)mu[3 * o + 1];
                mz[u] = (float)mu[3 * o + 2];
            }
            qx[u] = G.valid[u] ? G.qx[u] : -kFar;
            qy[u] = G.valid[u] ? G.qy[u] : -kFar;
            qz[u] = G.valid[u] ? G.qz[u] : -kFar;
        }
        float sum[2][3] = {}, comp[2][3] = {};
        uint32_t nown = 0;
        unsigned long long cnt[3] = {0, 0, 0};
        traverse<true, false>(
            rec, trel, thi, tlo, G, W, stk_cap, theta2, lane, err, nown, cnt, [&](uint32_t nl) {
                const uint32_t nr = (nl + 31u) & ~31u;
                if ((uint32_t)lane < nr - nl) {
                    W.list[nl + lane] = make_float4(kFar, kFar, kFar, 0.f);
                    W.tgt[nl + lane] = kNoTarget;
                }
                __syncwarp();
                for (uint32_t k0 = 0; k0 < nr; k0 += 32) {
                    float ax, ay, az;
                    const float4 *e = W.list + k0;
                    rotate32(lane, mx, my, mz, sum, comp, ax, ay, az,
                             [&](int slot, float(&dx)[2], float(&dy)[2], float(&dz)[2],
                                 float(&m)[2]) {
                                 const float4 c = e[slot];
#pragma unroll
                                 for (int u = 0; u < 2; ++u) {
                                     dx[u] = qx[u] - c.x;
                                     dy[u] = qy[u] - c.y;
                                     dz[u] = qz[u] - c.z;
                                     m[u] = c.w;
                                 }
                             });
                    const uint32_t t = W.tgt[k0 + lane];
                    if (t != kNoTarget) {
                        double *dst = (t & kNodeTarget) ? Gn + 3 * (size_t)(t & ~kNodeTarget)
                                                        : U + 3 * (size_t)t;
                        atomicAdd(dst, (double)ax);
                        atomicAdd(dst + 1, (double)ay);
                        atomicAdd(dst + 2, (double)az);
                    }
                }
            });
        // the group's own leaves: pairs among the group's bodies, self excluded, separations
        // from the split absolute positions; own entries in blocks of 32, padded far away
        {
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const uint32_t k = lane + 32 * u;
                if (k >= nown) {
                    W.own[2 * k] = make_float4(kFar, kFar, kFar, 0.f);
                    W.own[2 * k + 1] = make_float4(0.f, 0.f, 0.f, __uint_as_float(kNoTarget));
                }
            }
            __syncwarp();
            // sinks without a body sit far away on the other side: no pair reaches zero
            float4 mh[2], ml[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                mh[u] = G.valid[u] ? thi[G.s[u]] : make_float4(-kFar, -kFar, -kFar, 0.f);
                ml[u] = G.valid[u] ? tlo[G.s[u]] : make_float4(0.f, 0.f, 0.f, 0.f);
            }
            for (uint32_t k0 = 0; k0 < nown; k0 += 32) {
                const float4 *own = W.own + 2 * k0;
                float ax, ay, az;
                rotate32(lane, mx, my, mz, sum, comp, ax, ay, az,
                         [&](int slot, float(&dx)[2], float(&dy)[2], float(&dz)[2],
                             float(&m)[2]) {
                             const float4 eh = own[2 * slot], el = own[2 * slot + 1];
#pragma unroll
                             for (int u = 0; u < 2; ++u) {
                                 if (__float_as_uint(el.w) == G.s[u] && G.valid[u]) {
                                     dx[u] = dy[u] = dz[u] = kFar;
                                     m[u] = 0.f;
                                 } else {
                                     dx[u] = (mh[u].x - eh.x) + (ml[u].x - el.x);
                                     dy[u] = (mh[u].y - eh.y) + (ml[u].y - el.y);
                                     dz[u] = (mh[u].z - eh.z) + (ml[u].z - el.z);
                                     m[u] = eh.w;
                                 }
                             }
                         });
                const uint32_t t = __float_as_uint(own[2 * lane + 1].w);
                if (t != kNoTarget) {
                    atomicAdd(&U[3 * (size_t)t], (double)ax);
                    atomicAdd(&U[3 * (size_t)t + 1], (double)ay);
                    atomicAdd(&U[3 * (size_t)t + 2], (double)az);
                }
            }
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            if (!G.valid[u]) continue;
            const uint32_t s = G.s[u];
            const size_t o = tid[s];
            const double mux = mu[3 * o], muy = mu[3 * o + 1], muz = mu[3 * o + 2];
            double ysx = (double)sum[u][0] - (double)comp[u][0];
            double ysy = (double)sum[u][1] - (double)comp[u][1];
            double ysz = (double)sum[u][2] - (double)comp[u][2];
            // Heavy bodies in FP64, sink side here, source side reduced over the block.  Two
            // rows meet in every (body o, heavy h) pair: o's row with source h (for a light o;
            // a heavy o's row is its direct sum), and h's direct-sum row with source o.
            const double X = b.x[o], Y = b.y[o], Z = b.z[o];
            const bool o_heavy = is_heavy((uint32_t)o, heavy_ids, n_heavy);
            const double mo = n_heavy > 0 ? body_mass(thi[s], tlo[s], (uint32_t)o, heavy_ids,
                                                      heavy, n_heavy)
                                          : 0.0;
#pragma unroll
            for (int h = 0; h < kMaxHeavy; ++h) {
                if (h >= n_heavy || heavy_ids[h] == o) continue;
                const Heavy q = heavy[h];
                const double dx = X - q.x, dy = Y - q.y, dz = Z - q.z;
                const double ri = inv_dist(fma(dx, dx, fma(dy, dy, dz * dz)));
                const double inv2 = ri * ri;
                const double inv3 = inv2 * ri;
                if (!o_heavy) {
                    const double dm = dx * mux + dy * muy + dz * muz;
                    const double c3 = 3.0 * dm * inv2;
                    const double wx = inv3 * (mux - c3 * dx), wy = inv3 * (muy - c3 * dy),
                                 wz = inv3 * (muz - c3 * dz);
                    ysx -= q.m * wx;
                    ysy -= q.m * wy;
                    ysz -= q.m * wz;
                    hx[h][0] += q.m * wx;
                    hx[h][1] += q.m * wy;
                    hx[h][2] += q.m * wz;
                }
                const double hmx = hmu[h][0], hmy = hmu[h][1], hmz = hmu[h][2];
                const double dh = dx * hmx + dy * hmy + dz * hmz;
                const double ch = 3.0 * dh * inv2;
                const double vx = inv3 * (hmx - ch * dx), vy = inv3 * (hmy - ch * dy),
                             vz = inv3 * (hmz - ch * dz);
                ysx += mo * vx;
                ysy += mo * vy;
                ysz += mo * vz;
                hx[h][0] -= mo * vx;
                hx[h][1] -= mo * vy;
                hx[h][2] -= mo * vz;
            }
            ysink[3 * (size_t)s] = ysx;
            ysink[3 * (size_t)s + 1] = ysy;
            ysink[3 * (size_t)s + 2] = ysz;
        }
    }
    // the group's share of the heavy bodies' source sums, into its own slot of hpart (added up
    // by k_heavy_finish: no block barrier, so a finished warp exits)
#pragma unroll
    for (int h = 0; h < kMaxHeavy; ++h) {
        if (h >= n_heavy) break;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            double val = hx[h][d];
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) val += __shfl_xor_sync(kFull, val, off);
            if (lane == 0) hpart[((size_t)h * n_groups + g) * 4 + d] = val;
        }
        if (lane == 0) hpart[((size_t)h * n_groups + g) * 4 + 3] = 0.0;
    }
}

int launch_walk_group(const NodeF *rec, const float4 *thi, const float4 *tlo,
                      const float4 *trel, const uint32_t *tid, const uint32_t *gstart,
                      const uint32_t *gsplit, uint32_t n_groups, uint32_t stk_cap, double theta,
                      const Bodies &b, const uint32_t *heavy_ids, int n_heavy, double *acc,
                      double *hpart, uint32_t *hcount, uint32_t *err,
                      unsigned long long *counts, cudaStream_t st, double *phi) {
    const uint32_t threads = kGroupWarps * 32;
    const uint32_t blocks = walk_group_blocks(n_groups);
    const size_t smem = (size_t)kGroupWarps * group_warp_bytes(stk_cap);
    const float theta2 = (float)(theta * theta);
    auto k = phi ? k_walk_group<false, true>
                 : (counts ? k_walk_group<true, false> : k_walk_group<false, false>);
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k<<<blocks, threads, smem, st>>>(rec, thi, tlo, trel, tid, gstart, gsplit, n_groups, stk_cap,
                                     theta2, b, heavy_ids, n_heavy, acc, phi, hpart, err,
                                     counts);
    if (n_heavy <= 0) return 1;
    k_heavy_finish<<<dim3(kFinishBlocks, n_heavy), kFinishThreads, 0, st>>>(
        hpart, n_groups, heavy_ids, hcount, acc, phi, nullptr);
    return 2;
}

void launch_adj_group(const AdjArgs &a, cudaStream_t st) {
    const uint32_t threads = kGroupWarps * 32;
    const uint32_t blocks = (a.n_groups + kGroupWarps - 1) / kGroupWarps;
    const size_t smem = (size_t)kGroupWarps *
                        (group_warp_bytes(a.stk_cap) + kGroupListCap * sizeof(uint32_t));
    cudaFuncSetAttribute(k_adj_group, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_adj_group<<<blocks, threads, smem, st>>>(
        a.recf, a.thi, a.tlo, a.trel, a.tid, a.gstart, a.gsplit, a.n_groups, a.stk_cap,
        (float)(a.theta * a.theta), a.bodies, a.heavy, a.n_heavy, a.mu, a.ysink, a.U, a.G,
        a.hpart, a.err);
    if (a.n_heavy > 0)
        k_heavy_finish<<<dim3(kFinishBlocks, a.n_heavy), kFinishThreads, 0, st>>>(
            a.hpart, a.n_groups, a.heavy, a.hcount, nullptr, nullptr, a.yheavy);
}

}  // namespace kd
