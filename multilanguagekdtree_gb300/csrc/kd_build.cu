// kd_build.cu -- GPU construction of the reference's median-split kD-tree.
//
// What it reproduces (MarkCLewis/MultiLanguageKDTree, Parallel/RustVersion/src/
// array_kd_tree.rs:515-583 build_tree_par4 and :63-130 build_tree):
//   * a segment of more than `leaf` bodies is split at mid = len/2; the left child holds the
//     len/2 bodies with the smallest coordinate along split_dim (quickstat_index post
//     condition, quickstat.rs:9-34 and its test :211-216) and split_val is the coordinate
//     of the body at mid;
//   * split_dim is the dimension of largest extent of the segment's bounding box taken
//     from +-1e100, strict > from dim 0 (array_kd_tree.rs:532-557), size = that extent.
// Because every split is an exact median, the tree's shape and every segment [start, end)
// depend on n alone; the host precomputes them.  Which bodies fill a segment is decided
// here, bit-exactly, by an exact rank select on the total order (coordinate, body index)
// -- the body index only matters for equal coordinates, where the reference's own choice
// depends on its random pivots.
//
// Structure: levels whose segments exceed kLocalMax bodies run as multi-block passes
// (bounding box -> split -> exact median select -> stable partition into the other
// ping-pong buffer, which also reduces the children's bounding boxes), except the last two
// of them, which one block per segment does in shared memory with one read and one write of
// the bodies (k_pair); below that, one thread block takes a whole segment into shared memory
// and finishes its subtree there (per-dimension sorted lists: bounds and medians read off the
// lists, one segmented stable partition of the lists per level).
#include "kd_internal.cuh"

namespace kd {

static constexpr uint32_t kFull = 0xffffffffu;

// Order-preserving map double -> uint64 (no NaN reaches the build).  -0.0 and +0.0 compare
// equal under the reference's `<`, so both get the key of +0.0.  Integer operations only:
// on this GPU every FP64 instruction, compares and min/max included, runs on the narrow
// FP64 pipe, so the build orders, bounds and bins bodies through these keys.
__device__ __forceinline__ unsigned long long ord_key(double v) {
    unsigned long long b = (unsigned long long)__double_as_longlong(v);
    if ((b << 1) == 0ull) b = 0ull;
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// Monotone (non-decreasing) double -> float by truncating the mantissa, flushing magnitudes
// below the float range to zero and saturating above it; integer operations only.
__device__ __forceinline__ float trunc_float(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const uint32_t sign = (uint32_t)(b >> 63) << 31;
    const int e = (int)((b >> 52) & 0x7ff) - 1023 + 127;
    uint32_t fb;
    if (e >= 255)
        fb = 0x7f800000u;
    else if (e <= 0)
        fb = 0u;
    else
        fb = ((uint32_t)e << 23) | (uint32_t)((b >> 29) & 0x7fffffu);
    return __uint_as_float(fb | sign);
}
__device__ __forceinline__ double ord_val(unsigned long long k) {
    unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double((long long)b);
}

// Split dimension and size from a bounding box, as array_kd_tree.rs:532-557: the box starts
// at +-1e100, the extent is max - min in FP64, the first strictly larger extent wins.  The
// comparison is decided on FP32 estimates of the extents whenever their error bounds
// separate them, so FP64 instructions run only for `size` and for near ties.
__device__ __forceinline__ void choose_split(const double mn_in[3], const double mx_in[3],
                                             uint32_t &sd, double &size) {
    double mn[3], mx[3];
    float ef[3], er[3];
    bool ok = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        // clamps at +-1e100 on order-preserving keys (integer operations)
        mn[d] = ord_val(min(ord_key(mn_in[d]), ord_key(1e100)));
        mx[d] = ord_val(max(ord_key(mx_in[d]), ord_key(-1e100)));
        const float a = trunc_float(mx[d]), b = trunc_float(mn[d]);
        ef[d] = a - b;
        er[d] = 2.4e-7f * (fabsf(a) + fabsf(b)) + 1.2e-7f * fabsf(ef[d]);
        ok = ok && isfinite(ef[d]) && isfinite(er[d]);
    }
    // the current winner is carried in scalars (no array indexed at run time)
    sd = 0;
    float bef = ef[0], ber = er[0];
    double bmx = mx[0], bmn = mn[0];
#pragma unroll
    for (int d = 1; d < 3; ++d) {
        bool gt;
        if (ok && ef[d] - er[d] > bef + ber)
            gt = true;
        else if (ok && ef[d] + er[d] < bef - ber)
            gt = false;
        else
            gt = __dsub_rn(mx[d], mn[d]) > __dsub_rn(bmx, bmn);
        if (gt) {
            sd = (uint32_t)d;
            bef = ef[d];
            ber = er[d];
            bmx = mx[d];
            bmn = mn[d];
        }
    }
    size = __dsub_rn(bmx, bmn);
}

__device__ __forceinline__ const double *pick(const double *x, const double *y,
                                              const double *z, uint32_t d) {
    return d == 0 ? x : (d == 1 ? y : z);
}

// In-place bitonic sort of `total` (key, val) pairs made of independent power-of-two
// blocks of length P, ascending by (key, val).  Caller synchronises before the call.
__device__ void bitonic_blocks(unsigned long long *key, unsigned long long *val,
                               uint32_t total, uint32_t P) {
    const uint32_t half = total >> 1;
    for (uint32_t k = 2; k <= P; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t q = threadIdx.x; q < half; q += blockDim.x) {
                uint32_t t = ((q & ~(j - 1)) << 1) | (q & (j - 1));
                uint32_t p = t | j;
                bool asc = (k == P) || ((t & k) == 0);
                unsigned long long ka = key[t], kb = key[p];
                unsigned long long va = val[t], vb = val[p];
                bool gt = (ka > kb) || (ka == kb && va > vb);
                if (gt == asc) {
                    key[t] = kb; key[p] = ka;
                    val[t] = vb; val[p] = va;
                }
            }
            __syncthreads();
        }
    }
}

__device__ __forceinline__ uint32_t next_pow2(uint32_t v) {
    return v <= 1 ? 1u : (1u << (32 - __clz(v - 1)));
}

// ------------------------------------------------------------------ work init

template <typename T>
__device__ __forceinline__ T warp_min(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(kFull, v, o));
    return v;
}
template <typename T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(kFull, v, o));
    return v;
}
// 64-bit keys: minimum (maximum) of the high words, then of the low words among the lanes
// that hold it -- two warp reductions instead of a five-step shuffle tree of 64-bit values.
__device__ __forceinline__ unsigned long long warp_min(unsigned long long v) {
    const uint32_t hi = (uint32_t)(v >> 32), lo = (uint32_t)v;
    const uint32_t mh = __reduce_min_sync(kFull, hi);
    const uint32_t ml = __reduce_min_sync(kFull, hi == mh ? lo : 0xffffffffu);
    return ((unsigned long long)mh << 32) | ml;
}
__device__ __forceinline__ unsigned long long warp_max(unsigned long long v) {
    const uint32_t hi = (uint32_t)(v >> 32), lo = (uint32_t)v;
    const uint32_t mh = __reduce_max_sync(kFull, hi);
    const uint32_t ml = __reduce_max_sync(kFull, hi == mh ? lo : 0u);
    return ((unsigned long long)mh << 32) | ml;
}
// The build's first work arrays (positions and body ids in original order; skipped when wx is
// null, for a level 0 that reads the bodies in place); with `bmin` set, also the bounding box
// of the whole set (segment 0 of level 0) on ordered keys.
__global__ __launch_bounds__(256) void k_init_work(Bodies b, double *wx, double *wy, double *wz,
                                                   uint32_t *wid, uint32_t n,
                                                   unsigned long long *bmin,
                                                   unsigned long long *bmax) {
    unsigned long long mn[3] = {~0ull, ~0ull, ~0ull}, mx[3] = {0ull, 0ull, 0ull};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x) {
        const double x = b.x[i], y = b.y[i], z = b.z[i];
        if (wx) {
            wx[i] = x;
            wy[i] = y;
            wz[i] = z;
            wid[i] = i;
        }
        const unsigned long long k0 = ord_key(x), k1 = ord_key(y), k2 = ord_key(z);
        mn[0] = min(mn[0], k0); mx[0] = max(mx[0], k0);
        mn[1] = min(mn[1], k1); mx[1] = max(mx[1], k1);
        mn[2] = min(mn[2], k2); mx[2] = max(mx[2], k2);
    }
    if (!bmin) return;
    __shared__ unsigned long long red[8][6];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        mn[d] = warp_min(mn[d]);
        mx[d] = warp_max(mx[d]);
    }
    if (lane == 0) {
        for (int d = 0; d < 3; ++d) { red[warp][d] = mn[d]; red[warp][3 + d] = mx[d]; }
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        const int d = threadIdx.x;
        unsigned long long a = ~0ull, c = 0ull;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            a = min(a, red[w][d]);
            c = max(c, red[w][3 + d]);
        }
        atomicMin(&bmin[d], a);
        atomicMax(&bmax[d], c);
    }
}

void launch_init_work(const Bodies &b, Work &w, uint32_t n, unsigned long long *bmin,
                      unsigned long long *bmax, cudaStream_t st, bool copy) {
    int blocks = (int)((n + 255) / 256);
    if (blocks > sm_count() * 16) blocks = sm_count() * 16;  // a few thousand box atomics
    if (bmin) {
        cudaMemsetAsync(bmin, 0xff, sizeof(unsigned long long) * 3, st);
        cudaMemsetAsync(bmax, 0x00, sizeof(unsigned long long) * 3, st);
    }
    if (copy)
        k_init_work<<<blocks, 256, 0, st>>>(b, w.x[0], w.y[0], w.z[0], w.id[0], n, bmin, bmax);
    else
        k_init_work<<<blocks, 256, 0, st>>>(b, nullptr, nullptr, nullptr, nullptr, n, bmin, bmax);
}

__global__ void k_gather_keys(const double *vals, uint64_t n_vals, const uint64_t *idx,
                              uint32_t n, double *key, uint32_t *id, uint32_t *err) {
    bool bad = false;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x) {
        const uint64_t j = idx[i];
        const bool ok = j < n_vals && j <= 0xffffffffull;
        key[i] = ok ? vals[j] : 0.0;
        id[i] = (uint32_t)j;
        bad |= !ok || !isfinite(ok ? vals[j] : 0.0);
    }
    if (bad) atomicOr(err, kErrNumeric);
}

void launch_gather_keys(const double *vals, uint64_t n_vals, const uint64_t *idx, uint32_t n,
                        double *key, uint32_t *id, uint32_t *err, cudaStream_t st) {
    int blocks = (int)((n + 255) / 256);
    if (blocks > sm_count() * 16) blocks = sm_count() * 16;
    k_gather_keys<<<blocks, 256, 0, st>>>(vals, n_vals, idx, n, key, id, err);
}

// The partition leaves the selected element somewhere in [goal, n); swap it to goal.
__global__ void k_place_selected(uint32_t *id, const uint32_t *med_pos, uint32_t goal) {
    const uint32_t p = *med_pos;
    const uint32_t t = id[goal];
    id[goal] = id[p];
    id[p] = t;
}

void launch_place_selected(uint32_t *id, const uint32_t *med_pos, uint32_t goal, cudaStream_t st) {
    k_place_selected<<<1, 1, 0, st>>>(id, med_pos, goal);
}

// ------------------------------------------------------------------ level passes

struct TileRef {
    uint32_t seg, tile, id, start, cnt, lo, hi;
};

__device__ __forceinline__ bool tile_at(const Topology &t, const LevelArgs &lv, uint32_t idx,
                                        TileRef &r) {
    r.seg = idx / lv.tiles;
    r.tile = idx - r.seg * lv.tiles;
    r.id = lv.ids[r.seg];
    r.start = t.start[r.id];
    r.cnt = t.count[r.id];
    r.lo = r.tile * (uint32_t)kTile;
    if (r.lo >= r.cnt) return false;
    r.hi = min(r.cnt, r.lo + (uint32_t)kTile);
    return true;
}

__device__ __forceinline__ bool tile_of(const Topology &t, const LevelArgs &lv, TileRef &r) {
    return tile_at(t, lv, blockIdx.x, r);
}

__device__ __forceinline__ double warp_fmin(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(kFull, v, o));
    return v;
}
__device__ __forceinline__ double warp_fmax(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(kFull, v, o));
    return v;
}

// Bounding box of every segment: block-local min/max, then 64-bit atomics on the ordered
// keys (min and max are exact, so the result does not depend on the order).
__global__ __launch_bounds__(kTileThreads) void k_bbox(Topology t, LevelArgs lv,
                                                       const double *wx, const double *wy,
                                                       const double *wz,
                                                       unsigned long long *bmin,
                                                       unsigned long long *bmax) {
    TileRef r;
    if (!tile_of(t, lv, r)) return;
    unsigned long long mn[3] = {~0ull, ~0ull, ~0ull}, mx[3] = {0ull, 0ull, 0ull};
    for (uint32_t k = r.lo + threadIdx.x; k < r.hi; k += blockDim.x) {
        const unsigned long long k0 = ord_key(wx[r.start + k]), k1 = ord_key(wy[r.start + k]),
                                 k2 = ord_key(wz[r.start + k]);
        mn[0] = min(mn[0], k0); mx[0] = max(mx[0], k0);
        mn[1] = min(mn[1], k1); mx[1] = max(mx[1], k1);
        mn[2] = min(mn[2], k2); mx[2] = max(mx[2], k2);
    }
    __shared__ unsigned long long red[kTileThreads / 32][6];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        mn[d] = warp_min(mn[d]);
        mx[d] = warp_max(mx[d]);
    }
    if (lane == 0) {
        for (int d = 0; d < 3; ++d) { red[warp][d] = mn[d]; red[warp][3 + d] = mx[d]; }
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        int d = threadIdx.x;
        unsigned long long a = ~0ull, b = 0ull;
        for (int w = 0; w < kTileThreads / 32; ++w) {
            a = min(a, red[w][d]);
            b = max(b, red[w][3 + d]);
        }
        atomicMin(&bmin[r.seg * 3 + d], a);
        atomicMax(&bmax[r.seg * 3 + d], b);
    }
}

// First-pass bin of a coordinate: linear in [lo, hi] along the split dimension.  The
// truncating conversion, the float difference to lo, the product by a positive scale and the
// truncation to an integer are each monotone in v, so bin(v1) < bin(v2) implies v1 < v2:
// the bins order the bodies consistently with (coordinate, id), and equal coordinates share
// a bin.
__device__ __forceinline__ uint32_t lin_bin(double v, float lo, float scale) {
    const float f = (trunc_float(v) - lo) * scale;
    return f >= (float)(kHistBins - 1) ? (uint32_t)(kHistBins - 1) : (uint32_t)f;
}

// Split choice of a segment from its bounding box (ordered keys), as SegSel plus the node's
// split_dim and size: the first-pass linear bins span [lo, hi] of the split coordinate.
__device__ __forceinline__ SegSel make_segsel(const unsigned long long *bmin,
                                              const unsigned long long *bmax, uint32_t seg,
                                              uint32_t cnt, uint32_t rank, double &size) {
    double mn[3], mx[3];
    for (int d = 0; d < 3; ++d) {
        mn[d] = ord_val(bmin[seg * 3 + d]);
        mx[d] = ord_val(bmax[seg * 3 + d]);
    }
    uint32_t sd;
    choose_split(mn, mx, sd, size);
    SegSel s;
    s.sd = sd;
    s.lo = trunc_float(sd == 0 ? mn[0] : (sd == 1 ? mn[1] : mn[2]));
    const float range = trunc_float(sd == 0 ? mx[0] : (sd == 1 ? mx[1] : mx[2])) - s.lo;
    const float scale = (float)kHistBins / range;
    s.scale = (range > 0.0f && isfinite(scale)) ? scale : 0.0f;
    s.digit = 0;
    s.c = cnt;
    s.r = rank;
    s.pad = 0;
    s.kmed = 0;
    s.idmed = 0;
    s.posmed = 0;
    s.pad2 = 0;
    return s;
}

// Split dimension, size and the first-pass binning of every segment (levels whose medians
// k_select finds over the whole segment).
__global__ void k_split(Topology t, LevelArgs lv, const unsigned long long *bmin,
                        const unsigned long long *bmax, SegSel *sel, NodeOut no) {
    uint32_t seg = blockIdx.x * blockDim.x + threadIdx.x;
    if (seg >= lv.G) return;
    uint32_t id = lv.ids[seg];
    uint32_t cnt = t.count[id];
    double size;
    const SegSel s = make_segsel(bmin, bmax, seg, cnt, split_rank(lv, cnt), size);
    no.split_dim[id] = (uint8_t)s.sd;
    no.size[id] = size;
    sel[seg] = s;
}

// Block-wide search of the histogram bin holding rank r.  Every thread owns
// kHistBins/blockDim consecutive bins.  Returns digit / count below / count in bin through
// shared memory.
__device__ void find_bin(const uint32_t *h, uint32_t r, uint32_t *out3,
                         uint32_t nb = kHistBins) {
    const int per = nb >= blockDim.x ? (int)(nb / blockDim.x) : 1;
    __shared__ uint32_t wsum[32];
    uint32_t mine = 0;
    for (int i = 0; i < per; ++i)
        if (threadIdx.x * per + i < nb) mine += h[threadIdx.x * per + i];
    // block exclusive scan of `mine`
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t inc = mine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t v = __shfl_up_sync(kFull, inc, o);
        if (lane >= o) inc += v;
    }
    if (lane == 31) wsum[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint32_t v = lane < nw ? wsum[lane] : 0u;
        uint32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t u = __shfl_up_sync(kFull, x, o);
            if (lane >= o) x += u;
        }
        if (lane < nw) wsum[lane] = x - v;
    }
    __syncthreads();
    uint32_t before = wsum[warp] + inc - mine;
    if (r >= before && r < before + mine) {
        uint32_t cum = before;
        for (int i = 0; i < per; ++i) {
            if (threadIdx.x * per + i >= nb) break;
            uint32_t c = h[threadIdx.x * per + i];
            if (r < cum + c) {
                out3[0] = (uint32_t)(threadIdx.x * per + i);
                out3[1] = cum;
                out3[2] = c;
                break;
            }
            cum += c;
        }
    }
    __syncthreads();
}

// First pass over big segments: the split choice (every block of a segment makes the same
// one from the segment's bounding box), a histogram of linear bins of the split coordinate,
// and -- in the segment's last block to finish -- the bin holding the wanted rank.  A block
// takes kHistTiles consecutive tiles of one segment, so that zeroing its kHistBins shared
// bins and merging them into the segment's histogram is paid once per kHistTiles * kTile
// bodies.  `done` counts the finished blocks of every segment (the last one resets it).
#ifndef KD_HIST_TILES
#define KD_HIST_TILES 8
#endif
constexpr uint32_t kHistTiles = KD_HIST_TILES;

__global__ __launch_bounds__(kTileThreads) void k_hist(Topology t, LevelArgs lv,
                                                       const double *wx, const double *wy,
                                                       const double *wz,
                                                       const unsigned long long *bmin,
                                                       const unsigned long long *bmax,
                                                       SegSel *sel, NodeOut no, uint32_t *hist,
                                                       uint32_t *done) {
    const uint32_t per_seg = (lv.tiles + kHistTiles - 1) / kHistTiles;
    const uint32_t seg = blockIdx.x / per_seg;
    const uint32_t t0 = (blockIdx.x - seg * per_seg) * kHistTiles;
    const uint32_t id = lv.ids[seg];
    const uint32_t cnt = t.count[id];
    double size;
    const SegSel s = make_segsel(bmin, bmax, seg, cnt, split_rank(lv, cnt), size);
    __shared__ uint32_t h[kHistBins];
    __shared__ uint32_t out3[3];
    __shared__ bool last;
    TileRef r;
    const bool has = tile_at(t, lv, seg * lv.tiles + t0, r);  // block-uniform
    uint32_t *gh = hist + (size_t)seg * kHistBins;
    // a block that holds the whole segment has its final bins in shared memory already
    const bool alone = per_seg == 1u;
    if (has) {
        const uint32_t hi = min(r.cnt, r.lo + kHistTiles * (uint32_t)kTile);
        for (int b = threadIdx.x; b < kHistBins; b += blockDim.x) h[b] = 0;
        __syncthreads();
        const double *w = pick(wx, wy, wz, s.sd) + r.start;
        constexpr int kRows = kTile / kTileThreads;
        // the next tile's keys are requested before this tile's are binned, so that the
        // loads of one overlap the shared-memory atomics of the other
        double v[kRows];
#pragma unroll
        for (int i = 0; i < kRows; ++i) {
            const uint32_t k = r.lo + (uint32_t)i * kTileThreads + threadIdx.x;
            v[i] = k < hi ? w[k] : 0.0;
        }
        for (uint32_t base = r.lo; base < hi; base += kTile) {
            double nv[kRows];
#pragma unroll
            for (int i = 0; i < kRows; ++i) {
                const uint32_t k = base + kTile + (uint32_t)i * kTileThreads + threadIdx.x;
                nv[i] = k < hi ? w[k] : 0.0;
            }
#pragma unroll
            for (int i = 0; i < kRows; ++i)
                if (base + (uint32_t)i * kTileThreads + threadIdx.x < hi)
                    atomicAdd(&h[lin_bin(v[i], s.lo, s.scale)], 1u);
#pragma unroll
            for (int i = 0; i < kRows; ++i) v[i] = nv[i];
        }
        __syncthreads();
        if (!alone)
            for (int b = threadIdx.x; b < kHistBins; b += blockDim.x)
                if (h[b]) atomicAdd(&gh[b], h[b]);
    }
    if (!alone) {
        // the segment's last block sees every block's bins
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) last = atomicAdd(&done[seg], 1u) == per_seg - 1;
        __syncthreads();
        if (!last) return;
        __threadfence();
        for (int b = threadIdx.x; b < kHistBins; b += blockDim.x) h[b] = __ldcg(&gh[b]);
        __syncthreads();
    }
    find_bin(h, s.r, out3);
    if (threadIdx.x == 0) {
        SegSel o = s;
        o.digit = out3[0];
        o.r = s.r - out3[1];
        o.c = out3[2];
        sel[seg] = o;
        no.split_dim[id] = (uint8_t)s.sd;
        no.size[id] = size;
        if (!alone) done[seg] = 0u;
    }
}

// Gather the keys of the selected first-pass bin as candidates (unordered; the exact
// select below does not depend on their order), and count per tile the bodies of lower bins:
// they go left whatever the median inside the bin (bins order the bodies as their keys do),
// so tile_cnt starts as that count and k_select adds the candidates that go left.
__global__ __launch_bounds__(kTileThreads) void k_collect(Topology t, LevelArgs lv,
                                                          const double *wx, const double *wy,
                                                          const double *wz, const SegSel *sel,
                                                          uint32_t *cand_cnt,
                                                          unsigned long long *ckey,
                                                          uint32_t *cpos, uint32_t *tile_cnt) {
    TileRef r;
    if (!tile_of(t, lv, r)) return;
    const SegSel s = sel[r.seg];
    const double *w = pick(wx, wy, wz, s.sd) + r.start;
    const int lane = threadIdx.x & 31;
    uint32_t below = 0;
    constexpr int kRows = kTile / kTileThreads;
    double vr[kRows];
#pragma unroll
    for (int i = 0; i < kRows; ++i) {
        const uint32_t k = r.lo + (uint32_t)i * kTileThreads + threadIdx.x;
        vr[i] = k < r.hi ? w[k] : 0.0;
    }
#pragma unroll
    for (int i = 0; i < kRows; ++i) {
        const uint32_t k = r.lo + (uint32_t)i * kTileThreads + threadIdx.x;
        bool in = k < r.hi;
        const double v = vr[i];
        const unsigned long long key = ord_key(v);
        const uint32_t bin = lin_bin(v, s.lo, s.scale);
        below += (in && bin < s.digit) ? 1u : 0u;
        bool hit = in && bin == s.digit;
        uint32_t m = __ballot_sync(kFull, hit);
        if (m) {
            uint32_t leader = __ffs(m) - 1, slot = 0;
            if (lane == (int)leader) slot = atomicAdd(&cand_cnt[r.seg], (uint32_t)__popc(m));
            slot = __shfl_sync(kFull, slot, leader);
            if (hit) {
                uint32_t o = slot + __popc(m & ((1u << lane) - 1u));
                ckey[r.start + o] = key;
                cpos[r.start + o] = k;
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) below += __shfl_xor_sync(kFull, below, o);
    __shared__ uint32_t ws[kTileThreads / 32];
    if (lane == 0) ws[threadIdx.x >> 5] = below;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t tot = 0;
        for (int i = 0; i < kTileThreads / 32; ++i) tot += ws[i];
        tile_cnt[(size_t)r.seg * lv.tiles + r.tile] = tot;
    }
}

__device__ __forceinline__ bool goes_left(unsigned long long key, uint32_t id,
                                          unsigned long long kmed, uint32_t idmed) {
    return key < kmed || (key == kmed && id < idmed);
}

// Body ids of a segment: the work array's, or -- at a level 0 that reads the bodies in place,
// in their original order -- the position itself.
struct IdView {
    const uint32_t *p;
    uint32_t base;
    __device__ __forceinline__ uint32_t operator[](uint32_t i) const { return p ? p[i] : base + i; }
};

// The last step of k_select when more than 32 candidates are left (a refinement that could
// not narrow them): a bitonic sort of (key, id) and a pick at the wanted rank.
template <typename Get>
__device__ __forceinline__ void select_sorted(unsigned long long *skey, unsigned long long *sval,
                                              uint32_t c, uint32_t r, SegSel *sel, uint32_t seg,
                                              NodeOut no, uint32_t nid, const double *w,
                                              const IdView &ids, Get &get,
                                              unsigned long long &s_kmed, uint32_t &s_idmed) {
    const uint32_t P = next_pow2(c);
    for (uint32_t j = threadIdx.x; j < P; j += blockDim.x) {
        if (j < c) {
            unsigned long long key;
            uint32_t pos;
            get(j, key, pos);
            skey[j] = key;
            sval[j] = ((unsigned long long)ids[pos] << 32) | pos;
        } else {
            skey[j] = ~0ull;
            sval[j] = ~0ull;
        }
    }
    __syncthreads();
    if (P > 1) bitonic_blocks(skey, sval, P, P);
    if (threadIdx.x == 0) {
        unsigned long long v = sval[r];
        uint32_t pos = (uint32_t)(v & 0xffffffffull);
        sel[seg].kmed = skey[r];
        sel[seg].idmed = (uint32_t)(v >> 32);
        sel[seg].posmed = pos;
        no.split_val[nid] = w[pos];
        s_kmed = skey[r];
        s_idmed = (uint32_t)(v >> 32);
    }
}

// Tile offsets of the partition (see k_select), one block per segment.
constexpr int kSmallSegTiles = 8;  // non-multi segments: at most kMultiMin / kTile tiles
static_assert(kMultiMin <= (uint32_t)(kSmallSegTiles * kTile), "tile counters of a small segment");

__device__ __forceinline__ void tile_offsets(const Topology &t, const LevelArgs &lv,
                                             const Scratch &s, const SegSel &st, uint32_t seg,
                                             uint32_t nid, uint32_t start, const double *w,
                                             const IdView &ids, unsigned long long kmed,
                                             uint32_t idmed) {
    __shared__ uint32_t scnt[kSmallSegTiles];
    __shared__ uint32_t wsum[32];
    __shared__ uint32_t carry;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t cnt = t.count[nid];
    const uint32_t ntiles = (cnt + kTile - 1) / kTile;
    uint32_t *tc = s.tile_cnt + (size_t)seg * lv.tiles;
    uint32_t *to = s.tile_off + (size_t)seg * lv.tiles;
    if (lv.multi) {
        // the candidates of the first-pass bin that go left, added to the lower-bin counts
        for (uint32_t j = threadIdx.x; j < st.c; j += blockDim.x) {
            const uint32_t pos = s.cpos[0][start + j];
            if (goes_left(s.ckey[0][start + j], ids[pos], kmed, idmed))
                atomicAdd(&tc[pos / kTile], 1u);
        }
    } else {
        if (threadIdx.x < kSmallSegTiles) scnt[threadIdx.x] = 0u;
        __syncthreads();
        // one ballot per warp row (a row of 32 never straddles a tile) and one atomic
        for (uint32_t base = 0; base < cnt; base += blockDim.x) {
            const uint32_t j = base + threadIdx.x;
            const bool L = j < cnt && goes_left(ord_key(w[j]), ids[j], kmed, idmed);
            const uint32_t m = __ballot_sync(kFull, L);
            const uint32_t tile = (base + 32u * warp) / kTile;
            if (lane == 0 && m && tile < (uint32_t)kSmallSegTiles)
                atomicAdd(&scnt[tile], (uint32_t)__popc(m));
        }
        __syncthreads();
        if (threadIdx.x < ntiles && threadIdx.x < kSmallSegTiles) tc[threadIdx.x] = scnt[threadIdx.x];
        if (threadIdx.x == 0 && ntiles > kSmallSegTiles) atomicOr(s.err, kErrSelect);
    }
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint32_t base = 0; base < ntiles; base += blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t v = i < ntiles ? __ldcg(&tc[i]) : 0u;
        uint32_t inc = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(kFull, inc, o);
            if (lane >= o) inc += u;
        }
        if (lane == 31) wsum[warp] = inc;
        __syncthreads();
        uint32_t wpre = 0;
        for (int q = 0; q < warp; ++q) wpre += wsum[q];
        if (i < ntiles) to[i] = carry + wpre + inc - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry += wpre + inc;
        __syncthreads();
    }
    if (threadIdx.x == 0 && carry != split_rank(lv, cnt)) atomicOr(s.err, kErrSelect);
}

// Exact median of every segment: radix refinement until at most kSelCap candidates are
// left, then a bitonic sort of (key, id) in shared memory and a pick at the wanted rank.
// Candidates start as the collected first-pass bin (multi: buffer 0, which the refinement
// passes, alternating between buffers 1 and 2, leave intact) or the whole segment.  Then the
// partition's tile offsets: the bodies going left per tile (multi: k_collect's lower-bin
// counts plus the candidates that go left; else counted here over the segment), scanned
// over the segment's tiles; a total other than the wanted rank is a failed select.
__global__ __launch_bounds__(kSelThreads) void k_select(Topology t, LevelArgs lv,
                                                        const double *wx, const double *wy,
                                                        const double *wz, const uint32_t *wid,
                                                        SegSel *sel, Scratch s, NodeOut no) {
    // the refinement histogram and the final sort never live at the same time
    __shared__ unsigned long long sbuf[2 * kSelCap];
    unsigned long long *skey = sbuf, *sval = sbuf + kSelCap;
    uint32_t *h = reinterpret_cast<uint32_t *>(sbuf);
    static_assert(kHistBins * sizeof(uint32_t) <= 2 * kSelCap * sizeof(unsigned long long),
                  "histogram must fit in the sort buffer");
    __shared__ uint32_t out3[3];
    __shared__ uint32_t ncomp;
    __shared__ unsigned long long red_k[2][kSelThreads / 32];
    __shared__ uint32_t red_i[2][kSelThreads / 32];
    __shared__ unsigned long long s_kmed;
    __shared__ uint32_t s_idmed;

    const uint32_t seg = blockIdx.x;
    const uint32_t nid = lv.ids[seg];
    const uint32_t start = t.start[nid];
    SegSel st = sel[seg];
    const double *w = pick(wx, wy, wz, st.sd) + start;
    const IdView ids{wid ? wid + start : nullptr, start};
    uint32_t c = st.c, r = st.r;
    int src = lv.multi ? 0 : -1;  // -1: the candidates are the segment itself
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (threadIdx.x == 0) {  // a failed select keeps the split's defaults
        s_kmed = st.kmed;
        s_idmed = st.idmed;
    }

    auto get = [&](uint32_t j, unsigned long long &key, uint32_t &pos) {
        if (src < 0) {
            pos = j;
            key = ord_key(w[j]);
        } else {
            pos = (src == 0 ? s.cpos[0] : (src == 1 ? s.cpos[1] : s.cpos[2]))[start + j];
            key = (src == 0 ? s.ckey[0] : (src == 1 ? s.ckey[1] : s.ckey[2]))[start + j];
        }
    };

    // refine until at most 32 candidates are left (ranked in one warp below); a pass that
    // cannot narrow any further (the error path) leaves up to kSelCap for the block sort
    for (int iter = 0; c > 32u; ++iter) {
        if (iter >= lv.max_iters) {
            if (threadIdx.x == 0) atomicOr(s.err, kErrSelect);
            c = min(c, (uint32_t)kSelCap);
            if (r >= c) r = c - 1;
            break;
        }
        // the first pass over a whole segment uses the linear bins of its bounding box;
        // later passes use the key bits below the candidates' common prefix (then the id)
        const bool lin = src < 0 && iter == 0 && st.scale > 0.0f;
        // key and id range of the candidates
        unsigned long long kmn = ~0ull, kmx = 0ull;
        uint32_t imn = kFull, imx = 0u;
        for (uint32_t j = threadIdx.x; j < (lin ? 0u : c); j += blockDim.x) {
            unsigned long long key;
            uint32_t pos;
            get(j, key, pos);
            uint32_t id = ids[pos];
            kmn = min(kmn, key); kmx = max(kmx, key);
            imn = min(imn, id); imx = max(imx, id);
        }
        kmn = warp_min(kmn); kmx = warp_max(kmx);
        imn = warp_min(imn); imx = warp_max(imx);
        if (lane == 0) {
            red_k[0][warp] = kmn; red_k[1][warp] = kmx;
            red_i[0][warp] = imn; red_i[1][warp] = imx;
        }
        kmn = ~0ull; kmx = 0; imn = kFull; imx = 0;
        __syncthreads();
        for (int i = 0; i < nw; ++i) {
            kmn = min(kmn, red_k[0][i]); kmx = max(kmx, red_k[1][i]);
            imn = min(imn, red_i[0][i]); imx = max(imx, red_i[1][i]);
        }
        // bins for about 32 candidates each (at least 256, at most kHistBins): the zeroing
        // and the scan of the histogram then cost in proportion to the candidates
        int nbits = 8;
        while (nbits < kHistBits && (c >> (nbits + 5)) > 0u) ++nbits;
        const uint32_t nb = 1u << nbits;
        const bool bykey = kmn != kmx;
        int bits = bykey ? 64 - __clzll((long long)(kmn ^ kmx)) : 32 - __clz((int)(imn ^ imx));
        const uint32_t shift = bits > nbits ? (uint32_t)(bits - nbits) : 0u;
        // the candidate's bin; its id is loaded only when the pass bins by id
        auto digit = [&](unsigned long long key, uint32_t pos) -> uint32_t {
            if (lin) return lin_bin(ord_val(key), st.lo, st.scale) >> (kHistBits - nbits);
            return bykey ? ((uint32_t)(key >> shift) & (nb - 1)) : ((ids[pos] >> shift) & (nb - 1));
        };
        for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x) h[b] = 0;
        if (threadIdx.x == 0) ncomp = 0;
        __syncthreads();
        for (uint32_t j = threadIdx.x; j < c; j += blockDim.x) {
            unsigned long long key;
            uint32_t pos;
            get(j, key, pos);
            atomicAdd(&h[digit(key, pos)], 1u);
        }
        __syncthreads();
        find_bin(h, r, out3, nb);
        const uint32_t dig = out3[0], below = out3[1], inbin = out3[2];
        const int dst = src == 1 ? 2 : 1;
        for (uint32_t base = 0; base < c; base += blockDim.x) {
            const uint32_t j = base + threadIdx.x;
            const bool in = j < c;
            unsigned long long key = 0;
            uint32_t pos = 0;
            if (in) get(j, key, pos);
            const bool hit = in && digit(key, pos) == dig;
            const uint32_t m = __ballot_sync(kFull, hit);
            if (m) {
                uint32_t leader = __ffs(m) - 1, slot = 0;
                if (lane == (int)leader) slot = atomicAdd(&ncomp, (uint32_t)__popc(m));
                slot = __shfl_sync(kFull, slot, leader);
                if (hit) {
                    uint32_t o = slot + __popc(m & ((1u << lane) - 1u));
                    (dst == 1 ? s.ckey[1] : s.ckey[2])[start + o] = key;
                    (dst == 1 ? s.cpos[1] : s.cpos[2])[start + o] = pos;
                }
            }
        }
        __syncthreads();
        c = inbin;
        r -= below;
        src = dst;
        __syncthreads();
    }

    if (c <= 32u) {
        // rank of each candidate among the others by (key, id): the one of rank r is the median
        if (warp == 0) {
            unsigned long long key = ~0ull;
            uint32_t pos = 0, id = kFull;
            if ((uint32_t)lane < c) {
                get((uint32_t)lane, key, pos);
                id = ids[pos];
            }
            uint32_t rank = 0;
            for (uint32_t j = 0; j < c; ++j) {
                const unsigned long long kj = __shfl_sync(kFull, key, j);
                const uint32_t ij = __shfl_sync(kFull, id, j);
                rank += (kj < key || (kj == key && ij < id)) ? 1u : 0u;
            }
            if ((uint32_t)lane < c && rank == r) {
                sel[seg].kmed = key;
                sel[seg].idmed = id;
                sel[seg].posmed = pos;
                no.split_val[nid] = w[pos];
                s_kmed = key;
                s_idmed = id;
            }
        }
    } else {
        select_sorted(skey, sval, c, r, sel, seg, no, nid, w, ids, get, s_kmed, s_idmed);
    }
    __syncthreads();
    if (lv.tiles > 1) tile_offsets(t, lv, s, st, seg, nid, start, w, ids, s_kmed, s_idmed);
}

// Asynchronous global -> shared copies (cp.async) of the partition's tile.  The wait is the
// hardware's group count, not a spin loop.
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(a), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(a), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// The partition's tile in shared memory: positions and ids as read, and the tile's bodies in
// output order (left child first, then right) as indices into them.
struct ScatTile {
    double x[kTile], y[kTile], z[kTile];
    uint32_t id[kTile];
    uint16_t order[kTile];
};

// Stable partition: bodies keep their relative order inside each child.  With `nbmin`
// set, the bounding boxes of the two children (segments 2*seg and 2*seg+1 of the next
// level) are reduced on the way.  A block stages its tile in shared memory, ranks every body
// inside its child (one ballot per row of the tile, a table of per-(row, warp) counts and its
// scan), and then writes the tile out in output order: consecutive threads write consecutive
// destinations, one contiguous run per child.
__global__ __launch_bounds__(kTileThreads, 3) void k_part_scatter(
    Topology t, LevelArgs lv, const double *sx, const double *sy, const double *sz,
    const uint32_t *sid, double *dx, double *dy, double *dz, uint32_t *did, const SegSel *sel,
    const uint32_t *tile_off, unsigned long long *nbmin, unsigned long long *nbmax,
    uint32_t *err) {
    extern __shared__ __align__(16) unsigned char scat_raw[];
    ScatTile &S = *reinterpret_cast<ScatTile *>(scat_raw);
    TileRef r;
    if (!tile_at(t, lv, blockIdx.x, r)) return;  // block-uniform
    constexpr int kRows = kTile / kTileThreads;
    constexpr int kWarps = kTileThreads / 32;
    __shared__ uint32_t cntL[kRows][kWarps], cntR[kRows][kWarps];
    __shared__ uint32_t s_nl;
    __shared__ unsigned long long red[kWarps][12];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t lt = (1u << lane) - 1u;
    const uint32_t n = r.hi - r.lo;  // bodies of this tile
#pragma unroll
    for (int i = 0; i < kRows; ++i) {
        const uint32_t q = (uint32_t)i * kTileThreads + threadIdx.x;
        if (q < n) {
            const uint32_t k = r.start + r.lo + q;
            cp_async8(&S.x[q], sx + k);
            cp_async8(&S.y[q], sy + k);
            cp_async8(&S.z[q], sz + k);
            if (sid)
                cp_async4(&S.id[q], sid + k);
            else
                S.id[q] = k;  // a level 0 read in place: the position is the body id
        }
    }
    const SegSel s = sel[r.seg];
    const uint32_t mid = split_rank(lv, r.cnt);
    // without tile offsets every segment is one tile: nothing goes left before it
    const uint32_t lbase = tile_off ? tile_off[(size_t)r.seg * lv.tiles + r.tile] : 0u;
    const uint32_t rbase = r.lo - lbase;
    cp_async_wait_all();
    __syncthreads();

    // [child][dim] running bounds of this thread, as ordered keys
    unsigned long long cmn[2][3] = {{~0ull, ~0ull, ~0ull}, {~0ull, ~0ull, ~0ull}};
    unsigned long long cmx[2][3] = {{0ull, 0ull, 0ull}, {0ull, 0ull, 0ull}};
    uint32_t bl[kRows], br[kRows];
#pragma unroll
    for (int i = 0; i < kRows; ++i) {
        const uint32_t q = (uint32_t)i * kTileThreads + threadIdx.x;
        const bool in = q < n;
        bool isL = false;
        if (in) {
            const unsigned long long kx = ord_key(S.x[q]), ky = ord_key(S.y[q]),
                                     kz = ord_key(S.z[q]);
            const unsigned long long key = s.sd == 0 ? kx : (s.sd == 1 ? ky : kz);
            isL = goes_left(key, S.id[q], s.kmed, s.idmed);
            if (nbmin) {
                if (isL) {
                    cmn[0][0] = min(cmn[0][0], kx); cmx[0][0] = max(cmx[0][0], kx);
                    cmn[0][1] = min(cmn[0][1], ky); cmx[0][1] = max(cmx[0][1], ky);
                    cmn[0][2] = min(cmn[0][2], kz); cmx[0][2] = max(cmx[0][2], kz);
                } else {
                    cmn[1][0] = min(cmn[1][0], kx); cmx[1][0] = max(cmx[1][0], kx);
                    cmn[1][1] = min(cmn[1][1], ky); cmx[1][1] = max(cmx[1][1], ky);
                    cmn[1][2] = min(cmn[1][2], kz); cmx[1][2] = max(cmx[1][2], kz);
                }
            }
        }
        bl[i] = __ballot_sync(kFull, in && isL);
        br[i] = __ballot_sync(kFull, in && !isL);
    }
    if (lane == 0) {
#pragma unroll
        for (int i = 0; i < kRows; ++i) {
            cntL[i][warp] = __popc(bl[i]);
            cntR[i][warp] = __popc(br[i]);
        }
    }
    __syncthreads();
    if (warp == 0) {
        // exclusive scan over the kRows x kWarps counts in row-major (element) order
        constexpr int kCells = kRows * kWarps;
        static_assert(kCells <= 64, "two cells per lane");
        uint32_t a0 = 0, a1 = 0, b0 = 0, b1 = 0;
        const int c0 = 2 * lane, c1 = 2 * lane + 1;
        if (c0 < kCells) { a0 = cntL[c0 / kWarps][c0 % kWarps]; b0 = cntR[c0 / kWarps][c0 % kWarps]; }
        if (c1 < kCells) { a1 = cntL[c1 / kWarps][c1 % kWarps]; b1 = cntR[c1 / kWarps][c1 % kWarps]; }
        uint32_t sa = a0 + a1, sb = b0 + b1;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t ua = __shfl_up_sync(kFull, sa, o), ub = __shfl_up_sync(kFull, sb, o);
            if (lane >= o) { sa += ua; sb += ub; }
        }
        const uint32_t ea = sa - a0 - a1, eb = sb - b0 - b1;
        // a one-tile segment checks here what the select kernels check otherwise: exactly
        // the wanted rank went left
        if (lane == 31) {
            s_nl = sa;
            if (!tile_off && sa != mid) atomicOr(err, kErrSelect);
        }
        __syncwarp();
        if (c0 < kCells) { cntL[c0 / kWarps][c0 % kWarps] = ea; cntR[c0 / kWarps][c0 % kWarps] = eb; }
        if (c1 < kCells) { cntL[c1 / kWarps][c1 % kWarps] = ea + a0; cntR[c1 / kWarps][c1 % kWarps] = eb + b0; }
    }
    __syncthreads();
    const uint32_t nl = s_nl;
#pragma unroll
    for (int i = 0; i < kRows; ++i) {
        const uint32_t q = (uint32_t)i * kTileThreads + threadIdx.x;
        if ((bl[i] | br[i]) >> lane & 1u) {
            const bool isL = bl[i] >> lane & 1u;
            const uint32_t slot = isL ? cntL[i][warp] + __popc(bl[i] & lt)
                                      : nl + cntR[i][warp] + __popc(br[i] & lt);
            S.order[slot] = (uint16_t)q;
        }
    }
    __syncthreads();
    // write-out in output order: slots [0, nl) are the tile's left bodies, the rest its right
    const uint32_t lstart = r.start + lbase, rstart = r.start + mid + rbase - nl;
    const uint32_t end = r.start + r.cnt;
    for (uint32_t j = threadIdx.x; j < n; j += kTileThreads) {
        const uint32_t q = S.order[j];
        const uint32_t dst = (j < nl ? lstart : rstart) + j;
        // a failed select (flagged by the select kernels) must not write outside the segment
        if (dst < end) {
            const double vx = S.x[q], vy = S.y[q], vz = S.z[q];
            const uint32_t vid = S.id[q];
            dx[dst] = vx;
            dy[dst] = vy;
            dz[dst] = vz;
            did[dst] = vid;
            if (lv.med_pos && vid == s.idmed) {
                const unsigned long long key = ord_key(s.sd == 0 ? vx : (s.sd == 1 ? vy : vz));
                if (key == s.kmed) *lv.med_pos = dst;
            }
        }
    }
    if (nbmin) {
#pragma unroll
        for (int c = 0; c < 2; ++c)
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                cmn[c][d] = warp_min(cmn[c][d]);
                cmx[c][d] = warp_max(cmx[c][d]);
            }
        if (lane == 0) {
            for (int c = 0; c < 2; ++c)
                for (int d = 0; d < 3; ++d) {
                    red[warp][6 * c + d] = cmn[c][d];
                    red[warp][6 * c + 3 + d] = cmx[c][d];
                }
        }
        __syncthreads();
        if (threadIdx.x < 12) {
            const int c = threadIdx.x / 6, q = threadIdx.x % 6, d = q % 3;
            const bool is_max = q >= 3;
            unsigned long long v = is_max ? 0ull : ~0ull;
            for (int wq = 0; wq < kWarps; ++wq)
                v = is_max ? max(v, red[wq][threadIdx.x]) : min(v, red[wq][threadIdx.x]);
            const size_t child = 2 * (size_t)r.seg + c;
            if (is_max)
                atomicMax(&nbmax[child * 3 + d], v);
            else
                atomicMin(&nbmin[child * 3 + d], v);
        }
    }
}

// Levels whose segments hold at most kWarpSelMax bodies choose their splits and medians in
// k_split_select_warp (one warp per segment; defined with the subtree finish below).
constexpr uint32_t kWarpSelMax = 4096;
constexpr int kWarpSelWarps = 8;
__global__ __launch_bounds__(kWarpSelWarps * 32) void k_split_select_warp(
    Topology t, LevelArgs lv, const unsigned long long *bmin, const unsigned long long *bmax,
    const double *wx, const double *wy, const double *wz, const uint32_t *wid, SegSel *sel,
    NodeOut no, uint32_t *tile_off, uint32_t *err);

int launch_level(const Topology &t, const LevelArgs &lv, const NodeOut &no, Work &w, int cur,
                 Scratch &s, int lvl, uint32_t G_next, cudaStream_t st, bool box0_ready,
                 uint32_t seg_max) {
    const int nxt = cur ^ 1;
    const uint32_t G = lv.G;
    const uint32_t grid = G * lv.tiles;
    unsigned long long *bmin = s.bmin[lvl & 1], *bmax = s.bmax[lvl & 1];
    unsigned long long *nbmin = G_next ? s.bmin[(lvl + 1) & 1] : nullptr;
    unsigned long long *nbmax = G_next ? s.bmax[(lvl + 1) & 1] : nullptr;
    int launched = 0;
    if (lvl == 0 && !box0_ready) {
        cudaMemsetAsync(bmin, 0xff, sizeof(unsigned long long) * 3 * G, st);
        cudaMemsetAsync(bmax, 0x00, sizeof(unsigned long long) * 3 * G, st);
        k_bbox<<<grid, kTileThreads, 0, st>>>(t, lv, w.x[cur], w.y[cur], w.z[cur], bmin, bmax);
        ++launched;
    }
    if (G_next) {
        cudaMemsetAsync(nbmin, 0xff, sizeof(unsigned long long) * 3 * G_next, st);
        cudaMemsetAsync(nbmax, 0x00, sizeof(unsigned long long) * 3 * G_next, st);
    }
    // tile offsets of the partition: written by the select kernels when a segment spans
    // several tiles; a one-tile segment's scatter counts and checks by itself
    uint32_t *tile_off = lv.tiles > 1 ? s.tile_off : nullptr;
    if (lv.multi) {
        // split + histogram (+ bin search), candidates (+ lower-bin counts), exact median
        // (+ tile offsets)
        // one histogram block per segment keeps its bins in shared memory: no global bins
        if (lv.tiles > kHistTiles)
            cudaMemsetAsync(s.hist, 0, sizeof(uint32_t) * kHistBins * (size_t)G, st);
        cudaMemsetAsync(s.cand_cnt, 0, sizeof(uint32_t) * G, st);
        k_hist<<<G * ((lv.tiles + kHistTiles - 1) / kHistTiles), kTileThreads, 0, st>>>(
            t, lv, w.x[cur], w.y[cur], w.z[cur], bmin, bmax, s.sel, no, s.hist, s.done);
        k_collect<<<grid, kTileThreads, 0, st>>>(t, lv, w.x[cur], w.y[cur], w.z[cur], s.sel,
                                                 s.cand_cnt, s.ckey[0], s.cpos[0], s.tile_cnt);
        k_select<<<G, kSelThreads, 0, st>>>(t, lv, w.x[cur], w.y[cur], w.z[cur], w.id[cur],
                                            s.sel, s, no);
        launched += 3;
    } else if (seg_max > kWarpSelMax) {
        k_split<<<(G + 127) / 128, 128, 0, st>>>(t, lv, bmin, bmax, s.sel, no);
        k_select<<<G, kSelThreads, 0, st>>>(t, lv, w.x[cur], w.y[cur], w.z[cur], w.id[cur],
                                            s.sel, s, no);
        launched += 2;
    } else {
        k_split_select_warp<<<(G + kWarpSelWarps - 1) / kWarpSelWarps, kWarpSelWarps * 32, 0,
                              st>>>(t, lv, bmin, bmax, w.x[cur], w.y[cur], w.z[cur], w.id[cur],
                                    s.sel, no, tile_off, s.err);
        launched += 1;
    }
    // set on every launch: the attribute belongs to the current device's context
    cudaFuncSetAttribute(k_part_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sizeof(ScatTile));
    k_part_scatter<<<grid, kTileThreads, sizeof(ScatTile), st>>>(
        t, lv, w.x[cur], w.y[cur], w.z[cur], w.id[cur], w.x[nxt], w.y[nxt], w.z[nxt], w.id[nxt],
        s.sel, tile_off, nbmin, nbmax, s.err);
    return launched + 1;
}

// ------------------------------------------------------------------ local subtree finish

constexpr int kLocalWarps = kLocalThreads / 32;
constexpr int kLocalLevels = 16;
constexpr int kLocalSizeSlots = 256;
// Candidate filter of the radix select: the top `kb` bits of the key and the top `ib` bits of
// the id are fixed to kp / ip.
struct RadixState {
    int kb, ib;
    unsigned long long kp;
    uint32_t ip;
    __device__ __forceinline__ bool match(unsigned long long key, uint32_t id) const {
        const bool km = kb == 0 || (key >> (64 - kb)) == kp;
        const bool im = ib == 0 || (id >> (32 - ib)) == ip;
        return km && im;
    }
    // digit of width w just below the fixed bits (key first, then id)
    __device__ __forceinline__ uint32_t digit(unsigned long long key, uint32_t id, int w) const {
        if (kb < 64) return (uint32_t)(key >> (64 - kb - w)) & ((1u << w) - 1u);
        return (id >> (32 - ib - w)) & ((1u << w) - 1u);
    }
    __device__ __forceinline__ int width() const {
        return kb < 64 ? min(8, 64 - kb) : min(8, 32 - ib);
    }
    // (key, id) orders below every candidate: its fixed bits compare lower
    __device__ __forceinline__ bool below(unsigned long long key, uint32_t id) const {
        if (kb > 0) {
            const unsigned long long t = kb == 64 ? key : (key >> (64 - kb));
            if (t != kp) return t < kp;
            if (kb < 64) return false;
        }
        return ib > 0 && (id >> (32 - ib)) < ip;
    }
    __device__ __forceinline__ void fix(uint32_t d, int w) {
        if (kb < 64) {
            kp = (kp << w) | d;
            kb += w;
        } else {
            ip = (ip << w) | d;
            ib += w;
        }
    }
};

// Split choice and exact median of a level's segments when they are small (at most
// kWarpSelMax bodies): one warp per segment, no block barrier.  Lane 0 chooses the split as
// k_split does; the warp then narrows the (key, id) candidates with 8-bit radix passes over a
// warp-private histogram, as the subtree finish does for its larger nodes, until at most 32
// remain, and ranks those by comparison.  Writes the segment's SegSel and node fields, and
// with tile_off set (segments of two tiles) the partition's tile offsets, checking that
// exactly the wanted rank goes left.
__global__ __launch_bounds__(kWarpSelWarps * 32) void k_split_select_warp(
    Topology t, LevelArgs lv, const unsigned long long *bmin, const unsigned long long *bmax,
    const double *wx, const double *wy, const double *wz, const uint32_t *wid, SegSel *sel,
    NodeOut no, uint32_t *tile_off, uint32_t *err) {
    __shared__ uint32_t hist[kWarpSelWarps][256];
    __shared__ unsigned long long ckey[kWarpSelWarps][32];
    __shared__ uint32_t cid[kWarpSelWarps][32], cpos[kWarpSelWarps][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t seg = blockIdx.x * kWarpSelWarps + warp;
    if (seg >= lv.G) return;  // warp-uniform; no block barrier below
    const uint32_t lt = (1u << lane) - 1u;
    const uint32_t nid = lv.ids[seg];
    const uint32_t start = t.start[nid], cn = t.count[nid];
    uint32_t sd = 0;
    if (lane == 0) {
        double mn[3], mx[3];
        for (int d = 0; d < 3; ++d) {
            mn[d] = ord_val(bmin[seg * 3 + d]);
            mx[d] = ord_val(bmax[seg * 3 + d]);
        }
        double size;
        choose_split(mn, mx, sd, size);
        no.split_dim[nid] = (uint8_t)sd;
        no.size[nid] = size;
    }
    sd = __shfl_sync(kFull, sd, 0);
    const double *w = pick(wx, wy, wz, sd) + start;
    const uint32_t *ids = wid + start;
    const unsigned long long kmin = bmin[seg * 3 + sd], kmax = bmax[seg * 3 + sd];
    const uint32_t rank0 = split_rank(lv, cn);
    uint32_t r = rank0, ccount = cn;
    RadixState rs;
    rs.kb = __clzll((long long)(kmin ^ kmax));
    rs.kp = rs.kb == 0 ? 0ull : (rs.kb == 64 ? kmin : (kmin >> (64 - rs.kb)));
    rs.ib = 0;
    rs.ip = 0;
    uint32_t *h = hist[warp];
    while (ccount > 32) {
        if (rs.kb == 64 && rs.ib == 32) {  // cannot happen with distinct ids
            if (lane == 0) atomicOr(err, kErrSelect);
            break;
        }
        const int wd = rs.width();
#pragma unroll
        for (int q = 0; q < 8; ++q) h[lane * 8 + q] = 0u;
        __syncwarp();
        for (uint32_t k = lane; k < cn; k += 32) {
            const unsigned long long key = ord_key(w[k]);
            const uint32_t id = ids[k];
            if (rs.match(key, id)) atomicAdd(&h[rs.digit(key, id, wd)], 1u);
        }
        __syncwarp();
        uint32_t mine = 0;
#pragma unroll
        for (int q = 0; q < 8; ++q) mine += h[lane * 8 + q];
        uint32_t inc = mine;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t v = __shfl_up_sync(kFull, inc, off);
            if (lane >= off) inc += v;
        }
        const uint32_t before = inc - mine;
        uint32_t dsel = 0, below = 0, cnt = 0;
        const bool owner = r >= before && r < inc;
        if (owner) {
            uint32_t cum = before;
            for (int q = 0; q < 8; ++q) {
                const uint32_t c = h[lane * 8 + q];
                if (r < cum + c) {
                    dsel = (uint32_t)(lane * 8 + q);
                    below = cum;
                    cnt = c;
                    break;
                }
                cum += c;
            }
        }
        const uint32_t om = __ballot_sync(kFull, owner);
        if (!om) {  // the wanted rank is not among the candidates: a failed select
            if (lane == 0) atomicOr(err, kErrSelect);
            break;
        }
        const int src = __ffs(om) - 1;
        dsel = __shfl_sync(kFull, dsel, src);
        below = __shfl_sync(kFull, below, src);
        cnt = __shfl_sync(kFull, cnt, src);
        rs.fix(dsel, wd);
        r -= below;
        ccount = cnt;
        __syncwarp();
    }
    // gather the <= 32 candidates, then rank them by comparison
    // with it, per tile the bodies that order below every candidate: they go left
    uint32_t ng = 0, lo0 = 0, lo1 = 0;
    for (uint32_t base = 0; base < cn; base += 32) {
        const uint32_t k = base + lane;
        bool hit = false;
        unsigned long long key = 0;
        uint32_t id = 0;
        if (k < cn) {
            key = ord_key(w[k]);
            id = ids[k];
            hit = rs.match(key, id);
            if (!hit && rs.below(key, id)) {
                lo0 += k < (uint32_t)kTile ? 1u : 0u;
                lo1 += k >= (uint32_t)kTile ? 1u : 0u;
            }
        }
        const uint32_t m = __ballot_sync(kFull, hit);
        if (hit) {
            const uint32_t off = ng + __popc(m & lt);
            if (off < 32) {
                ckey[warp][off] = key;
                cid[warp][off] = id;
                cpos[warp][off] = k;
            }
        }
        ng += __popc(m);
    }
    __syncwarp();
    const bool have = (uint32_t)lane < min(ng, 32u);
    const unsigned long long mk = have ? ckey[warp][lane] : ~0ull;
    const uint32_t mi = have ? cid[warp][lane] : kFull;
    uint32_t rank = 0;
    for (int q = 0; q < 32; ++q) {
        const unsigned long long ok = __shfl_sync(kFull, mk, q);
        const uint32_t oi = __shfl_sync(kFull, mi, q);
        rank += (ok < mk || (ok == mk && oi < mi)) ? 1u : 0u;
    }
    const uint32_t wm = __ballot_sync(kFull, have && rank == r);
    if (!wm) {
        if (lane == 0) atomicOr(err, kErrSelect);
        return;
    }
    if (lane == __ffs(wm) - 1) {
        const uint32_t pos = cpos[warp][lane];
        SegSel s;
        s.sd = sd;
        s.scale = 0.0f;
        s.digit = 0;
        s.c = cn;
        s.r = rank0;
        s.pad = 0;
        s.kmed = mk;
        s.idmed = mi;
        s.posmed = pos;
        s.lo = 0.0f;
        s.pad2 = 0;
        sel[seg] = s;
        no.split_val[nid] = w[pos];
    }
    if (!tile_off) return;  // one tile: the scatter counts and checks by itself
    // the bodies going left in each of the segment's (at most two) tiles: those below every
    // candidate, counted in the gather, and the candidates that order below the median
    const int ml = __ffs(wm) - 1;
    const unsigned long long kmed = __shfl_sync(kFull, mk, ml);
    const uint32_t idmed = __shfl_sync(kFull, mi, ml);
    const bool cl = have && goes_left(mk, mi, kmed, idmed);
    const uint32_t cpk = have ? cpos[warp][lane] : 0u;
    uint32_t c0 = lo0 + (cl && cpk < (uint32_t)kTile ? 1u : 0u);
    uint32_t c1 = lo1 + (cl && cpk >= (uint32_t)kTile ? 1u : 0u);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        c0 += __shfl_xor_sync(kFull, c0, o);
        c1 += __shfl_xor_sync(kFull, c1, o);
    }
    if (lane == 0) {
        uint32_t *to = tile_off + (size_t)seg * lv.tiles;
        to[0] = 0u;
        if (cn > (uint32_t)kTile) to[1] = c0;
        if (c0 + c1 != rank0) atomicOr(err, kErrSelect);
    }
}

// ------------------------------------------------------------------ the last two levels

// The last two multi-block levels (segments of at most kPairMax bodies, whose grandchildren
// are local roots; the last level alone when the whole set is its only segment) in one block
// per segment, with one read and one write of the bodies instead of two: the block stages the
// segment's positions in shared memory, selects the segment's median, reduces the children's
// bounding boxes, selects both children's medians at once, and writes the bodies out in the
// order two stable partitions leave them (the left child's left child first).  A select
// narrows its candidates with 8-bit radix passes over the key's offset from the node's
// smallest key, then over the id, and ranks the last <= 32 in one warp.
constexpr int kPairThreads = 256;
constexpr int kPairWarps = kPairThreads / 32;
static_assert(kPairMax < 65536u, "16-bit positions and per-class counts");
static_assert(kPairThreads == 256, "one thread per radix bin");

struct PairShared {
    uint32_t hist[2][256];
    uint32_t wsum[kPairWarps];
    unsigned long long wsum64[kPairWarps];
    uint32_t res[2][3];  // per selection: bin of the wanted rank, count below it, count in it
    uint32_t ccnt[2];
    unsigned long long ckey[2][32];
    uint32_t cid[2][32], cpos[2][32];
    unsigned long long kmed[2];
    uint32_t idmed[2], posmed[2], sd[2];
    uint32_t nleft;
    unsigned long long red[kPairWarps][12];
    unsigned long long box[12];  // the children's bounds: [side][min x, y, z, max x, y, z]
};

__device__ __forceinline__ RadixState radix_start(unsigned long long kmn, unsigned long long kmx) {
    RadixState q;
    q.kb = __clzll((long long)(kmn ^ kmx));
    q.kp = q.kb == 0 ? 0ull : (q.kb == 64 ? kmn : (kmn >> (64 - q.kb)));
    q.ib = 0;
    q.ip = 0;
    return q;
}

// A radix pass over the key bits (fixed bits kb < 64): the pass's digit of a key is
// (key >> sh) - base, and the key has the fixed bits exactly when that is below lim.
struct KeyWindow {
    unsigned long long base, lim;
    uint32_t sh;
};
__device__ __forceinline__ KeyWindow key_window(const RadixState &q, int w) {
    KeyWindow k;
    k.sh = (uint32_t)(64 - q.kb - w);
    k.base = q.kp << w;
    k.lim = 1ull << w;
    return k;
}

// Exact select by (key, id) of rank r0 (r1) among the bodies of selection 0 (1), along the
// coordinate array v0 (v1): with ns = 1 the whole segment of cn bodies; with ns = 2 the
// bodies j with side[j] == s, n0 and n1 of them.  kmn / kmx: each selection's bounds on that
// coordinate as ordered keys.  Leaves the median's key, id and position in P.kmed, P.idmed
// and P.posmed (key ~0 and position kFull, with kErrSelect in err, when a select fails,
// also when it would need more than max_rounds radix passes).
__device__ void pair_select(PairShared &P, const double *v0, const double *v1,
                            const uint8_t *side, uint32_t cn, const uint32_t *gid, int ns,
                            unsigned long long kmn0, unsigned long long kmx0,
                            unsigned long long kmn1, unsigned long long kmx1, uint32_t n0,
                            uint32_t n1, uint32_t r0, uint32_t r1, int max_rounds,
                            uint32_t *err) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // the passes bin key - kmn (the offset from the selection's smallest key): the first one
    // takes the 8 bits below the range's top bit and spreads the bodies over 129-256 bins,
    // where the key's own bits below its common prefix can leave them in two
    RadixState q0 = radix_start(0ull, kmx0 - kmn0), q1 = radix_start(0ull, kmx1 - kmn1);
    bool a0 = n0 > 32u, a1 = ns > 1 && n1 > 32u;  // still narrowing
    bool f0 = r0 >= n0, f1 = ns > 1 && r1 >= n1;   // failed
    a0 = a0 && !f0;
    a1 = a1 && !f1;
    for (int round = 0; a0 || a1; ++round) {
        // at most 8 passes over the key and 4 over the id (distinct ids always narrow);
        // fewer when the caller lowers the limit to test this failure path
        if (round >= max_rounds) {
            f0 = f0 || a0;
            f1 = f1 || a1;
            break;
        }
        if (a0 && q0.kb == 64 && q0.ib == 32) { a0 = false; f0 = true; }
        if (a1 && q1.kb == 64 && q1.ib == 32) { a1 = false; f1 = true; }
        if (!(a0 || a1)) break;
        const int w0 = q0.width(), w1 = q1.width();
        const KeyWindow k0 = key_window(q0, w0), k1 = key_window(q1, w1);
        // passes over the id: only for keys equal in all 64 bits
        const bool byid0 = q0.kb == 64, byid1 = q1.kb == 64;
        P.hist[0][threadIdx.x] = 0u;
        P.hist[1][threadIdx.x] = 0u;
        __syncthreads();
        for (uint32_t j = threadIdx.x; j < cn; j += kPairThreads) {
            const bool s = ns > 1 && side[j] != 0;
            if (!(s ? a1 : a0)) continue;
            const unsigned long long key = ord_key((s ? v1 : v0)[j]) - (s ? kmn1 : kmn0);
            if (s ? byid1 : byid0) {
                const RadixState q = s ? q1 : q0;
                const uint32_t id = gid[j];
                if (q.match(key, id))
                    atomicAdd(&P.hist[s ? 1 : 0][q.digit(key, id, s ? w1 : w0)], 1u);
            } else {
                const unsigned long long d = (key >> (s ? k1.sh : k0.sh)) - (s ? k1.base : k0.base);
                if (d < (s ? k1.lim : k0.lim)) atomicAdd(&P.hist[s ? 1 : 0][(uint32_t)d], 1u);
            }
        }
        __syncthreads();
        // both histograms scanned at once: selection 0 in the low 16 bits, 1 in the high
        const uint32_t h = P.hist[0][threadIdx.x] | (P.hist[1][threadIdx.x] << 16);
        uint32_t inc = h;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(kFull, inc, o);
            if (lane >= o) inc += u;
        }
        if (lane == 31) P.wsum[warp] = inc;
        __syncthreads();
        uint32_t pre = 0, tot = 0;
#pragma unroll
        for (int q = 0; q < kPairWarps; ++q) {
            const uint32_t x = P.wsum[q];
            pre += q < warp ? x : 0u;
            tot += x;
        }
        const uint32_t before = pre + inc - h;
        const uint32_t b0 = before & 0xffffu, h0 = h & 0xffffu, b1 = before >> 16, h1 = h >> 16;
        if (a0 && r0 >= b0 && r0 < b0 + h0) {
            P.res[0][0] = threadIdx.x;
            P.res[0][1] = b0;
            P.res[0][2] = h0;
        }
        if (a1 && r1 >= b1 && r1 < b1 + h1) {
            P.res[1][0] = threadIdx.x;
            P.res[1][1] = b1;
            P.res[1][2] = h1;
        }
        __syncthreads();
        // a wanted rank beyond the candidates' count has no bin: a failed select
        if (a0) {
            if (r0 >= (tot & 0xffffu)) {
                a0 = false;
                f0 = true;
            } else {
                q0.fix(P.res[0][0], w0);
                r0 -= P.res[0][1];
                a0 = P.res[0][2] > 32u;
            }
        }
        if (a1) {
            if (r1 >= (tot >> 16)) {
                a1 = false;
                f1 = true;
            } else {
                q1.fix(P.res[1][0], w1);
                r1 -= P.res[1][1];
                a1 = P.res[1][2] > 32u;
            }
        }
    }
    // the <= 32 candidates of each selection, then their ranks by (key, id) in one warp each
    if (threadIdx.x < 2) P.ccnt[threadIdx.x] = 0u;
    const KeyWindow g0 = key_window(q0, q0.width()), g1 = key_window(q1, q1.width());
    const bool byid0 = q0.kb == 64, byid1 = q1.kb == 64;
    __syncthreads();
    for (uint32_t j = threadIdx.x; j < cn; j += kPairThreads) {
        const bool s = ns > 1 && side[j] != 0;
        if (s ? f1 : f0) continue;
        const unsigned long long key = ord_key((s ? v1 : v0)[j]);
        const unsigned long long rel = key - (s ? kmn1 : kmn0);
        bool hit;
        if (s ? byid1 : byid0) {
            const RadixState q = s ? q1 : q0;
            hit = q.match(rel, gid[j]);
        } else {
            hit = (rel >> (s ? g1.sh : g0.sh)) - (s ? g1.base : g0.base) < (s ? g1.lim : g0.lim);
        }
        if (hit) {
            const uint32_t k = atomicAdd(&P.ccnt[s ? 1 : 0], 1u);
            if (k < 32u) {
                P.ckey[s ? 1 : 0][k] = key;
                P.cid[s ? 1 : 0][k] = gid[j];
                P.cpos[s ? 1 : 0][k] = j;
            }
        }
    }
    __syncthreads();
    if (warp < ns) {
        const bool failed = warp ? f1 : f0;
        const uint32_t r = warp ? r1 : r0;
        const uint32_t m = min(P.ccnt[warp], 32u);
        const bool have = !failed && (uint32_t)lane < m;
        const unsigned long long mk = have ? P.ckey[warp][lane] : ~0ull;
        const uint32_t mi = have ? P.cid[warp][lane] : kFull;
        const uint32_t mp = have ? P.cpos[warp][lane] : kFull;
        uint32_t rank = 0;
        for (int q = 0; q < 32; ++q) {
            const unsigned long long ok = __shfl_sync(kFull, mk, q);
            const uint32_t oi = __shfl_sync(kFull, mi, q);
            rank += (ok < mk || (ok == mk && oi < mi)) ? 1u : 0u;
        }
        const uint32_t wm = __ballot_sync(kFull, have && rank == r);
        const int ml = wm ? __ffs(wm) - 1 : 0;
        const unsigned long long km = __shfl_sync(kFull, mk, ml);
        const uint32_t im = __shfl_sync(kFull, mi, ml), pm = __shfl_sync(kFull, mp, ml);
        if (lane == 0) {
            P.kmed[warp] = wm ? km : ~0ull;
            P.idmed[warp] = wm ? im : kFull;
            P.posmed[warp] = wm ? pm : kFull;
            if (!wm) atomicOr(err, kErrSelect);
        }
    }
    __syncthreads();
}

__device__ __forceinline__ bool left_of(unsigned long long key, const uint32_t *gid, uint32_t j,
                                        unsigned long long kmed, uint32_t idmed) {
    // the id is read only for a key equal to the median's
    return key < kmed || (key == kmed && gid[j] < idmed);
}

__global__ __launch_bounds__(kPairThreads, 3) void k_pair(
    Topology t, const uint32_t *ids, const uint32_t *ids2, const unsigned long long *bmin,
    const unsigned long long *bmax, const double *sx, const double *sy, const double *sz,
    const uint32_t *sid, double *dx, double *dy, double *dz, uint32_t *did, NodeOut no,
    uint32_t cap, int max_rounds, uint32_t *err) {
    extern __shared__ __align__(16) unsigned char pair_raw[];
    __shared__ PairShared P;
    double *X = reinterpret_cast<double *>(pair_raw), *Y = X + cap, *Z = Y + cap;
    uint16_t *order = reinterpret_cast<uint16_t *>(Z + cap);
    uint8_t *side = reinterpret_cast<uint8_t *>(order + cap);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t seg = blockIdx.x;
    const uint32_t nid = ids[seg];
    const uint32_t start = t.start[nid], cn = t.count[nid];
    if (cn > cap) {  // block-uniform; the host sizes cap to the level's largest segment
        if (threadIdx.x == 0) atomicOr(err, kErrSelect);
        return;
    }
    const bool two = ids2 != nullptr;
    const uint32_t *gid = sid + start;
    for (uint32_t j = threadIdx.x; j < cn; j += kPairThreads) {
        cp_async8(&X[j], sx + start + j);
        cp_async8(&Y[j], sy + start + j);
        cp_async8(&Z[j], sz + start + j);
    }
    // the ids are read by the write-out (and for keys equal to a median's): brought into L2
    // now, one 128-byte line per thread
    for (uint32_t j = threadIdx.x * 32u; j < cn; j += kPairThreads * 32u)
        asm volatile("prefetch.global.L2 [%0];" ::"l"(gid + j));
    if (threadIdx.x == 0 && cn > 0) asm volatile("prefetch.global.L2 [%0];" ::"l"(gid + cn - 1));
    // the children, read after the first select
    const uint32_t id0 = two ? ids2[2 * seg] : 0u, id1 = two ? ids2[2 * seg + 1] : 0u;
    const uint32_t half0 = two ? t.count[id0] / 2 : 0u, half1 = two ? t.count[id1] / 2 : 0u;
    if (threadIdx.x == 0) {
        double mn[3], mx[3];
        for (int d = 0; d < 3; ++d) {
            mn[d] = ord_val(bmin[seg * 3 + d]);
            mx[d] = ord_val(bmax[seg * 3 + d]);
        }
        uint32_t sd;
        double size;
        choose_split(mn, mx, sd, size);
        no.split_dim[nid] = (uint8_t)sd;
        no.size[nid] = size;
        P.sd[0] = sd;
        P.nleft = 0u;
    }
    cp_async_wait_all();
    __syncthreads();

    // ---- the segment's median
    const uint32_t sdA = P.sd[0];
    const double *vA = pick(X, Y, Z, sdA);
    pair_select(P, vA, vA, side, cn, gid, 1, bmin[seg * 3 + sdA], bmax[seg * 3 + sdA], 0ull,
                0ull, cn, 0u, cn / 2, 0u, max_rounds, err);
    const unsigned long long kmA = P.kmed[0];
    const uint32_t imA = P.idmed[0];
    if (threadIdx.x == 0 && P.posmed[0] < cn) no.split_val[nid] = vA[P.posmed[0]];

    // ---- sides, and the children's bounding boxes (two levels)
    unsigned long long cmn[2][3] = {{~0ull, ~0ull, ~0ull}, {~0ull, ~0ull, ~0ull}};
    unsigned long long cmx[2][3] = {{0ull, 0ull, 0ull}, {0ull, 0ull, 0ull}};
    uint32_t nl = 0;
    for (uint32_t j = threadIdx.x; j < cn; j += kPairThreads) {
        const unsigned long long kx = ord_key(X[j]), ky = ord_key(Y[j]), kz = ord_key(Z[j]);
        const unsigned long long key = sdA == 0 ? kx : (sdA == 1 ? ky : kz);
        const bool L = left_of(key, gid, j, kmA, imA);
        side[j] = L ? 0 : 1;
        nl += L ? 1u : 0u;
        if (two) {
            if (L) {
                cmn[0][0] = min(cmn[0][0], kx); cmx[0][0] = max(cmx[0][0], kx);
                cmn[0][1] = min(cmn[0][1], ky); cmx[0][1] = max(cmx[0][1], ky);
                cmn[0][2] = min(cmn[0][2], kz); cmx[0][2] = max(cmx[0][2], kz);
            } else {
                cmn[1][0] = min(cmn[1][0], kx); cmx[1][0] = max(cmx[1][0], kx);
                cmn[1][1] = min(cmn[1][1], ky); cmx[1][1] = max(cmx[1][1], ky);
                cmn[1][2] = min(cmn[1][2], kz); cmx[1][2] = max(cmx[1][2], kz);
            }
        }
    }
    nl = __reduce_add_sync(kFull, nl);
    if (lane == 0) atomicAdd(&P.nleft, nl);
    if (two) {
#pragma unroll
        for (int c = 0; c < 2; ++c)
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                cmn[c][d] = warp_min(cmn[c][d]);
                cmx[c][d] = warp_max(cmx[c][d]);
            }
        if (lane == 0) {
#pragma unroll
            for (int c = 0; c < 2; ++c)
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    P.red[warp][6 * c + d] = cmn[c][d];
                    P.red[warp][6 * c + 3 + d] = cmx[c][d];
                }
        }
    }
    __syncthreads();
    const uint32_t nL = P.nleft;
    if (threadIdx.x == 0 && nL != cn / 2) atomicOr(err, kErrSelect);

    // ---- the children's splits and medians
    if (two) {
        if (threadIdx.x < 12) {
            const bool is_max = threadIdx.x % 6 >= 3;
            unsigned long long v = is_max ? 0ull : ~0ull;
            for (int q = 0; q < kPairWarps; ++q)
                v = is_max ? max(v, P.red[q][threadIdx.x]) : min(v, P.red[q][threadIdx.x]);
            P.box[threadIdx.x] = v;
        }
        __syncthreads();
        if (threadIdx.x < 2) {
            const int c = threadIdx.x;
            double mn[3], mx[3];
            for (int d = 0; d < 3; ++d) {
                mn[d] = ord_val(P.box[6 * c + d]);
                mx[d] = ord_val(P.box[6 * c + 3 + d]);
            }
            uint32_t sd;
            double size;
            choose_split(mn, mx, sd, size);
            const uint32_t cid = c ? id1 : id0;
            no.split_dim[cid] = (uint8_t)sd;
            no.size[cid] = size;
            P.sd[c] = sd;
        }
        __syncthreads();
        const uint32_t sd0 = P.sd[0], sd1 = P.sd[1];
        const double *v0 = pick(X, Y, Z, sd0), *v1 = pick(X, Y, Z, sd1);
        pair_select(P, v0, v1, side, cn, gid, 2, P.box[sd0], P.box[3 + sd0], P.box[6 + sd1],
                    P.box[9 + sd1], nL, cn - nL, half0, half1, max_rounds, err);
        if (threadIdx.x < 2) {
            const uint32_t pm = P.posmed[threadIdx.x];
            if (pm < cn) no.split_val[threadIdx.x ? id1 : id0] = (threadIdx.x ? v1 : v0)[pm];
        }
        const unsigned long long km0 = P.kmed[0], km1 = P.kmed[1];
        const uint32_t im0 = P.idmed[0], im1 = P.idmed[1];
        // class = 2 * side in the segment + side in the child: LL, LR, RL, RR
        for (uint32_t j = threadIdx.x; j < cn; j += kPairThreads) {
            const uint32_t sa = side[j];
            const unsigned long long key = ord_key((sa ? v1 : v0)[j]);
            const bool L = left_of(key, gid, j, sa ? km1 : km0, sa ? im1 : im0);
            side[j] = (uint8_t)(2u * sa + (L ? 0u : 1u));
        }
        __syncthreads();
    }

    // ---- stable partition by class: each thread takes a run of consecutive bodies; the
    // per-class counts (16-bit fields of one 64-bit word) are scanned over the block
    const uint32_t E = (cn + kPairThreads - 1) / kPairThreads;
    const uint32_t j0 = min(cn, threadIdx.x * E), j1 = min(cn, j0 + E);
    unsigned long long cnt = 0;
    for (uint32_t j = j0; j < j1; ++j) cnt += 1ull << (16 * side[j]);
    unsigned long long inc = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long u = __shfl_up_sync(kFull, inc, o);
        if (lane >= o) inc += u;
    }
    if (lane == 31) P.wsum64[warp] = inc;
    __syncthreads();
    unsigned long long pre = 0, tot = 0;
#pragma unroll
    for (int q = 0; q < kPairWarps; ++q) {
        const unsigned long long x = P.wsum64[q];
        pre += q < warp ? x : 0ull;
        tot += x;
    }
    unsigned long long run = pre + inc - cnt;
    const uint32_t t0 = (uint32_t)(tot & 0xffffu), t1 = (uint32_t)((tot >> 16) & 0xffffu),
                   t2 = (uint32_t)((tot >> 32) & 0xffffu);
    const uint32_t base1 = t0, base2 = t0 + t1, base3 = t0 + t1 + t2;
    if (threadIdx.x == 0 && two && (t0 != half0 || t2 != half1)) atomicOr(err, kErrSelect);
    for (uint32_t j = j0; j < j1; ++j) {
        const uint32_t c = side[j];
        const uint32_t base = c == 0 ? 0u : (c == 1 ? base1 : (c == 2 ? base2 : base3));
        order[base + (uint32_t)((run >> (16 * c)) & 0xffffu)] = (uint16_t)j;
        run += 1ull << (16 * c);
    }
    __syncthreads();
    for (uint32_t j = threadIdx.x; j < cn; j += kPairThreads) {
        const uint32_t q = order[j];
        const uint32_t dst = start + j;
        dx[dst] = X[q];
        dy[dst] = Y[q];
        dz[dst] = Z[q];
        did[dst] = gid[q];
    }
}

int launch_pair(const Topology &t, const uint32_t *ids, const uint32_t *ids2, uint32_t G,
                uint32_t cap, const unsigned long long *bmin, const unsigned long long *bmax,
                const NodeOut &no, Work &w, int cur, int max_rounds, uint32_t *err,
                cudaStream_t st) {
    const int nxt = cur ^ 1;
    const size_t smem = ((size_t)cap * (3 * sizeof(double) + sizeof(uint16_t) + 1) + 15) &
                        ~(size_t)15;
    // set on every launch: the attribute belongs to the current device's context
    cudaFuncSetAttribute(k_pair, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_pair<<<G, kPairThreads, smem, st>>>(t, ids, ids2, bmin, bmax, w.x[cur], w.y[cur],
                                          w.z[cur], w.id[cur], w.x[nxt], w.y[nxt], w.z[nxt],
                                          w.id[nxt], no, cap, max_rounds, err);
    return 1;
}

// Mixed leaf record: origin o = position of the leaf's first body, as hi + lo floats.  The
// leaf's first position is noted in perm2 for every body of the leaf, whose offset from o
// goes to trel with the tree-ordered bodies.
template <class Smem>
__device__ __forceinline__ NodeF leaf_nodef(Smem &S, uint32_t st, uint32_t cn,
                                            uint32_t s0, const LocalOut &o) {
    const uint32_t l0 = S.perm[st];
    const double ox = S.xyz[0][l0], oy = S.xyz[1][l0], oz = S.xyz[2][l0];
    for (uint32_t k = st; k < st + cn; ++k) S.perm2[k] = (uint16_t)st;
    NodeF r;
    const float hx = (float)ox, hy = (float)oy, hz = (float)oz;
    r.hi = make_float4(hx, hy, hz, 0.0f);
    r.lo = make_float4((float)(ox - (double)hx), (float)(oy - (double)hy),
                       (float)(oz - (double)hz), 0.0f);
    r.a = s0 + st;
    r.b = cn;
    r.pad0 = r.pad1 = 0u;
    return r;
}

// Sums of a leaf's bodies (tree positions [st, st+cn) of this block): full mass (f, for the
// FP64 records) and light mass (g, for the mixed records), each only when wanted.
template <class Smem>
__device__ __forceinline__ void leaf_sums(const Smem &S, uint32_t st, uint32_t cn,
                                          const LocalOut &o, double f[4], double g[4]) {
    f[0] = f[1] = f[2] = f[3] = 0.0;
    g[0] = g[1] = g[2] = g[3] = 0.0;
    for (uint32_t k = st; k < st + cn; ++k) {
        const uint32_t l = S.perm[k];
        const double mm = S.m[l];
        if (o.recd) {
            f[0] += mm;
            f[1] = fma(mm, S.xyz[0][l], f[1]);
            f[2] = fma(mm, S.xyz[1][l], f[2]);
            f[3] = fma(mm, S.xyz[2][l], f[3]);
        }
        if (o.recf && !is_heavy(S.id[l], o.heavy, o.n_heavy)) {
            g[0] += mm;
            g[1] = fma(mm, S.xyz[0][l], g[1]);
            g[2] = fma(mm, S.xyz[1][l], g[2]);
            g[3] = fma(mm, S.xyz[2][l], g[3]);
        }
    }
}

__device__ __forceinline__ void store_moments(const Moments &mo, uint32_t id, const double v[4]) {
    mo.M[id] = v[0];
    mo.S[3 * (size_t)id] = v[1];
    mo.S[3 * (size_t)id + 1] = v[2];
    mo.S[3 * (size_t)id + 2] = v[3];
}

__device__ __forceinline__ void load_moments(const Moments &mo, uint32_t id, double v[4]) {
    v[0] = mo.M[id];
    v[1] = mo.S[3 * (size_t)id];
    v[2] = mo.S[3 * (size_t)id + 1];
    v[3] = mo.S[3 * (size_t)id + 2];
}

// The bottom-up pass and the tree-ordered outputs of a finished segment: its bodies in tree
// order in perm, its internal nodes in the level table.
template <class Smem>
__device__ __forceinline__ void local_finish(Smem &S, const Topology &t, const NodeOut &no,
                                             const LocalOut &o, uint32_t root, uint32_t s0,
                                             uint32_t c0, uint32_t leaf) {
    // ================================================================ bottom-up moments
    // Three phases: every leaf at once (sums, records), the internal nodes' sums level by
    // level from the deepest (left + right), then every internal node's record at once.
    const bool want_d = o.recd != nullptr, want_f = o.recf != nullptr;
    // Node sums are also kept in shared memory, by node id within the segment's subtree
    // while they fit (every node of a 640-body subtree at leaf size 7), so that the phases
    // read them without a round trip through L2.
    const uint32_t nsets = (want_d ? 1u : 0u) + (want_f ? 1u : 0u);
    const uint32_t mslots = nsets ? (uint32_t)(kLocalWarps * 128 / 4) / nsets : 0u;
    auto keep_sums = [&](uint32_t id, const double f[4], const double g[4]) {
        if (id - root >= mslots) return;
        double *m = S.mom + 4 * (id - root) * nsets;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            if (want_d) m[q] = f[q];
            if (want_f) m[(want_d ? 4 : 0) + q] = g[q];
        }
    };
    auto read_sums = [&](uint32_t id, double f[4], double g[4]) {
        if (id - root < mslots) {
            const double *m = S.mom + 4 * (id - root) * nsets;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                if (want_d) f[q] = m[q];
                if (want_f) g[q] = m[(want_d ? 4 : 0) + q];
            }
        } else {
            if (want_d) load_moments(o.mo, id, f);
            if (want_f) load_moments(o.mof, id, g);
        }
    };
    const uint32_t nint = S.lvl_off[S.nlvl];  // internal nodes (table slots [0, nint))
    if (c0 <= leaf) {
        if (threadIdx.x == 0) {
            double f[4], g[4];
            leaf_sums(S, 0, c0, o, f, g);
            if (want_d) {
                store_moments(o.mo, root, f);
                o.recd[root] = make_noded(f[0], f[1], f[2], f[3], 0.0, s0, c0);
            }
            if (want_f) {
                store_moments(o.mof, root, g);
                o.recf[root] = leaf_nodef(S, 0, c0, s0, o);
            }
        }
    }
    // ---- leaves: the children of internal nodes with at most `leaf` bodies
    for (uint32_t u = threadIdx.x; u < 2 * nint; u += blockDim.x) {
        const uint32_t i = u >> 1;
        const uint32_t st = S.tab_st[i], cn = S.tab_cn[i], nid = S.tab_id[i];
        const uint32_t lc = cn / 2;
        const uint32_t cst = (u & 1) ? st + lc : st, ccn = (u & 1) ? cn - lc : lc;
        if (ccn > leaf) continue;
        const uint32_t cid = (u & 1) ? nid + 1 + t.ttab[lc] : nid + 1;
        double f[4], g[4];
        leaf_sums(S, cst, ccn, o, f, g);
        if (want_d) {
            store_moments(o.mo, cid, f);
            o.recd[cid] = make_noded(f[0], f[1], f[2], f[3], 0.0, s0 + cst, ccn);
        }
        if (want_f) {
            store_moments(o.mof, cid, g);
            o.recf[cid] = leaf_nodef(S, cst, ccn, s0, o);
        }
        keep_sums(cid, f, g);
    }
    __syncthreads();
    // ---- internal nodes' sums, deepest level first
    for (int L = (int)S.nlvl - 1; L >= 0; --L) {
        for (uint32_t i = S.lvl_off[L] + threadIdx.x; i < S.lvl_off[L + 1]; i += blockDim.x) {
            const uint32_t cn = S.tab_cn[i], nid = S.tab_id[i];
            const uint32_t lc = cn / 2;
            double fs[4] = {0.0, 0.0, 0.0, 0.0}, gs[4] = {0.0, 0.0, 0.0, 0.0};
            for (int side = 0; side < 2; ++side) {
                const uint32_t cid = side ? nid + 1 + t.ttab[lc] : nid + 1;
                double f[4], g[4];
                read_sums(cid, f, g);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    if (want_d) fs[q] = __dadd_rn(fs[q], f[q]);
                    if (want_f) gs[q] = __dadd_rn(gs[q], g[q]);
                }
            }
            if (want_d) store_moments(o.mo, nid, fs);
            if (want_f) store_moments(o.mof, nid, gs);
            keep_sums(nid, fs, gs);
        }
        __syncthreads();
    }
    // ---- internal nodes' records
    for (uint32_t i = threadIdx.x; i < nint; i += blockDim.x) {
        const uint32_t cn = S.tab_cn[i], nid = S.tab_id[i];
        double fs[4], gs[4];
        read_sums(nid, fs, gs);
        const double size =
            nid - root < (uint32_t)kLocalSizeSlots ? S.nsize[nid - root] : no.size[nid];
        const uint32_t right = nid + 1 + t.ttab[cn / 2];
        if (want_d) {
            const NodeD q = make_noded(fs[0], fs[1], fs[2], fs[3], size, right, 0u);
            o.recd[nid] = q;
            o.recp[nid] = make_nodep(q);
        }
        if (want_f) o.recf[nid] = make_nodef(gs[0], gs[1], gs[2], gs[3], size, right, 0u);
    }

    // ================================================================ tree-ordered bodies
    __syncthreads();  // leaf starts in perm2 (a root leaf has no level barrier above)
    for (uint32_t k = threadIdx.x; k < c0; k += blockDim.x) {
        const uint32_t l = S.perm[k];
        const uint32_t id = S.id[l];
        const double x = S.xyz[0][l], y = S.xyz[1][l], z = S.xyz[2][l], mm = S.m[l];
        if (o.tpos) o.tpos[s0 + k] = make_double4_32a(x, y, z, mm);
        o.tid[s0 + k] = id;
        {
            const float hx = (float)x, hy = (float)y, hz = (float)z;
            const bool hv = is_heavy(id, o.heavy, o.n_heavy);
            const float fm = hv ? 0.0f : (float)mm;
            // light mass split hi (thi.w) + lo (tlo.w): the heavy bodies' direct sums read
            // every light mass back to ~2^-48 relative
            const float fml = hv ? 0.0f : (float)(mm - (double)fm);
            o.thi[s0 + k] = make_float4(hx, hy, hz, fm);
            o.tlo[s0 + k] = make_float4((float)(x - (double)hx), (float)(y - (double)hy),
                                        (float)(z - (double)hz), fml);
            if (o.recf) {
                const uint32_t l0 = S.perm[S.perm2[k]];
                o.trel[s0 + k] = make_float4((float)(x - S.xyz[0][l0]), (float)(y - S.xyz[1][l0]),
                                             (float)(z - S.xyz[2][l0]), fm);
            }
        }
    }
}

// One thread block owns a segment of at most kLocalMax bodies and builds its whole subtree
// in shared memory from three sorted lists.  The segment's bodies are sorted once along each
// dimension by (ordered key, local index) -- the local index orders bodies as their ids do,
// since every partition above was stable -- with a stable block radix sort of 16-bit
// indices over the key bits below the segment's common prefix.  Each node then owns the same
// range [st, st + cn) of all three lists, each sorted along its dimension: its bounding box
// is the lists' first and last entries, its median the entry st + cn/2 of the split
// dimension's list, whose first half is the left child (the exact rank-len/2 median on
// (coordinate, body id)).  A level flags its nodes' left bodies and partitions the other two
// lists stably within every node at once (one block scan per level), so a level costs the
// same few passes over the segment whatever the size and number of its nodes.  At the end
// each leaf's bodies are put in index order, and the node sums and records are formed
// bottom-up.
template <int kCap>
struct LocalSmem {
    double xyz[3][kCap];  // positions, one row per dimension
    double m[kCap];
    uint32_t id[kCap];
    uint16_t lst[2][3][kCap];  // the three sorted lists; levels alternate between the copies
    uint16_t perm[kCap], perm2[kCap];
    union {
        struct {                     // sort, per dimension: a position's rank within its
            uint16_t rank[3][kCap];  // warp's run of its digit, and the digit
            uint8_t dig[3][kCap];
        } so;
        struct {                           // levels
            uint16_t node[kCap];           // node of a position (slot within the level)
            uint8_t fb[kCap];              // a position's partition flags, bit d for list d
            uint8_t flag[kCap];            // body goes to the left child
            uint16_t estart[3][kCap / 2];  // scan value at each node's first position
            uint16_t cslot[kCap];          // next-level slot of child 2j + side of node j
        } lv;
    };
    union {  // radix counters (sort), then internal nodes' moment sums (bottom-up)
        uint32_t hist[kLocalWarps][256];
        double mom[kLocalWarps * 128];
    };
    uint32_t tab_id[kCap];
    uint16_t tab_st[kCap], tab_cn[kCap];
    uint8_t tab_sd[kCap];
    uint32_t lvl_off[kLocalLevels + 1];
    uint32_t nlvl;
    uint32_t wcnt[kLocalWarps];
    uint32_t wscan[kLocalWarps][4];
    unsigned long long red[kLocalWarps][6];
    double nsize[kLocalSizeSlots];
};
static_assert(kLocalThreads == 256, "one thread per radix digit");
constexpr uint16_t kNoNode = 0xffffu;

// Exclusive block scan of three counts per thread (v[d] in, prefix out); `tot` gets the
// totals.  Two block barriers.
template <class Smem>
__device__ __forceinline__ void block_scan3(Smem &S, uint32_t (&v)[3], int lane, int warp) {
    uint32_t inc[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        inc[d] = v[d];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(kFull, inc[d], o);
            if (lane >= o) inc[d] += u;
        }
        if (lane == 31) S.wscan[warp][d] = inc[d];
    }
    __syncthreads();
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        uint32_t pre = 0;
        for (int w = 0; w < warp; ++w) pre += S.wscan[w][d];
        v[d] = pre + inc[d] - v[d];
    }
    __syncthreads();
}

// Stable sorts of the segment's local indices along the three dimensions by (ordered key,
// index) into S.lst[0][d], side by side: warps 0-2 sort x, 3-5 y, 6-7 z, so that the three
// sorts share every block barrier.  LSD radix passes of 8 bits over the top 24 of the key
// bits below the segment's common prefix in that dimension (all of them when there are at
// most 24, and the sort is exact); each warp ranks the positions of its chunk in order (the
// peers of a digit by eight ballots), a digit-major scan over the group's counts gives every
// run its offset, and the positions are scattered, ties keeping the index order.  Runs of keys
// equal in the sorted window -- values within about 2^-24 of the segment's range of each
// other -- are then ordered by the whole key, every entry ranking itself within its run.
template <class Smem>
__device__ void sort_lists(Smem &S, uint32_t c0, const unsigned long long (&kmin)[3],
                           const unsigned long long (&kmax)[3], int lane, int warp) {
    constexpr int kFirst[4] = {0, 3, 6, kLocalWarps};  // warps of dimension d: [kFirst[d], kFirst[d+1])
    int lsb[3], passes[3], np = 0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int dbits = kmin[d] == kmax[d] ? 0 : 64 - __clzll((long long)(kmin[d] ^ kmax[d]));
        lsb[d] = dbits > 24 ? dbits - 24 : 0;  // the sorted window is bits [lsb, dbits)
        passes[d] = (dbits - lsb[d] + 7) / 8;
        np = max(np, passes[d]);
        // ping-pong so that the last pass writes S.lst[0][d]; the first reads the identity
        uint16_t *src0 = S.lst[passes[d] & 1][d];
        for (uint32_t k = threadIdx.x; k < c0; k += blockDim.x) src0[k] = (uint16_t)k;
    }
    __syncthreads();
    // this warp's dimension and its values (selected, not indexed at run time)
    const int md = warp < kFirst[1] ? 0 : (warp < kFirst[2] ? 1 : 2);
    const int mfirst = md == 0 ? kFirst[0] : (md == 1 ? kFirst[1] : kFirst[2]);
    const int mnw = (md == 0 ? kFirst[1] : (md == 1 ? kFirst[2] : kFirst[3])) - mfirst;
    const int mlsb = md == 0 ? lsb[0] : (md == 1 ? lsb[1] : lsb[2]);
    const int mpasses = md == 0 ? passes[0] : (md == 1 ? passes[1] : passes[2]);
    const uint32_t chunk = ((c0 + mnw - 1) / mnw + 31u) & ~31u;
    const uint32_t w0 = min(c0, (uint32_t)(warp - mfirst) * chunk), w1 = min(c0, w0 + chunk);
    const uint32_t lt = (1u << lane) - 1u;
    for (int q = 0; q < np; ++q) {
        if (q < mpasses) {  // warp-uniform
            const int shift = mlsb + 8 * q;
            const uint16_t *src = S.lst[(mpasses - q) & 1][md];
            uint32_t *h = S.hist[warp];
#pragma unroll
            for (int j = 0; j < 8; ++j) h[lane * 8 + j] = 0u;
            __syncwarp();
            for (uint32_t base = w0; base < w1; base += 32) {
                const uint32_t p = base + lane;
                const bool valid = p < w1;
                const uint32_t body = valid ? src[p] : 0u;
                const uint32_t dg =
                    valid ? (uint32_t)(ord_key(S.xyz[md][body]) >> shift) & 0xffu : 0u;
                uint32_t peers = __ballot_sync(kFull, valid);
#pragma unroll
                for (int b = 0; b < 8; ++b) {
                    const uint32_t bb = __ballot_sync(kFull, (dg >> b) & 1u);
                    peers &= ((dg >> b) & 1u) ? bb : ~bb;
                }
                uint32_t cnt = 0;
                if (valid) {
                    cnt = h[dg];
                    S.so.rank[md][p] = (uint16_t)(cnt + __popc(peers & lt));
                    S.so.dig[md][p] = (uint8_t)dg;
                }
                __syncwarp();
                // the highest lane of each run adds the run's size
                if (valid && (peers >> lane) == 1u) h[dg] = cnt + __popc(peers);
                __syncwarp();
            }
        }
        __syncthreads();
        {   // thread t: offsets of digit t in each dimension, warp by warp, after every
            // smaller digit
            const uint32_t t = threadIdx.x;
            uint32_t v[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                v[d] = 0u;
                if (q < passes[d])
                    for (int w = kFirst[d]; w < kFirst[d + 1]; ++w) v[d] += S.hist[w][t];
            }
            block_scan3(S, v, lane, warp);
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                if (q >= passes[d]) continue;
                uint32_t run = v[d];
                for (int w = kFirst[d]; w < kFirst[d + 1]; ++w) {
                    const uint32_t c = S.hist[w][t];
                    S.hist[w][t] = run;
                    run += c;
                }
            }
        }
        __syncthreads();
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            if (q >= passes[d]) continue;
            const uint16_t *src = S.lst[(passes[d] - q) & 1][d];
            uint16_t *dst = S.lst[(passes[d] - q - 1) & 1][d];
            const uint32_t cd = ((c0 + (kFirst[d + 1] - kFirst[d]) - 1) /
                                     (uint32_t)(kFirst[d + 1] - kFirst[d]) + 31u) & ~31u;
            for (uint32_t p = threadIdx.x; p < c0; p += blockDim.x)
                dst[S.hist[kFirst[d] + p / cd][S.so.dig[d][p]] + S.so.rank[d][p]] = src[p];
        }
        __syncthreads();
    }
    // runs of keys equal in the window, in whole-key order: every position of a run ranks its
    // body among the run's by (key, index) and is written to that rank, in parallel
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if (lsb[d] == 0) continue;  // every distinguishing bit was sorted on
        const uint16_t *l = S.lst[0][d];
        uint16_t *tmp = S.lst[1][d];
        const int sh = lsb[d];
        for (uint32_t p = threadIdx.x; p < c0; p += blockDim.x) {
            const uint16_t v = l[p];
            const unsigned long long kv = ord_key(S.xyz[d][v]), wv = kv >> sh;
            uint32_t a2 = p, e = p + 1;  // the run [a2, e)
            while (a2 > 0 && (ord_key(S.xyz[d][l[a2 - 1]]) >> sh) == wv) --a2;
            while (e < c0 && (ord_key(S.xyz[d][l[e]]) >> sh) == wv) ++e;
            uint32_t r = 0;
            for (uint32_t k = a2; k < e; ++k) {
                const uint16_t u = l[k];
                const unsigned long long ku = ord_key(S.xyz[d][u]);
                r += (ku < kv || (ku == kv && u < v)) ? 1u : 0u;
            }
            tmp[a2 + r] = v;
        }
    }
    __syncthreads();
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if (lsb[d] == 0) continue;
        for (uint32_t p = threadIdx.x; p < c0; p += blockDim.x) S.lst[0][d][p] = S.lst[1][d][p];
    }
    __syncthreads();
}

template <int kCap>
__global__ __launch_bounds__(kLocalThreads, 4) void k_local(
    Topology t, const uint32_t *roots, NodeOut no, const double *wx, const double *wy,
    const double *wz, const uint32_t *wid, LocalOut o, uint32_t *err) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    LocalSmem<kCap> &S = *reinterpret_cast<LocalSmem<kCap> *>(smem_raw);
    const uint32_t root = roots[blockIdx.x];
    const uint32_t s0 = t.start[root], c0 = t.count[root];
    const uint32_t leaf = t.leaf;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

    unsigned long long kmn[3] = {~0ull, ~0ull, ~0ull}, kmx[3] = {0ull, 0ull, 0ull};
    for (uint32_t k = threadIdx.x; k < c0; k += blockDim.x) {
        const double x = wx[s0 + k], y = wy[s0 + k], z = wz[s0 + k];
        S.xyz[0][k] = x;
        S.xyz[1][k] = y;
        S.xyz[2][k] = z;
        const uint32_t id = wid[s0 + k];
        S.id[k] = id;
        S.m[k] = o.mass[id];
        const unsigned long long k0 = ord_key(x), k1 = ord_key(y), k2 = ord_key(z);
        kmn[0] = min(kmn[0], k0); kmx[0] = max(kmx[0], k0);
        kmn[1] = min(kmn[1], k1); kmx[1] = max(kmx[1], k1);
        kmn[2] = min(kmn[2], k2); kmx[2] = max(kmx[2], k2);
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        kmn[d] = warp_min(kmn[d]);
        kmx[d] = warp_max(kmx[d]);
    }
    if (lane == 0) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            S.red[warp][d] = kmn[d];
            S.red[warp][3 + d] = kmx[d];
        }
    }
    if (threadIdx.x == 0) {
        const uint32_t g0 = c0 > leaf ? 1u : 0u;
        S.tab_st[0] = 0;
        S.tab_cn[0] = (uint16_t)c0;
        S.tab_id[0] = root;
        S.lvl_off[0] = 0;
        S.lvl_off[1] = g0;
        S.nlvl = g0;
    }
    __syncthreads();

    if (c0 > leaf) {  // block-uniform
        // ================================================================ sorted lists
        unsigned long long a[3], b[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            a[d] = ~0ull;
            b[d] = 0ull;
            for (int w = 0; w < kLocalWarps; ++w) {
                a[d] = min(a[d], S.red[w][d]);
                b[d] = max(b[d], S.red[w][3 + d]);
            }
        }
        sort_lists(S, c0, a, b, lane, warp);
        // ================================================================ levels
        int cur = 0;
        uint32_t plo = 0;  // first table slot of the previous level
        for (uint32_t L = 0;; ++L) {
            const uint32_t lo = S.lvl_off[L], hi = S.lvl_off[L + 1];
            if (hi == lo) break;
            uint16_t(*Lc)[kCap] = S.lst[cur];
            uint16_t(*Ln)[kCap] = S.lst[cur ^ 1];
            // ---- split of every node: bounds from the lists' ends, median at st + cn/2
            for (uint32_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
                const uint32_t st = S.tab_st[i], cn = S.tab_cn[i], nid = S.tab_id[i];
                double mn[3], mx[3];
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    mn[d] = S.xyz[d][Lc[d][st]];
                    mx[d] = S.xyz[d][Lc[d][st + cn - 1]];
                }
                uint32_t sd;
                double size;
                choose_split(mn, mx, sd, size);
                const double sv = S.xyz[sd][Lc[sd][st + cn / 2]];
                no.split_dim[nid] = (uint8_t)sd;
                no.size[nid] = size;
                no.split_val[nid] = sv;
                if (nid - root < (uint32_t)kLocalSizeSlots) S.nsize[nid - root] = size;
                S.tab_sd[i] = (uint8_t)sd;
            }
            __syncthreads();
            // ---- each position's node (from its parent's node and side); the left bodies
            // flagged from the split lists
            for (uint32_t p = threadIdx.x; p < c0; p += blockDim.x) {
                uint32_t j = 0;
                if (L > 0) {
                    const uint32_t jp = S.lv.node[p];  // node of p one level up
                    if (jp != kNoNode) {
                        const uint32_t ip = plo + jp;
                        const uint32_t side = p >= (uint32_t)S.tab_st[ip] + S.tab_cn[ip] / 2u;
                        j = S.lv.cslot[2 * jp + side];
                    } else {
                        j = kNoNode;
                    }
                }
                S.lv.node[p] = (uint16_t)j;
                if (j != kNoNode) {
                    const uint32_t i = lo + j;
                    const uint32_t st = S.tab_st[i], cn = S.tab_cn[i], sd = S.tab_sd[i];
                    // a node whose children are both leaves keeps its lists unpartitioned:
                    // its leaves are read from its split dimension's list
                    if (cn > 2u * leaf) S.lv.flag[Lc[sd][p]] = (p - st) < cn / 2 ? 1u : 0u;
                }
            }
            __syncthreads();
            // ---- stable partition of the lists inside every node: a block scan of the left
            // flags along each list (zero where a list needs no partition) gives each left
            // body its rank among the node's left bodies
            const uint32_t per = (c0 + blockDim.x - 1) / blockDim.x;
            const uint32_t p0 = min(c0, threadIdx.x * per), p1 = min(c0, p0 + per);
            // the flags of position p along the three lists, bit d (zero where the list
            // needs no partition), kept in dig[p]
            uint32_t e[3] = {0u, 0u, 0u};
            for (uint32_t p = p0; p < p1; ++p) {
                const uint32_t j = S.lv.node[p];
                uint32_t fb = 0u;
                if (j != kNoNode && S.tab_cn[lo + j] > 2u * leaf) {
                    const uint32_t sd = S.tab_sd[lo + j];
#pragma unroll
                    for (int d = 0; d < 3; ++d)
                        if ((uint32_t)d != sd) fb |= (uint32_t)S.lv.flag[Lc[d][p]] << d;
                }
                S.lv.fb[p] = (uint8_t)fb;
#pragma unroll
                for (int d = 0; d < 3; ++d) e[d] += (fb >> d) & 1u;
            }
            block_scan3(S, e, lane, warp);
            {   // the scan value at every node's first position
                uint32_t r[3] = {e[0], e[1], e[2]};
                for (uint32_t p = p0; p < p1; ++p) {
                    const uint32_t j = S.lv.node[p];
                    if (j != kNoNode && p == S.tab_st[lo + j]) {
#pragma unroll
                        for (int d = 0; d < 3; ++d) S.lv.estart[d][j] = (uint16_t)r[d];
                    }
                    const uint32_t fb = S.lv.fb[p];
#pragma unroll
                    for (int d = 0; d < 3; ++d) r[d] += (fb >> d) & 1u;
                }
            }
            __syncthreads();
            for (uint32_t p = p0; p < p1; ++p) {
                const uint32_t j = S.lv.node[p];
                const uint32_t fb = S.lv.fb[p];
                uint32_t st = 0, half = 0, sd = 3;
                const bool part = j != kNoNode && S.tab_cn[lo + j] > 2u * leaf;
                if (part) {
                    st = S.tab_st[lo + j];
                    half = S.tab_cn[lo + j] / 2u;
                    sd = S.tab_sd[lo + j];
                }
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    const uint16_t v = Lc[d][p];
                    uint32_t q = p;
                    if (part && (uint32_t)d != sd) {
                        const uint32_t f = (fb >> d) & 1u;
                        const uint32_t rl = e[d] - S.lv.estart[d][j];  // left bodies before p
                        q = f ? st + rl : st + half + (p - st - rl);
                        e[d] += f;
                    }
                    Ln[d][q] = v;
                }
            }
            __syncthreads();
            cur ^= 1;
            // ---- children that are still internal, appended as the next level
            const uint32_t G = hi - lo;
            uint32_t fill = hi;
            for (uint32_t base = 0; base < 2 * G; base += blockDim.x) {
                const uint32_t u = base + threadIdx.x;
                bool keep = false;
                uint32_t cst = 0, ccn = 0, cid = 0;
                if (u < 2 * G) {
                    const uint32_t i = lo + (u >> 1);
                    const uint32_t st = S.tab_st[i], cn = S.tab_cn[i], id = S.tab_id[i];
                    const uint32_t lc = cn / 2;
                    if (u & 1) {
                        cst = st + lc;
                        ccn = cn - lc;
                        cid = id + 1 + t.ttab[lc];
                    } else {
                        cst = st;
                        ccn = lc;
                        cid = id + 1;
                    }
                    keep = ccn > leaf;
                }
                const uint32_t m = __ballot_sync(kFull, keep);
                if (lane == 0) S.wcnt[warp] = __popc(m);
                __syncthreads();
                uint32_t off = fill, tot = 0;
                for (int q = 0; q < kLocalWarps; ++q) {
                    if (q < warp) off += S.wcnt[q];
                    tot += S.wcnt[q];
                }
                if (u < 2 * G) {
                    const uint32_t slot = off + __popc(m & ((1u << lane) - 1u));
                    S.lv.cslot[u] = keep && slot < (uint32_t)kCap ? (uint16_t)(slot - hi) : kNoNode;
                    if (keep && slot < (uint32_t)kCap) {
                        S.tab_st[slot] = (uint16_t)cst;
                        S.tab_cn[slot] = (uint16_t)ccn;
                        S.tab_id[slot] = cid;
                    }
                }
                fill += tot;
                __syncthreads();
            }
            if (threadIdx.x == 0) {
                if (L + 2 > (uint32_t)kLocalLevels || fill > (uint32_t)kCap) {
                    atomicOr(err, kErrSelect);
                    fill = hi;  // stop: cannot happen for segments of <= kCap bodies
                }
                S.lvl_off[L + 2] = fill;
                if (fill > hi) S.nlvl = L + 2;
            }
            __syncthreads();
            plo = lo;
        }
        // ================================================================ leaf order
        // every leaf's bodies (the same in all three lists) in index order
        uint16_t(*Lf)[kCap] = S.lst[cur];
        const uint32_t nint = S.lvl_off[S.nlvl];
        for (uint32_t u = threadIdx.x; u < 2 * nint; u += blockDim.x) {
            const uint32_t i = u >> 1;
            const uint32_t st = S.tab_st[i], cn = S.tab_cn[i], lc = cn / 2;
            const uint32_t cst = (u & 1) ? st + lc : st, ccn = (u & 1) ? cn - lc : lc;
            if (ccn > leaf) continue;
            // a parent with two leaves left its other lists unpartitioned
            const uint16_t *lf = cn > 2u * leaf ? Lf[0] : Lf[S.tab_sd[i]];
            for (uint32_t a = 0; a < ccn; ++a) {  // insertion sort of <= leaf entries
                const uint16_t v = lf[cst + a];
                uint32_t b = a;
                while (b > 0 && S.perm[cst + b - 1] > v) {
                    S.perm[cst + b] = S.perm[cst + b - 1];
                    --b;
                }
                S.perm[cst + b] = v;
            }
        }
    } else {
        for (uint32_t k = threadIdx.x; k < c0; k += blockDim.x) S.perm[k] = (uint16_t)k;
    }
    __syncthreads();
    local_finish(S, t, no, o, root, s0, c0, leaf);
}

void launch_local(const Topology &t, const uint32_t *roots, uint32_t n_roots,
                  const NodeOut &no, const Work &w, int cur, const LocalOut &out,
                  uint32_t *err, cudaStream_t st) {
    // set on every launch: the attribute belongs to the current device's context, and a
    // process may hold contexts on several devices
    const size_t smem = sizeof(LocalSmem<kLocalMax>);
    cudaFuncSetAttribute(k_local<kLocalMax>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    k_local<kLocalMax><<<n_roots, kLocalThreads, smem, st>>>(t, roots, no, w.x[cur], w.y[cur],
                                                             w.z[cur], w.id[cur], out, err);
}

// ------------------------------------------------------------------ moments above the local roots

// One thread per local root climbs; the second child to arrive at a parent combines both
// children (left + right, a fixed order) and continues upward.
__global__ void k_moments_top(Topology t, const uint32_t *roots, uint32_t n_roots, NodeOut no,
                              LocalOut o) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_roots) return;
    const bool want_d = o.recd != nullptr, want_f = o.recf != nullptr;
    uint32_t node = t.parent[roots[i]];
    uint32_t *counter = want_d ? o.mo.counter : o.mof.counter;
    while (node != 0xffffffffu) {
        __threadfence();
        if (atomicAdd(&counter[node], 1u) == 0u) return;
        __threadfence();
        const uint32_t L = node + 1, R = t.right[node];
        const double size = no.size[node];
        if (want_d) {
            double v[4];
            v[0] = __dadd_rn(__ldcg(&o.mo.M[L]), __ldcg(&o.mo.M[R]));
            for (int d = 0; d < 3; ++d)
                v[1 + d] = __dadd_rn(__ldcg(&o.mo.S[3 * (size_t)L + d]),
                                     __ldcg(&o.mo.S[3 * (size_t)R + d]));
            store_moments(o.mo, node, v);
            const NodeD q = make_noded(v[0], v[1], v[2], v[3], size, R, 0u);
            o.recd[node] = q;
            o.recp[node] = make_nodep(q);
        }
        if (want_f) {
            double v[4];
            v[0] = __dadd_rn(__ldcg(&o.mof.M[L]), __ldcg(&o.mof.M[R]));
            for (int d = 0; d < 3; ++d)
                v[1 + d] = __dadd_rn(__ldcg(&o.mof.S[3 * (size_t)L + d]),
                                     __ldcg(&o.mof.S[3 * (size_t)R + d]));
            store_moments(o.mof, node, v);
            o.recf[node] = make_nodef(v[0], v[1], v[2], v[3], size, R, 0u);
        }
        node = t.parent[node];
    }
}

void launch_moments_top(const Topology &t, const uint32_t *roots, uint32_t n_roots,
                        const NodeOut &no, const LocalOut &out, cudaStream_t st) {
    uint32_t *counter = out.recd ? out.mo.counter : out.mof.counter;
    cudaMemsetAsync(counter, 0, sizeof(uint32_t) * t.n_nodes, st);
    k_moments_top<<<(n_roots + 127) / 128, 128, 0, st>>>(t, roots, n_roots, no, out);
}

}  // namespace kd
