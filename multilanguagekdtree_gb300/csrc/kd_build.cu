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
// (bounding box -> split -> radix select -> stable partition into the other ping-pong
// buffer); below that, one thread block takes a whole segment into shared memory and
// finishes its subtree there (bitonic sort per sub-segment per level).
#include "kd_internal.cuh"

namespace kd {

static constexpr uint32_t kFull = 0xffffffffu;

// Order-preserving map double -> uint64 (no NaN reaches the build).  -0.0 and +0.0 compare
// equal under the reference's `<`, so both get the key of +0.0.
__device__ __forceinline__ unsigned long long ord_key(double v) {
    unsigned long long b = (unsigned long long)__double_as_longlong(v);
    if (v == 0.0) b = 0ull;
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double ord_val(unsigned long long k) {
    unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double((long long)b);
}

__device__ __forceinline__ const double *pick(const double *x, const double *y,
                                              const double *z, uint32_t d) {
    return d == 0 ? x : (d == 1 ? y : z);
}

// Split dimension and size from a bounding box, as array_kd_tree.rs:532-557: the box starts
// at +-1e100, the extent is max - min, the first strictly larger extent wins.
__device__ __forceinline__ void choose_split(const double mn_in[3], const double mx_in[3],
                                             uint32_t &sd, double &size) {
    double mn[3], mx[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        mn[d] = fmin(1e100, mn_in[d]);
        mx[d] = fmax(-1e100, mx_in[d]);
    }
    sd = 0;
#pragma unroll
    for (int d = 1; d < 3; ++d)
        if (__dsub_rn(mx[d], mn[d]) > __dsub_rn(mx[sd], mn[sd])) sd = (uint32_t)d;
    size = __dsub_rn(mx[sd], mn[sd]);
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

__global__ void k_init_work(Bodies b, double *wx, double *wy, double *wz, uint32_t *wid,
                            uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x) {
        wx[i] = b.x[i];
        wy[i] = b.y[i];
        wz[i] = b.z[i];
        wid[i] = i;
    }
}

void launch_init_work(const Bodies &b, Work &w, uint32_t n, cudaStream_t st) {
    int blocks = (int)((n + 255) / 256);
    if (blocks > 4096) blocks = 4096;
    k_init_work<<<blocks, 256, 0, st>>>(b, w.x[0], w.y[0], w.z[0], w.id[0], n);
}

// ------------------------------------------------------------------ level passes

struct TileRef {
    uint32_t seg, tile, id, start, cnt, lo, hi;
};

__device__ __forceinline__ bool tile_of(const Topology &t, const LevelArgs &lv, TileRef &r) {
    r.seg = blockIdx.x / lv.tiles;
    r.tile = blockIdx.x - r.seg * lv.tiles;
    r.id = lv.ids[r.seg];
    r.start = t.start[r.id];
    r.cnt = t.count[r.id];
    r.lo = r.tile * (uint32_t)kTile;
    if (r.lo >= r.cnt) return false;
    r.hi = min(r.cnt, r.lo + (uint32_t)kTile);
    return true;
}

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
    double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t k = r.lo + threadIdx.x; k < r.hi; k += blockDim.x) {
        double v0 = wx[r.start + k], v1 = wy[r.start + k], v2 = wz[r.start + k];
        mn[0] = fmin(mn[0], v0); mx[0] = fmax(mx[0], v0);
        mn[1] = fmin(mn[1], v1); mx[1] = fmax(mx[1], v1);
        mn[2] = fmin(mn[2], v2); mx[2] = fmax(mx[2], v2);
    }
    __shared__ double red[kTileThreads / 32][6];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        mn[d] = warp_fmin(mn[d]);
        mx[d] = warp_fmax(mx[d]);
    }
    if (lane == 0) {
        for (int d = 0; d < 3; ++d) { red[warp][d] = mn[d]; red[warp][3 + d] = mx[d]; }
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        int d = threadIdx.x;
        double a = INFINITY, b = -INFINITY;
        for (int w = 0; w < kTileThreads / 32; ++w) {
            a = fmin(a, red[w][d]);
            b = fmax(b, red[w][3 + d]);
        }
        atomicMin(&bmin[r.seg * 3 + d], ord_key(a));
        atomicMax(&bmax[r.seg * 3 + d], ord_key(b));
    }
}

// Split dimension, size and the first radix window of every segment.
__global__ void k_split(Topology t, LevelArgs lv, const unsigned long long *bmin,
                        const unsigned long long *bmax, SegSel *sel, NodeOut no) {
    uint32_t seg = blockIdx.x * blockDim.x + threadIdx.x;
    if (seg >= lv.G) return;
    uint32_t id = lv.ids[seg];
    uint32_t cnt = t.count[id];
    double mn[3], mx[3];
    for (int d = 0; d < 3; ++d) {
        mn[d] = ord_val(bmin[seg * 3 + d]);
        mx[d] = ord_val(bmax[seg * 3 + d]);
    }
    uint32_t sd;
    double size;
    choose_split(mn, mx, sd, size);
    no.split_dim[id] = (uint8_t)sd;
    no.size[id] = size;
    unsigned long long kmin = bmin[seg * 3 + sd], kmax = bmax[seg * 3 + sd];
    int b = 64 - __clzll((long long)(kmin ^ kmax));
    SegSel s;
    s.sd = sd;
    s.shift = b > kHistBits ? (uint32_t)(b - kHistBits) : 0u;
    s.digit = 0;
    s.c = cnt;
    s.r = cnt / 2;
    s.pad = 0;
    s.kmed = 0;
    s.idmed = 0;
    s.posmed = 0;
    sel[seg] = s;
}

// First radix pass over big segments: histogram of the 12 bits just below the common
// prefix of the segment's keys.
__global__ __launch_bounds__(kTileThreads) void k_hist(Topology t, LevelArgs lv,
                                                       const double *wx, const double *wy,
                                                       const double *wz, const SegSel *sel,
                                                       uint32_t *hist) {
    TileRef r;
    if (!tile_of(t, lv, r)) return;
    __shared__ uint32_t h[kHistBins];
    for (int b = threadIdx.x; b < kHistBins; b += blockDim.x) h[b] = 0;
    __syncthreads();
    const SegSel s = sel[r.seg];
    const double *w = pick(wx, wy, wz, s.sd) + r.start;
    for (uint32_t k = r.lo + threadIdx.x; k < r.hi; k += blockDim.x) {
        uint32_t dig = (uint32_t)(ord_key(w[k]) >> s.shift) & (kHistBins - 1);
        atomicAdd(&h[dig], 1u);
    }
    __syncthreads();
    uint32_t *gh = hist + (size_t)r.seg * kHistBins;
    for (int b = threadIdx.x; b < kHistBins; b += blockDim.x)
        if (h[b]) atomicAdd(&gh[b], h[b]);
}

// Block-wide search of the histogram bin holding rank r.  Every thread owns
// kHistBins/blockDim consecutive bins.  Returns digit / count below / count in bin through
// shared memory.
__device__ void find_bin(const uint32_t *h, uint32_t r, uint32_t *out3) {
    const int per = kHistBins / blockDim.x;
    __shared__ uint32_t wsum[32];
    uint32_t mine = 0;
    for (int i = 0; i < per; ++i) mine += h[threadIdx.x * per + i];
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

__global__ __launch_bounds__(kTileThreads) void k_find(const uint32_t *hist, SegSel *sel) {
    __shared__ uint32_t out3[3];
    const uint32_t seg = blockIdx.x;
    find_bin(hist + (size_t)seg * kHistBins, sel[seg].r, out3);
    if (threadIdx.x == 0) {
        sel[seg].digit = out3[0];
        sel[seg].r -= out3[1];
        sel[seg].c = out3[2];
    }
}

// Gather the keys of the selected first-pass bin as candidates (unordered; the exact
// select below does not depend on their order).
__global__ __launch_bounds__(kTileThreads) void k_collect(Topology t, LevelArgs lv,
                                                          const double *wx, const double *wy,
                                                          const double *wz, const SegSel *sel,
                                                          uint32_t *cand_cnt,
                                                          unsigned long long *ckey,
                                                          uint32_t *cpos) {
    TileRef r;
    if (!tile_of(t, lv, r)) return;
    const SegSel s = sel[r.seg];
    const double *w = pick(wx, wy, wz, s.sd) + r.start;
    const int lane = threadIdx.x & 31;
    for (uint32_t base = r.lo; base < r.hi; base += blockDim.x) {
        uint32_t k = base + threadIdx.x;
        bool in = k < r.hi;
        unsigned long long key = in ? ord_key(w[k]) : 0ull;
        bool hit = in && (((uint32_t)(key >> s.shift) & (kHistBins - 1)) == s.digit);
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
}

// Exact median of every segment: radix refinement until at most kSelCap candidates are
// left, then a bitonic sort of (key, id) in shared memory and a pick at the wanted rank.
// Candidates start as the collected first-pass bin (multi) or the whole segment.
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

    const uint32_t seg = blockIdx.x;
    const uint32_t nid = lv.ids[seg];
    const uint32_t start = t.start[nid];
    SegSel st = sel[seg];
    const double *w = pick(wx, wy, wz, st.sd) + start;
    const uint32_t *ids = wid + start;
    uint32_t c = st.c, r = st.r;
    int src = lv.multi ? 0 : -1;  // -1: the candidates are the segment itself
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;

    auto get = [&](uint32_t j, unsigned long long &key, uint32_t &pos) {
        if (src < 0) {
            pos = j;
            key = ord_key(w[j]);
        } else {
            pos = s.cpos[src][start + j];
            key = s.ckey[src][start + j];
        }
    };

    for (int iter = 0; c > (uint32_t)kSelCap; ++iter) {
        if (iter >= kSelMaxIters) {
            if (threadIdx.x == 0) atomicOr(s.err, kErrSelect);
            c = kSelCap;
            if (r >= c) r = c - 1;
            break;
        }
        // key and id range of the candidates
        unsigned long long kmn = ~0ull, kmx = 0ull;
        uint32_t imn = kFull, imx = 0u;
        for (uint32_t j = threadIdx.x; j < c; j += blockDim.x) {
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
        for (int b = threadIdx.x; b < kHistBins; b += blockDim.x) h[b] = 0;
        if (threadIdx.x == 0) ncomp = 0;
        __syncthreads();
        kmn = ~0ull; kmx = 0; imn = kFull; imx = 0;
        for (int i = 0; i < nw; ++i) {
            kmn = min(kmn, red_k[0][i]); kmx = max(kmx, red_k[1][i]);
            imn = min(imn, red_i[0][i]); imx = max(imx, red_i[1][i]);
        }
        const bool bykey = kmn != kmx;
        int bits = bykey ? 64 - __clzll((long long)(kmn ^ kmx)) : 32 - __clz((int)(imn ^ imx));
        const uint32_t shift = bits > kHistBits ? (uint32_t)(bits - kHistBits) : 0u;
        auto digit = [&](unsigned long long key, uint32_t id) -> uint32_t {
            return bykey ? ((uint32_t)(key >> shift) & (kHistBins - 1))
                         : ((id >> shift) & (kHistBins - 1));
        };
        for (uint32_t j = threadIdx.x; j < c; j += blockDim.x) {
            unsigned long long key;
            uint32_t pos;
            get(j, key, pos);
            atomicAdd(&h[digit(key, ids[pos])], 1u);
        }
        __syncthreads();
        find_bin(h, r, out3);
        const uint32_t dig = out3[0], below = out3[1], inbin = out3[2];
        const int dst = src == 0 ? 1 : 0;
        for (uint32_t base = 0; base < c; base += blockDim.x) {
            uint32_t j = base + threadIdx.x;
            bool in = j < c;
            unsigned long long key = 0;
            uint32_t pos = 0;
            if (in) get(j, key, pos);
            bool hit = in && digit(key, ids[pos]) == dig;
            uint32_t m = __ballot_sync(kFull, hit);
            if (m) {
                uint32_t leader = __ffs(m) - 1, slot = 0;
                if (lane == (int)leader) slot = atomicAdd(&ncomp, (uint32_t)__popc(m));
                slot = __shfl_sync(kFull, slot, leader);
                if (hit) {
                    uint32_t o = slot + __popc(m & ((1u << lane) - 1u));
                    s.ckey[dst][start + o] = key;
                    s.cpos[dst][start + o] = pos;
                }
            }
        }
        __syncthreads();
        c = inbin;
        r -= below;
        src = dst;
        __syncthreads();
    }

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
    }
}

__device__ __forceinline__ bool goes_left(unsigned long long key, uint32_t id,
                                          unsigned long long kmed, uint32_t idmed) {
    return key < kmed || (key == kmed && id < idmed);
}

__global__ __launch_bounds__(kTileThreads) void k_part_count(Topology t, LevelArgs lv,
                                                             const double *wx, const double *wy,
                                                             const double *wz,
                                                             const uint32_t *wid,
                                                             const SegSel *sel,
                                                             uint32_t *tile_cnt) {
    TileRef r;
    if (!tile_of(t, lv, r)) return;
    const SegSel s = sel[r.seg];
    const double *w = pick(wx, wy, wz, s.sd) + r.start;
    const uint32_t *ids = wid + r.start;
    uint32_t cnt = 0;
    for (uint32_t k = r.lo + threadIdx.x; k < r.hi; k += blockDim.x)
        cnt += goes_left(ord_key(w[k]), ids[k], s.kmed, s.idmed) ? 1u : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(kFull, cnt, o);
    __shared__ uint32_t ws[kTileThreads / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t tot = 0;
        for (int i = 0; i < kTileThreads / 32; ++i) tot += ws[i];
        tile_cnt[(size_t)r.seg * lv.tiles + r.tile] = tot;
    }
}

// Exclusive scan of the left counts over the tiles of each segment; checks that exactly
// len/2 bodies go left.
__global__ __launch_bounds__(256) void k_tile_scan(Topology t, LevelArgs lv,
                                                   const uint32_t *tile_cnt, uint32_t *tile_off,
                                                   uint32_t *err) {
    const uint32_t seg = blockIdx.x;
    const uint32_t cnt = t.count[lv.ids[seg]];
    const uint32_t ntiles = (cnt + kTile - 1) / kTile;
    const uint32_t *tc = tile_cnt + (size_t)seg * lv.tiles;
    uint32_t *to = tile_off + (size_t)seg * lv.tiles;
    __shared__ uint32_t wsum[8];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint32_t base = 0; base < ntiles; base += blockDim.x) {
        uint32_t i = base + threadIdx.x;
        uint32_t v = i < ntiles ? tc[i] : 0u;
        uint32_t inc = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t u = __shfl_up_sync(kFull, inc, o);
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
    if (threadIdx.x == 0 && carry != cnt / 2) atomicOr(err, kErrSelect);
}

// Stable partition: bodies keep their relative order inside each child.
__global__ __launch_bounds__(kTileThreads) void k_part_scatter(
    Topology t, LevelArgs lv, const double *sx, const double *sy, const double *sz,
    const uint32_t *sid, double *dx, double *dy, double *dz, uint32_t *did, const SegSel *sel,
    const uint32_t *tile_off) {
    TileRef r;
    if (!tile_of(t, lv, r)) return;
    const SegSel s = sel[r.seg];
    const uint32_t mid = r.cnt / 2;
    const uint32_t lbase = tile_off[(size_t)r.seg * lv.tiles + r.tile];
    const uint32_t rbase = r.lo - lbase;
    __shared__ uint32_t wl[kTileThreads / 32], wr[kTileThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t lt = (1u << lane) - 1u;
    uint32_t runL = 0, runR = 0;
    for (uint32_t base = r.lo; base < r.hi; base += blockDim.x) {
        uint32_t k = base + threadIdx.x;
        bool in = k < r.hi;
        double vx = 0, vy = 0, vz = 0;
        uint32_t id = 0;
        if (in) {
            vx = sx[r.start + k];
            vy = sy[r.start + k];
            vz = sz[r.start + k];
            id = sid[r.start + k];
        }
        double key = s.sd == 0 ? vx : (s.sd == 1 ? vy : vz);
        bool isL = in && goes_left(ord_key(key), id, s.kmed, s.idmed);
        bool isR = in && !isL;
        uint32_t bl = __ballot_sync(kFull, isL), br = __ballot_sync(kFull, isR);
        if (lane == 0) { wl[warp] = __popc(bl); wr[warp] = __popc(br); }
        __syncthreads();
        uint32_t offL = 0, offR = 0, totL = 0, totR = 0;
        for (int q = 0; q < kTileThreads / 32; ++q) {
            if (q < warp) { offL += wl[q]; offR += wr[q]; }
            totL += wl[q];
            totR += wr[q];
        }
        const uint32_t dst = isL ? r.start + lbase + runL + offL + __popc(bl & lt)
                                 : r.start + mid + rbase + runR + offR + __popc(br & lt);
        // a failed select (flagged by k_tile_scan) must not write outside the segment
        if (in && dst < r.start + r.cnt) {
            dx[dst] = vx;
            dy[dst] = vy;
            dz[dst] = vz;
            did[dst] = id;
        }
        runL += totL;
        runR += totR;
        __syncthreads();
    }
}

int launch_level(const Topology &t, const LevelArgs &lv, const NodeOut &no, Work &w, int cur,
                 Scratch &s, cudaStream_t st) {
    const int nxt = cur ^ 1;
    const uint32_t G = lv.G;
    const uint32_t grid = G * lv.tiles;
    cudaMemsetAsync(s.bmin, 0xff, sizeof(unsigned long long) * 3 * G, st);
    cudaMemsetAsync(s.bmax, 0x00, sizeof(unsigned long long) * 3 * G, st);
    k_bbox<<<grid, kTileThreads, 0, st>>>(t, lv, w.x[cur], w.y[cur], w.z[cur], s.bmin, s.bmax);
    k_split<<<(G + 127) / 128, 128, 0, st>>>(t, lv, s.bmin, s.bmax, s.sel, no);
    if (lv.multi) {
        cudaMemsetAsync(s.hist, 0, sizeof(uint32_t) * kHistBins * (size_t)G, st);
        cudaMemsetAsync(s.cand_cnt, 0, sizeof(uint32_t) * G, st);
        k_hist<<<grid, kTileThreads, 0, st>>>(t, lv, w.x[cur], w.y[cur], w.z[cur], s.sel,
                                              s.hist);
        k_find<<<G, kTileThreads, 0, st>>>(s.hist, s.sel);
        k_collect<<<grid, kTileThreads, 0, st>>>(t, lv, w.x[cur], w.y[cur], w.z[cur], s.sel,
                                                 s.cand_cnt, s.ckey[0], s.cpos[0]);
    }
    k_select<<<G, kSelThreads, 0, st>>>(t, lv, w.x[cur], w.y[cur], w.z[cur], w.id[cur], s.sel,
                                        s, no);
    k_part_count<<<grid, kTileThreads, 0, st>>>(t, lv, w.x[cur], w.y[cur], w.z[cur], w.id[cur],
                                                s.sel, s.tile_cnt);
    k_tile_scan<<<G, 256, 0, st>>>(t, lv, s.tile_cnt, s.tile_off, s.err);
    k_part_scatter<<<grid, kTileThreads, 0, st>>>(t, lv, w.x[cur], w.y[cur], w.z[cur],
                                                  w.id[cur], w.x[nxt], w.y[nxt], w.z[nxt],
                                                  w.id[nxt], s.sel, s.tile_off);
    return lv.multi ? 9 : 6;
}

// ------------------------------------------------------------------ local subtree finish

struct LocalSmem {
    double x[kLocalMax], y[kLocalMax], z[kLocalMax];
    unsigned long long key[2 * kLocalMax];
    unsigned long long val[2 * kLocalMax];
    uint32_t id[kLocalMax];
    uint32_t tab_st[2][kLocalMax / 2], tab_cn[2][kLocalMax / 2], tab_id[2][kLocalMax / 2];
    uint16_t perm[kLocalMax];
    uint8_t sd[kLocalMax / 2];
    uint32_t G[2], qmax[2];
    uint32_t wcnt[kLocalThreads / 32];
};

__global__ __launch_bounds__(kLocalThreads) void k_local(Topology t, const uint32_t *roots,
                                                         NodeOut no, const double *wx,
                                                         const double *wy, const double *wz,
                                                         const uint32_t *wid,
                                                         const double *mass, dbl4 *tpos,
                                                         uint32_t *tid) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    LocalSmem &S = *reinterpret_cast<LocalSmem *>(smem_raw);
    const uint32_t root = roots[blockIdx.x];
    const uint32_t s0 = t.start[root], c0 = t.count[root];
    const uint32_t leaf = t.leaf;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = kLocalThreads / 32;

    for (uint32_t k = threadIdx.x; k < c0; k += blockDim.x) {
        S.x[k] = wx[s0 + k];
        S.y[k] = wy[s0 + k];
        S.z[k] = wz[s0 + k];
        S.id[k] = wid[s0 + k];
        S.perm[k] = (uint16_t)k;
    }
    int cur = 0;
    if (threadIdx.x == 0) {
        if (c0 > leaf) {
            S.tab_st[0][0] = 0;
            S.tab_cn[0][0] = c0;
            S.tab_id[0][0] = root;
            S.G[0] = 1;
            S.qmax[0] = c0;
        } else {
            S.G[0] = 0;
        }
    }
    __syncthreads();

    while (S.G[cur] > 0) {
        const uint32_t G = S.G[cur];
        // bounding box and split of every internal sub-segment: one warp each
        for (uint32_t i = warp; i < G; i += nwarps) {
            const uint32_t st = S.tab_st[cur][i], cn = S.tab_cn[cur][i];
            double mn[3] = {INFINITY, INFINITY, INFINITY};
            double mx[3] = {-INFINITY, -INFINITY, -INFINITY};
            for (uint32_t k = lane; k < cn; k += 32) {
                uint32_t l = S.perm[st + k];
                double v0 = S.x[l], v1 = S.y[l], v2 = S.z[l];
                mn[0] = fmin(mn[0], v0); mx[0] = fmax(mx[0], v0);
                mn[1] = fmin(mn[1], v1); mx[1] = fmax(mx[1], v1);
                mn[2] = fmin(mn[2], v2); mx[2] = fmax(mx[2], v2);
            }
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                mn[d] = warp_fmin(mn[d]);
                mx[d] = warp_fmax(mx[d]);
            }
            if (lane == 0) {
                uint32_t sd;
                double size;
                choose_split(mn, mx, sd, size);
                S.sd[i] = (uint8_t)sd;
                const uint32_t id = S.tab_id[cur][i];
                no.split_dim[id] = (uint8_t)sd;
                no.size[id] = size;
            }
        }
        __syncthreads();
        const uint32_t P = next_pow2(S.qmax[cur]);
        const uint32_t lgP = 31 - __clz(P);
        const uint32_t total = G * P;
        for (uint32_t q = threadIdx.x; q < total; q += blockDim.x) {
            const uint32_t i = q >> lgP, k = q & (P - 1);
            if (k < S.tab_cn[cur][i]) {
                const uint32_t l = S.perm[S.tab_st[cur][i] + k];
                const uint32_t sd = S.sd[i];
                const double v = sd == 0 ? S.x[l] : (sd == 1 ? S.y[l] : S.z[l]);
                S.key[q] = ord_key(v);
                S.val[q] = ((unsigned long long)S.id[l] << 16) | l;
            } else {
                S.key[q] = ~0ull;
                S.val[q] = ~0ull;
            }
        }
        __syncthreads();
        if (P > 1) bitonic_blocks(S.key, S.val, total, P);
        for (uint32_t q = threadIdx.x; q < total; q += blockDim.x) {
            const uint32_t i = q >> lgP, k = q & (P - 1);
            const uint32_t cn = S.tab_cn[cur][i];
            if (k < cn) {
                const uint32_t l = (uint32_t)(S.val[q] & 0xffffu);
                S.perm[S.tab_st[cur][i] + k] = (uint16_t)l;
                if (k == cn / 2) {
                    const uint32_t sd = S.sd[i];
                    no.split_val[S.tab_id[cur][i]] = sd == 0 ? S.x[l] : (sd == 1 ? S.y[l] : S.z[l]);
                }
            }
        }
        // children that are internal form the next table (order-preserving compaction)
        const int nx = cur ^ 1;
        if (threadIdx.x == 0) { S.G[nx] = 0; S.qmax[nx] = 0; }
        __syncthreads();
        for (uint32_t base = 0; base < 2 * G; base += blockDim.x) {
            const uint32_t u = base + threadIdx.x;
            bool keep = false;
            uint32_t cst = 0, ccn = 0, cid = 0;
            if (u < 2 * G) {
                const uint32_t i = u >> 1;
                const uint32_t st = S.tab_st[cur][i], cn = S.tab_cn[cur][i], id = S.tab_id[cur][i];
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
            uint32_t off = S.G[nx];
            for (int q = 0; q < warp; ++q) off += S.wcnt[q];
            if (keep) {
                const uint32_t o = off + __popc(m & ((1u << lane) - 1u));
                S.tab_st[nx][o] = cst;
                S.tab_cn[nx][o] = ccn;
                S.tab_id[nx][o] = cid;
                atomicMax(&S.qmax[nx], ccn);
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                uint32_t tot = 0;
                for (int q = 0; q < nwarps; ++q) tot += S.wcnt[q];
                S.G[nx] += tot;
            }
            __syncthreads();
        }
        cur = nx;
        __syncthreads();
    }

    for (uint32_t k = threadIdx.x; k < c0; k += blockDim.x) {
        const uint32_t l = S.perm[k];
        const uint32_t id = S.id[l];
        tpos[s0 + k] = make_double4_32a(S.x[l], S.y[l], S.z[l], mass[id]);
        tid[s0 + k] = id;
    }
}

void launch_local(const Topology &t, const uint32_t *roots, uint32_t n_roots,
                  const NodeOut &no, const Work &w, int cur, const double *mass,
                  dbl4 *tpos, uint32_t *tid, cudaStream_t st) {
    static bool attr_set = false;
    const size_t smem = sizeof(LocalSmem);
    if (!attr_set) {
        cudaFuncSetAttribute(k_local, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr_set = true;
    }
    k_local<<<n_roots, kLocalThreads, smem, st>>>(t, roots, no, w.x[cur], w.y[cur], w.z[cur],
                                                  w.id[cur], mass, tpos, tid);
}

}  // namespace kd
