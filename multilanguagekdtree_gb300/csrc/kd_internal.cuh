// kd_internal.cuh -- device data layout and launch wrappers shared by the build, walk and
// API translation units of libkdnbody.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace kd {

// 32-byte aligned (x, y, z, mass) body record in tree order
using dbl4 = double4_32a;

__device__ __forceinline__ dbl4 ldg_dbl4(const dbl4 *p) {
    const double2 *q = reinterpret_cast<const double2 *>(p);
    const double2 a = __ldg(q), b = __ldg(q + 1);
    return make_double4_32a(a.x, a.y, b.x, b.y);
}

// ---------------------------------------------------------------- tuning constants
// Segments of at most kLocalMax bodies finish their whole subtree in one thread block of
// kLocalThreads threads, in shared memory: ~56 KB at 640 bodies, four blocks per SM.
#ifndef KD_LOCAL_MAX
#define KD_LOCAL_MAX 640
#endif
#ifndef KD_LOCAL_THREADS
#define KD_LOCAL_THREADS 256
#endif
constexpr int kLocalMax = KD_LOCAL_MAX;
// The last two multi-block levels (segments of at most four local roots' bodies) run as one
// pass, one block per segment (k_pair).
constexpr uint32_t kPairMax = 4u * (uint32_t)KD_LOCAL_MAX;
constexpr int kLocalThreads = KD_LOCAL_THREADS;
constexpr int kTile = 2048;         // elements per block in the multi-block level passes
constexpr int kTileThreads = 256;
constexpr int kHistBits = 12;       // radix digit of the median select
constexpr int kHistBins = 1 << kHistBits;
constexpr int kSelCap = 2048;       // capacity of the select's shared-memory sort
#ifndef KD_SEL_THREADS
#define KD_SEL_THREADS 512
#endif
constexpr int kSelThreads = KD_SEL_THREADS;
#ifndef KD_MULTI_MIN
#define KD_MULTI_MIN 4096
#endif
constexpr uint32_t kMultiMin = KD_MULTI_MIN;  // segments above this use multi-block histograms
constexpr int kSelMaxIters = 16;    // radix refinement passes before giving up (error)
constexpr int kWalkWarps = 4;       // warps per walk block
constexpr int kStackMax = 32;       // traversal stack entries: one per lane of a warp
constexpr int kMaxHeavy = 8;        // bodies summed directly in FP64 on the mixed path

// device error flags (bit set in ctx->dev_err)
constexpr uint32_t kErrSelect = 1u;   // median select did not converge
constexpr uint32_t kErrStack = 2u;    // traversal stack overflow
constexpr uint32_t kErrNumeric = 4u;  // non-finite or negative input
constexpr uint32_t kErrHeavy = 8u;    // more heavy bodies than kMaxHeavy

// Multiprocessors of the current device (queried once per device): the grid-stride
// kernels size their grids by it.
int sm_count();

// ---------------------------------------------------------------- node records
// Walk record of the FP64 path.  Internal: a = right child (DFS id), b = 0; the left child
// is always id+1.  Leaf: a = first body in tree order, b = body count (>= 1).
struct __align__(16) NodeD {
    double cmx, cmy, cmz, m;
    double size2;
    uint32_t a, b;
    double pad;
};
static_assert(sizeof(NodeD) == 56 || sizeof(NodeD) == 64, "NodeD layout");

// FP32 split of an internal node's FP64 centre of mass and size^2 (hi.w), for the FP64
// walk's FP32 pre-test of the opening decision.
struct __align__(16) NodeP {
    float4 hi, lo;
};

// Walk record of the mixed path: centre of mass as hi+lo floats, size^2, light mass.  The
// opening test reads only `hi` and `a, b`; an accepted node also reads `lo`.  A leaf record
// holds instead its origin o (the position of its first body) as hi+lo floats; the bodies of
// a leaf are stored as FP32 offsets from o.
struct __align__(16) NodeF {
    float4 hi;  // cm hi x,y,z ; size^2
    float4 lo;  // cm lo x,y,z ; light mass
    uint32_t a, b, pad0, pad1;
};

// 1/sqrt(x) for x in [1e-30, 1e30]: the FP32 hardware estimate, then two Newton steps in
// FP64 (quadratic convergence from ~2^-23 to a few ulp).
__device__ __forceinline__ double rsqrt64(double x) {
    float f;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(f) : "f"((float)x));
    const double h = 0.5 * x;
    double y = (double)f;
    y = y * fma(-h * y, y, 1.5);
    y = y * fma(-h * y, y, 1.5);
    return y;
}

// 1/sqrt(x) by rsqrt64 inside its range, else by the rounded square root and division
// (x = 0 gives inf, as the reference's coincident bodies do).
__device__ __forceinline__ double inv_dist(double x) {
    return (x >= 1e-30 && x <= 1e30) ? rsqrt64(x) : __ddiv_rn(1.0, __dsqrt_rn(x));
}

// Per-segment state of the median select at one level of the multi-block build.
struct SegSel {
    uint32_t sd;      // split dimension
    float scale;      // first pass: bin = (float)(v - lo) * scale, clamped to the bin range
    uint32_t digit;   // selected first-pass bin
    uint32_t c;       // candidates left
    uint32_t r;       // rank wanted among the candidates
    uint32_t pad;
    uint64_t kmed;    // median key (order-preserving transform of the coordinate)
    uint32_t idmed;   // median body id (tie break)
    uint32_t posmed;  // position of the median inside the segment
    float lo;         // smallest coordinate along sd, truncated to float
    uint32_t pad2;
};

// ---------------------------------------------------------------- argument blocks
struct Topology {          // static per (n, leaf), DFS ids
    uint32_t n, leaf, n_nodes, n_leaves;
    const uint32_t *start;   // first body (tree order) of every node
    const uint32_t *count;   // bodies of every node
    const uint32_t *right;   // right child of internal nodes
    const uint32_t *parent;  // parent, 0xffffffff at the root
    const uint32_t *leaves;  // DFS ids of the leaves
    const uint32_t *ttab;    // DFS subtree size for 0..kLocalMax bodies
};

struct NodeOut {           // per-node results of the build
    uint8_t *split_dim;
    double *split_val;
    double *size;
};

struct LevelArgs {
    const uint32_t *ids;     // internal nodes of this level
    uint32_t G;              // number of segments
    uint32_t tiles;          // tiles per segment
    bool multi;              // multi-block select
    uint32_t rank;           // rank to select; kMedianRank = len/2 of every segment
    uint32_t *med_pos;       // if set: receives where the selected element was written
    int max_iters = kSelMaxIters;  // radix refinement passes of k_select before it gives up
};
constexpr uint32_t kMedianRank = 0xffffffffu;

__host__ __device__ __forceinline__ uint32_t split_rank(const LevelArgs &lv, uint32_t cnt) {
    return lv.rank == kMedianRank ? cnt / 2 : lv.rank;
}

struct Work {              // ping-pong buffers of the level passes (segment order)
    double *x[2], *y[2], *z[2];
    uint32_t *id[2];
};

struct Scratch {
    unsigned long long *bmin[2], *bmax[2];  // [G*3] ordered keys, ping-pong by level
    SegSel *sel;
    uint32_t *hist;                   // [G*kHistBins]
    uint32_t *cand_cnt;               // [G]
    unsigned long long *ckey[3];      // [n] candidate keys: collected (0), refined (1, 2)
    uint32_t *cpos[3];                // [n] candidate positions
    uint32_t *tile_cnt, *tile_off;    // [G*tiles]
    uint32_t *done;                   // [G] finished histogram blocks per segment (zeroed)
    uint32_t *err;
};

struct Bodies {             // master state, original order
    double *x, *y, *z, *vx, *vy, *vz, *m, *r;
};

// ---------------------------------------------------------------- launchers (kd_build.cu)
struct Moments {
    double *M;                // [n_nodes] mass
    double *S;                // [3*n_nodes] sum of m*p
    uint32_t *counter;        // [n_nodes] arrival counters of the upward pass
};

// What the subtree finish writes besides the tree itself.
struct LocalOut {
    const double *mass;          // master masses, original order
    dbl4 *tpos;                  // bodies in tree order (x, y, z, m)
    uint32_t *tid;               // body index of every tree position
    float4 *thi, *tlo;           // split coordinates (hi.w: light mass), tree order
    float4 *trel;                // offset from the leaf origin, light mass (mixed only)
    Moments mo;                  // full-mass moments (FP64 records)
    Moments mof;                 // light-mass moments (mixed records)
    NodeD *recd;                 // FP64 walk records, or nullptr
    NodeP *recp;                 // FP32 pre-test data of the FP64 records (with recd)
    NodeF *recf;                 // mixed walk records, or nullptr
    const uint32_t *heavy;       // bodies left out of the FP32 masses
    int n_heavy;
};

__device__ __forceinline__ bool is_heavy(uint32_t id, const uint32_t *heavy_ids, int n_heavy) {
    bool h = false;
    for (int i = 0; i < n_heavy; ++i) h |= heavy_ids[i] == id;
    return h;
}

// FP64 record: cm = S * (1/m) (the reference divides, array_kd_tree.rs:548-550; its sums
// already differ from ours in order, so one more rounding stays within the moment bound),
// size*size in the reference's IEEE order (:606).
__device__ __forceinline__ NodeD make_noded(double m, double sx, double sy, double sz,
                                            double size, uint32_t a, uint32_t b) {
    NodeD q;
    const double inv = __ddiv_rn(1.0, m);
    q.cmx = __dmul_rn(sx, inv);
    q.cmy = __dmul_rn(sy, inv);
    q.cmz = __dmul_rn(sz, inv);
    q.m = m;
    q.size2 = __dmul_rn(size, size);
    q.a = a;
    q.b = b;
    q.pad = 0.0;
    return q;
}

// Mixed record: cm as hi + lo floats.  A massless node gets a NaN cm and is never accepted.
__device__ __forceinline__ NodeF make_nodef(double m, double sx, double sy, double sz,
                                            double size, uint32_t a, uint32_t b) {
    NodeF r;
    const double inv = 1.0 / m;
    const double cx = sx * inv, cy = sy * inv, cz = sz * inv;
    const float hx = (float)cx, hy = (float)cy, hz = (float)cz;
    r.hi = make_float4(hx, hy, hz, (float)(size * size));
    r.lo = make_float4((float)(cx - (double)hx), (float)(cy - (double)hy),
                       (float)(cz - (double)hz), (float)m);
    r.a = a;
    r.b = b;
    r.pad0 = r.pad1 = 0u;
    return r;
}

__device__ __forceinline__ NodeP make_nodep(const NodeD &q) {
    NodeP p;
    const float hx = (float)q.cmx, hy = (float)q.cmy, hz = (float)q.cmz;
    p.hi = make_float4(hx, hy, hz, (float)q.size2);
    p.lo = make_float4((float)(q.cmx - (double)hx), (float)(q.cmy - (double)hy),
                       (float)(q.cmz - (double)hz), 0.0f);
    return p;
}

// Work arrays of the build (unless !copy: a level 0 that reads the bodies in place); with
// bmin/bmax set, also the level-0 bounding box into them.
void launch_init_work(const Bodies &b, Work &w, uint32_t n, unsigned long long *bmin,
                      unsigned long long *bmax, cudaStream_t st, bool copy = true);
// quickselect set-up: key[i] = vals[idx[i]], id[i] = idx[i]; flags an index >= n_vals
void launch_gather_keys(const double *vals, uint64_t n_vals, const uint64_t *idx, uint32_t n,
                        double *key, uint32_t *id, uint32_t *err, cudaStream_t st);
// puts the selected element at position `goal` (it was written at *med_pos)
void launch_place_selected(uint32_t *id, const uint32_t *med_pos, uint32_t goal, cudaStream_t st);
// One multi-block level.  `lvl` selects the bounding-box buffers (lvl & 1); the boxes of
// level 0 are computed here unless `box0_ready` (launch_init_work made them), deeper levels
// receive theirs from the previous level's scatter (`G_next` > 0 when the next level is a
// multi-block level too).  `seg_max`: the level's largest segment (small segments take a
// warp each for split and median).  Returns the number of kernels launched.
int launch_level(const Topology &t, const LevelArgs &lv, const NodeOut &no, Work &w, int cur,
                 Scratch &s, int lvl, uint32_t G_next, cudaStream_t st, bool box0_ready = false,
                 uint32_t seg_max = 0xffffffffu);
// The last one or two levels above the local roots in one pass: the segments `ids` (G of
// them, at most `cap` <= kPairMax bodies each, boxes in bmin/bmax) and, with `ids2` set, their
// children (ids2[2g], ids2[2g+1]) are split, and the bodies go from work buffer `cur` to the
// other in the order of the local roots.  A select needing more than max_rounds radix
// passes fails (kErrSelect).  Returns the number of kernels launched.
int launch_pair(const Topology &t, const uint32_t *ids, const uint32_t *ids2, uint32_t G,
                uint32_t cap, const unsigned long long *bmin, const unsigned long long *bmax,
                const NodeOut &no, Work &w, int cur, int max_rounds, uint32_t *err,
                cudaStream_t st);
// Subtree finish of every local root (each of at most kLocalMax bodies): split decisions,
// tree order, and the moments and walk records of all nodes below the local roots.
void launch_local(const Topology &t, const uint32_t *roots, uint32_t n_roots,
                  const NodeOut &no, const Work &w, int cur, const LocalOut &out,
                  uint32_t *err, cudaStream_t st);
// Moments and records of the nodes above the local roots (one thread per local root climbs).
void launch_moments_top(const Topology &t, const uint32_t *roots, uint32_t n_roots,
                        const NodeOut &no, const LocalOut &out, cudaStream_t st);

// ---------------------------------------------------------------- launchers (kd_walk.cu)
// stack_cap: traversal stack entries (at most kStackMax) before the walk reports kErrStack.
void launch_walk_fp64(const NodeD *rec, const NodeP *recp, const float4 *thi,
                      const float4 *tlo, const dbl4 *tpos, const uint32_t *tid, uint32_t n,
                      double theta, double *acc, uint32_t *err,
                      unsigned long long *counts, cudaStream_t st,
                      uint32_t stack_cap = kStackMax);
// Grouped mixed walk: groups of whole leaves, <= kGroupSinks bodies (two per lane of a warp),
// gstart[g]..gstart[g+1] in tree order, boxed in two parts split at gsplit[g]; stk_cap =
// per-warp stack entries (a multiple of 32).
constexpr int kGroupSinks = 64;
constexpr int kGroupWarps = 2;  // groups (warps) per block: a finished warp's block frees
                                // its SM slot sooner than with 4 or 8
#ifndef KD_GROUP_FLUSH
#define KD_GROUP_FLUSH 128
#endif
constexpr int kGroupFlush = KD_GROUP_FLUSH;  // list entries that trigger a sum
constexpr int kGroupListCap = kGroupFlush + 32 * 8;
// shared memory of one warp: interaction list, own-leaf list (two float4 per body: split
// positions), stack
__host__ __device__ inline uint32_t group_warp_bytes(uint32_t stk_cap) {
    return (uint32_t)((kGroupListCap + 2 * kGroupSinks) * sizeof(float4) +
                      stk_cap * sizeof(uint32_t));
}
// Thread blocks of the grouped walk (kGroupWarps groups each).
__host__ __device__ inline uint32_t walk_group_blocks(uint32_t n_groups) {
    return (n_groups + kGroupWarps - 1) / kGroupWarps;
}
// The walk, then (n_heavy > 0) the heavy bodies' own accelerations as FP64 direct sums over
// all bodies: every group's warp leaves its partial sums in hpart and k_heavy_finish adds
// them in a fixed order (hpart: heavy_partial_doubles(n_groups); hcount: kMaxHeavy zeroed
// words).  With phi set, also the potentials.  Returns the number of kernels launched.
constexpr int kFinishBlocks = 64;
constexpr int kFinishThreads = 256;
__host__ __device__ inline size_t heavy_partial_doubles(uint32_t n_groups) {
    return (size_t)kMaxHeavy * 4 * ((size_t)n_groups + kFinishBlocks);
}
int launch_walk_group(const NodeF *rec, const float4 *thi, const float4 *tlo,
                      const float4 *trel, const uint32_t *tid, const uint32_t *gstart,
                      const uint32_t *gsplit, uint32_t n_groups, uint32_t stk_cap, double theta,
                      const Bodies &b, const uint32_t *heavy_ids, int n_heavy, double *acc,
                      double *hpart, uint32_t *hcount, uint32_t *err,
                      unsigned long long *counts, cudaStream_t st, double *phi = nullptr);

// per-block sums (kinetic, potential) of 0.5 m v^2 and 0.5 m phi into part[2*blocks]
void launch_energy_partial(const Bodies &b, const double *phi, uint32_t n, double *part,
                           int blocks, cudaStream_t st);
// No update once the device error word is set (the state stays at the failed step's start).
void launch_kick_drift(Bodies &b, double *acc, uint32_t n, double dt, const uint32_t *err,
                       cudaStream_t st);
void launch_aos_to_soa(const void *aos, Bodies &b, uint32_t n, uint32_t *err, cudaStream_t st);
void launch_soa_to_aos(const Bodies &b, void *aos, uint32_t n, cudaStream_t st);
// The same conversions reading or writing pinned host records directly (a device-accessible
// address of page-locked host memory), at the host link's rate, with no device staging copy.
void launch_host_to_soa(const void *host, Bodies &b, uint32_t n, uint32_t *err, cudaStream_t st);
void launch_soa_to_host(const Bodies &b, void *host, uint32_t n, cudaStream_t st);
// FP64 direct sum for ns sinks; `partial` holds ns * ceil(n / kDirectChunk) * 3 doubles
constexpr uint32_t kDirectChunk = 1u << 18;
constexpr int kDirectThreads = 128;
void launch_direct(const Bodies &b, uint32_t n, const uint64_t *sinks, uint32_t ns,
                   double *partial, double *acc, cudaStream_t st);
// Heavy bodies (m >= frac * total mass, at most kMaxHeavy listed); scratch_total holds the
// total mass followed by 304 per-block partial sums.
void launch_find_heavy(const Bodies &b, uint32_t n, double frac, double *scratch_total,
                       uint32_t *heavy_ids, uint32_t *n_heavy, uint32_t *err, cudaStream_t st);

// ---------------------------------------------------------------- generators (kd_generate.cu)
// kind 0 ring, 1 Plummer, 2 circular_orbits; `scratch` holds 6*256 doubles.  Returns the
// number of kernels launched, or -1 for an unknown kind.
int launch_generate(int kind, Bodies &b, uint32_t n, uint64_t seed, double *scratch,
                    cudaStream_t st);

// ---------------------------------------------------------------- adjoint (kd_adjoint.cu)
struct AdjArgs {
    Topology topo;
    const NodeF *recf;
    const float4 *thi, *tlo, *trel;
    const uint32_t *tid;
    uint32_t n;
    double theta, dt;
    Bodies bodies;
    const uint32_t *heavy;
    int n_heavy;
    double *lx, *lv;        // adjoints of x and v, original order, 3n
    double *mu, *y;         // 3n scratch
    double *ysink;          // 3n, tree order
    double *yheavy;         // 3 * kMaxHeavy: the heavy bodies' source sums
    double *hpart;          // heavy_partial_doubles(n_groups): per-group parts of yheavy
    uint32_t *hcount;       // kMaxHeavy zeroed words (k_heavy_finish)
    double *U;              // 3n, tree order: pair-source sums
    double *G;              // 3 * n_nodes: node-source sums
    uint32_t *err;
    const uint32_t *gstart, *gsplit;  // sink groups of the grouped walk
    uint32_t n_groups, stk_cap;
};
// The transpose-Jacobian walk over the grouped interaction set (kd_group.cu).
void launch_adj_group(const AdjArgs &a, cudaStream_t st);
// One backward step over the tree currently built (mixed records).  Returns kernels launched.
int launch_adjoint_step(const AdjArgs &a, cudaStream_t st);

}  // namespace kd
