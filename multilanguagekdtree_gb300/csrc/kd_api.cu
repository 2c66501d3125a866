// kd_api.cu -- host runtime behind include/kdnbody.h: the per-n tree plan, device memory of
// a context, the step sequence and the C entry points.
//
// The reference's step (MarkCLewis/MultiLanguageKDTree Parallel/RustVersion/src/
// array_kd_tree.rs:623-664 simple_sim) is: reset the index vector, build the tree, compute
// every body's acceleration, kick-drift.  Here the same step is a fixed sequence of kernel
// launches on the context's stream; the bodies stay on the device between calls.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <charconv>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/kdnbody.h"
#include "kd_internal.cuh"

using namespace kd;

namespace {

thread_local std::string g_create_error;

constexpr uint32_t kNone = 0xffffffffu;

// nodes_needed_for_particles of Parallel/RustVersion/src/array_kd_tree.rs:45-53; the
// power of two 2^ceil(log2 x) is the smallest one >= x (equal for every x < 2^52).
uint64_t needed_par(uint64_t n, uint32_t leaf) {
    if (n <= leaf) return 1;
    const uint64_t min_leaves = n / (leaf / 2);
    uint64_t leaves = 1;
    while (leaves < min_leaves) leaves <<= 1;
    return 2 * leaves - 1;
}

// Sequential/RustVersion/src/array_kd_tree.rs:37-39
uint64_t needed_seq(uint64_t n, uint32_t leaf) { return 2 * (n / (leaf / 2) + 1); }

// The tree of n bodies: shape, segment of every node, DFS and PAR4 numbering, level lists.
struct Plan {
    uint32_t n = 0, leaf = 0, n_nodes = 0;
    std::vector<uint32_t> start, count, right, parent, leaves;
    std::vector<uint64_t> par4;           // PAR4 slot of every DFS node
    std::vector<std::vector<uint32_t>> glevels;  // internal nodes of the multi-block levels
    std::vector<uint32_t> gmax;           // largest segment per multi-block level
    std::vector<uint32_t> local_roots;
    std::vector<uint32_t> ttab;
    uint64_t par4_slots = 0, par4_last = 0;
    bool par4_ok = true;
    uint32_t depth = 0;                   // deepest node (root = 0)
    std::vector<uint32_t> gstart;         // sink groups of the grouped walk (tree positions)
    std::vector<uint32_t> gsplit;         // per group: split of the deepest node holding it
};

struct Memo {
    uint32_t leaf;
    std::unordered_map<uint64_t, uint64_t> t;
    uint64_t T(uint64_t nb) {
        if (nb <= leaf) return 1;
        auto it = t.find(nb);
        if (it != t.end()) return it->second;
        uint64_t v = 1 + T(nb / 2) + T(nb - nb / 2);
        t.emplace(nb, v);
        return v;
    }
};

bool make_plan(uint32_t n, uint32_t leaf, Plan &p, std::string &err) {
    p.n = n;
    p.leaf = leaf;
    Memo memo{leaf, {}};
    const uint64_t total = memo.T(n);
    if (total >= 0xffffffffull) {
        err = "too many nodes";
        return false;
    }
    p.n_nodes = (uint32_t)total;
    p.start.assign(p.n_nodes, 0);
    p.count.assign(p.n_nodes, 0);
    p.right.assign(p.n_nodes, 0);
    p.parent.assign(p.n_nodes, kNone);
    p.par4.assign(p.n_nodes, 0);
    p.par4_slots = needed_par(n, leaf);
    p.ttab.resize(kLocalMax + 1);
    for (uint32_t i = 0; i <= (uint32_t)kLocalMax; ++i) p.ttab[i] = (uint32_t)memo.T(i);

    struct E {
        uint32_t id, st, cn, parent;
        uint64_t par4, cap4;
    };
    std::vector<E> cur{{0u, 0u, n, kNone, 0ull, p.par4_slots}}, nxt;
    bool local_found = false;
    uint32_t level = 0;
    while (!cur.empty()) {
        p.depth = level++;
        uint32_t mx = 0;
        for (const E &e : cur) mx = std::max(mx, e.cn);
        if (!local_found && mx <= (uint32_t)kLocalMax) {
            local_found = true;
            for (const E &e : cur) p.local_roots.push_back(e.id);
        }
        std::vector<uint32_t> internal;
        nxt.clear();
        for (const E &e : cur) {
            p.start[e.id] = e.st;
            p.count[e.id] = e.cn;
            p.parent[e.id] = e.parent;
            p.par4[e.id] = e.par4;
            p.par4_last = std::max(p.par4_last, e.par4);
            if (e.cap4 < 1) p.par4_ok = false;
            if (e.cn > leaf) {
                internal.push_back(e.id);
                const uint32_t lc = e.cn / 2, rc = e.cn - lc;
                const uint32_t lid = e.id + 1;
                const uint32_t rid = e.id + 1 + (uint32_t)memo.T(lc);
                p.right[e.id] = rid;
                const uint64_t lcap = needed_par(lc, leaf);
                // build_tree_par4 splits its slice as [this | left: lcap | right: rest]
                if (1 + lcap > e.cap4) p.par4_ok = false;
                const uint64_t rcap = e.cap4 > 1 + lcap ? e.cap4 - 1 - lcap : 0;
                nxt.push_back({lid, e.st, lc, e.id, e.par4 + 1, lcap});
                nxt.push_back({rid, e.st + lc, rc, e.id, e.par4 + 1 + lcap, rcap});
            } else {
                p.leaves.push_back(e.id);
            }
        }
        if (!local_found) {
            p.glevels.push_back(internal);
            p.gmax.push_back(mx);
        }
        cur.swap(nxt);
    }
    // Sink groups: whole leaves in tree order, packed greedily up to kGroupSinks bodies.
    std::vector<std::pair<uint32_t, uint32_t>> lv;
    lv.reserve(p.leaves.size());
    for (uint32_t id : p.leaves) lv.emplace_back(p.start[id], p.count[id]);
    std::sort(lv.begin(), lv.end());
    p.gstart.clear();
    uint32_t fill = kGroupSinks;
    for (const auto &e : lv) {
        if (fill + e.second > (uint32_t)kGroupSinks) {
            p.gstart.push_back(e.first);
            fill = 0;
        }
        fill += e.second;
    }
    p.gstart.push_back(n);
    // The split position of the deepest node that holds a group whole (a node of c bodies
    // at position st splits at st + c/2); a one-leaf group has none (its end).
    p.gsplit.resize(p.gstart.size() - 1);
    for (size_t g = 0; g + 1 < p.gstart.size(); ++g) {
        const uint32_t g0 = p.gstart[g], g1 = p.gstart[g + 1];
        uint32_t st = 0, cn = n, sp = g1;
        while (cn > leaf) {
            const uint32_t mid = st + cn / 2;
            if (g1 <= mid) {
                cn = cn / 2;
            } else if (g0 >= mid) {
                st = mid;
                cn = cn - cn / 2;
            } else {
                sp = mid;
                break;
            }
        }
        p.gsplit[g] = sp;
    }
    return true;
}

template <typename T>
cudaError_t dalloc(T **ptr, size_t count) {
    *ptr = nullptr;
    if (count == 0) count = 1;
    return cudaMalloc((void **)ptr, sizeof(T) * count);
}

}  // namespace

struct kd_ctx {
    size_t n = 0;
    kd_params prm{};
    cudaStream_t st = nullptr;
    std::string err;
    Plan plan;

    // static topology on the device
    uint32_t *d_start = nullptr, *d_count = nullptr, *d_right = nullptr, *d_parent = nullptr,
             *d_leaves = nullptr, *d_ttab = nullptr, *d_local_roots = nullptr,
             *d_gstart = nullptr, *d_gsplit = nullptr;
    uint32_t n_groups = 0, group_stack = 0;
    // device-side limits (kd_set_device_limits): 0 = the defaults
    uint32_t stack_limit = 0;
    int select_passes = kSelMaxIters;
    uint32_t walk_stack() const {  // stack entries of the grouped walk (and its adjoint)
        return stack_limit && stack_limit < group_stack ? stack_limit : group_stack;
    }
    std::vector<uint32_t *> d_glevels;
    Topology topo{};

    Bodies bodies{};
    double *acc = nullptr;
    void *aos = nullptr;  // staging for host transfers
    Work work{};
    Scratch scr{};
    NodeOut nout{};
    Moments mom{}, momf{};  // FP64 and light (mixed) moments
    NodeD *recd = nullptr;
    NodeP *recp = nullptr;
    NodeF *recf = nullptr;
    dbl4 *tpos = nullptr;
    uint32_t *tid = nullptr;
    float4 *thi = nullptr, *tlo = nullptr, *trel = nullptr;
    uint32_t *dev_err = nullptr;
    unsigned long long *d_counts = nullptr;
    uint32_t *d_heavy = nullptr, *d_nheavy = nullptr;
    double *d_total = nullptr;
    double *d_hpart = nullptr;   // per-group partial direct sums of the heavy bodies
    uint32_t *d_hcount = nullptr;  // finished blocks of k_heavy_finish per heavy body
    double *gen_scratch = nullptr;
    double *phi = nullptr;  // potentials, allocated by the first kd_energy
    int n_heavy = 0;
    std::vector<uint32_t> heavy;
    int final_buf = 0;

    bool has_bodies = false, has_tree = false, tree_fp64 = false, tree_mixed = false;
    bool counting = false, timing = false;
    uint64_t counts[4] = {0, 0, 0, 0};
    uint64_t launches = 0;              // kernels enqueued since the last reset
    std::vector<cudaEvent_t> tev;       // per-step phase events (timing mode)
    kd_stats stats{};
    cudaEvent_t ev[6] = {};

    std::vector<void *> owned;

    // one step (build, walk, kick) as a CUDA graph: captured on first use, relaunched
    cudaGraphExec_t graph = nullptr;
    double graph_dt = 0.0;
    int graph_prec = -1, graph_heavy = -1;
    uint64_t graph_launches = 0;
    bool graph_off = false;  // capture failed once: launch directly from then on
    // one backward step (rebuild + transpose-Jacobian step) as a CUDA graph
    cudaGraphExec_t adj_graph = nullptr;
    double adj_graph_dt = 0.0;
    int adj_graph_heavy = -1;
    uint64_t adj_graph_launches = 0;

    // adjoint state, allocated by the first kd_forward
    bool adj_ready = false;
    int64_t adj_every = 0;
    double *lx = nullptr, *lv = nullptr, *amu = nullptr, *ay = nullptr, *ysink = nullptr,
           *yheavy = nullptr, *segbuf = nullptr;
    // segbuf holds the positions of the last checkpoint segment of tape seg_owner (as the
    // forward sweep left them), or nothing (0)
    uint64_t tapes = 0, seg_owner = 0;
    double *aU = nullptr, *aG = nullptr;
    // state buffers (6n doubles) of checkpoints, kept by the context and reused by later
    // forward sweeps once their tape is freed: no cudaMalloc (and its device-wide
    // synchronisation) in front of every sweep
    std::vector<double *> ck_free;

    int fail(int code, const char *fmt, ...) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        err = buf;
        return code;
    }
    int cuda_fail(cudaError_t e, const char *what) {
        return fail(e == cudaErrorMemoryAllocation ? KD_ENOMEM : KD_ECUDA, "%s: %s", what,
                    cudaGetErrorString(e));
    }
    template <typename T>
    cudaError_t alloc(T **p, size_t count) {
        cudaError_t e = dalloc(p, count);
        if (e == cudaSuccess) owned.push_back((void *)*p);
        return e;
    }
};

namespace {

#define KD_CHECK(ctx, expr)                                      \
    do {                                                         \
        cudaError_t e_ = (expr);                                 \
        if (e_ != cudaSuccess) return (ctx)->cuda_fail(e_, #expr); \
    } while (0)

int upload(kd_ctx *c, uint32_t **dst, const std::vector<uint32_t> &src) {
    KD_CHECK(c, c->alloc(dst, src.size()));
    if (!src.empty())
        KD_CHECK(c, cudaMemcpy(*dst, src.data(), src.size() * sizeof(uint32_t),
                               cudaMemcpyHostToDevice));
    return KD_OK;
}

int setup(kd_ctx *c) {
    const size_t n = c->n;
    Plan &p = c->plan;
    KD_CHECK(c, cudaSetDevice(c->prm.device));
    KD_CHECK(c, cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking));
    for (auto &e : c->ev) KD_CHECK(c, cudaEventCreate(&e));
    int rc;
    if ((rc = upload(c, &c->d_start, p.start))) return rc;
    if ((rc = upload(c, &c->d_count, p.count))) return rc;
    if ((rc = upload(c, &c->d_right, p.right))) return rc;
    if ((rc = upload(c, &c->d_parent, p.parent))) return rc;
    if ((rc = upload(c, &c->d_leaves, p.leaves))) return rc;
    if ((rc = upload(c, &c->d_ttab, p.ttab))) return rc;
    if ((rc = upload(c, &c->d_local_roots, p.local_roots))) return rc;
    if ((rc = upload(c, &c->d_gstart, p.gstart))) return rc;
    if ((rc = upload(c, &c->d_gsplit, p.gsplit))) return rc;
    c->n_groups = (uint32_t)p.gstart.size() - 1;
    // a wave pops <= 32 entries and pushes <= 64: at most 32 wait per depth, plus one push
    c->group_stack = 32u * (p.depth + 2u) + 64u;
    c->d_glevels.resize(p.glevels.size());
    size_t maxG = 1, maxGT = 1, maxGmulti = 1;
    for (size_t l = 0; l < p.glevels.size(); ++l) {
        if ((rc = upload(c, &c->d_glevels[l], p.glevels[l]))) return rc;
        const size_t G = p.glevels[l].size();
        const size_t tiles = (p.gmax[l] + kTile - 1) / kTile;
        maxG = std::max(maxG, G);
        maxGT = std::max(maxGT, G * tiles);
        if (p.gmax[l] > kMultiMin) maxGmulti = std::max(maxGmulti, G);
    }
    Topology &t = c->topo;
    t.n = (uint32_t)n;
    t.leaf = p.leaf;
    t.n_nodes = p.n_nodes;
    t.n_leaves = (uint32_t)p.leaves.size();
    t.start = c->d_start;
    t.count = c->d_count;
    t.right = c->d_right;
    t.parent = c->d_parent;
    t.leaves = c->d_leaves;
    t.ttab = c->d_ttab;

    Bodies &b = c->bodies;
    KD_CHECK(c, c->alloc(&b.x, n));
    KD_CHECK(c, c->alloc(&b.y, n));
    KD_CHECK(c, c->alloc(&b.z, n));
    KD_CHECK(c, c->alloc(&b.vx, n));
    KD_CHECK(c, c->alloc(&b.vy, n));
    KD_CHECK(c, c->alloc(&b.vz, n));
    KD_CHECK(c, c->alloc(&b.m, n));
    KD_CHECK(c, c->alloc(&b.r, n));
    KD_CHECK(c, c->alloc(&c->acc, 3 * n));
    KD_CHECK(c, c->alloc((double **)&c->aos, 8 * n));
    for (int k = 0; k < 2; ++k) {
        KD_CHECK(c, c->alloc(&c->work.x[k], n));
        KD_CHECK(c, c->alloc(&c->work.y[k], n));
        KD_CHECK(c, c->alloc(&c->work.z[k], n));
        KD_CHECK(c, c->alloc(&c->work.id[k], n));
    }
    for (int k = 0; k < 3; ++k) {
        KD_CHECK(c, c->alloc(&c->scr.ckey[k], n));
        KD_CHECK(c, c->alloc(&c->scr.cpos[k], n));
    }
    for (int k = 0; k < 2; ++k) {
        KD_CHECK(c, c->alloc(&c->scr.bmin[k], 3 * maxG));
        KD_CHECK(c, c->alloc(&c->scr.bmax[k], 3 * maxG));
    }
    KD_CHECK(c, c->alloc(&c->scr.sel, maxG));
    KD_CHECK(c, c->alloc(&c->scr.hist, (size_t)kHistBins * maxGmulti));
    KD_CHECK(c, c->alloc(&c->scr.cand_cnt, maxG));
    KD_CHECK(c, c->alloc(&c->scr.tile_cnt, maxGT));
    KD_CHECK(c, c->alloc(&c->scr.tile_off, maxGT));
    KD_CHECK(c, c->alloc(&c->scr.done, maxGmulti));
    KD_CHECK(c, cudaMemset(c->scr.done, 0, maxGmulti * sizeof(uint32_t)));
    KD_CHECK(c, c->alloc(&c->dev_err, 1));
    c->scr.err = c->dev_err;
    const size_t nn = p.n_nodes;
    KD_CHECK(c, c->alloc(&c->nout.split_dim, nn));
    KD_CHECK(c, c->alloc(&c->nout.split_val, nn));
    KD_CHECK(c, c->alloc(&c->nout.size, nn));
    KD_CHECK(c, c->alloc(&c->mom.M, nn));
    KD_CHECK(c, c->alloc(&c->mom.S, 3 * nn));
    KD_CHECK(c, c->alloc(&c->mom.counter, nn));
    KD_CHECK(c, c->alloc(&c->momf.M, nn));
    KD_CHECK(c, c->alloc(&c->momf.S, 3 * nn));
    c->momf.counter = c->mom.counter;
    KD_CHECK(c, c->alloc(&c->recd, nn));
    KD_CHECK(c, c->alloc(&c->recp, nn));
    KD_CHECK(c, c->alloc(&c->recf, nn));
    KD_CHECK(c, c->alloc(&c->tpos, n));
    KD_CHECK(c, c->alloc(&c->tid, n));
    KD_CHECK(c, c->alloc(&c->thi, n));
    KD_CHECK(c, c->alloc(&c->tlo, n));
    KD_CHECK(c, c->alloc(&c->trel, n));
    KD_CHECK(c, c->alloc(&c->d_counts, 4));
    KD_CHECK(c, c->alloc(&c->d_heavy, kMaxHeavy));
    KD_CHECK(c, c->alloc(&c->d_nheavy, 1));
    KD_CHECK(c, c->alloc(&c->d_total, 1 + 304));  // total mass + per-block partials
    KD_CHECK(c, c->alloc(&c->d_hpart, heavy_partial_doubles(c->n_groups)));
    KD_CHECK(c, c->alloc(&c->d_hcount, kMaxHeavy));
    KD_CHECK(c, cudaMemset(c->d_hcount, 0, kMaxHeavy * sizeof(uint32_t)));
    KD_CHECK(c, c->alloc(&c->gen_scratch, 6 * 256));
    KD_CHECK(c, cudaMemset(c->dev_err, 0, sizeof(uint32_t)));
    // the build's ping-pong buffers start as valid bodies (id 0 at the origin), so a slot a
    // failed select leaves unwritten never holds an out-of-range id
    for (int k = 0; k < 2; ++k) {
        KD_CHECK(c, cudaMemset(c->work.x[k], 0, n * sizeof(double)));
        KD_CHECK(c, cudaMemset(c->work.y[k], 0, n * sizeof(double)));
        KD_CHECK(c, cudaMemset(c->work.z[k], 0, n * sizeof(double)));
        KD_CHECK(c, cudaMemset(c->work.id[k], 0, n * sizeof(uint32_t)));
    }
    KD_CHECK(c, cudaMemset(c->nout.split_dim, 0, nn));
    KD_CHECK(c, cudaMemset(c->nout.split_val, 0, nn * sizeof(double)));
    KD_CHECK(c, cudaMemset(c->nout.size, 0, nn * sizeof(double)));
    return KD_OK;
}

// Read and clear the device error word; translate it.
int check_device(kd_ctx *c) {
    uint32_t e = 0;
    KD_CHECK(c, cudaMemcpyAsync(&e, c->dev_err, sizeof e, cudaMemcpyDeviceToHost, c->st));
    KD_CHECK(c, cudaStreamSynchronize(c->st));
    if (e) {
        KD_CHECK(c, cudaMemsetAsync(c->dev_err, 0, sizeof(uint32_t), c->st));
        if (e & kErrNumeric)
            return c->fail(KD_ENUMERIC, "non-finite position/velocity/mass or negative mass");
        if (e & kErrStack) return c->fail(KD_EDEVICE, "traversal stack overflow");
        if (e & kErrSelect) return c->fail(KD_EDEVICE, "median select failed to converge");
        return c->fail(KD_EDEVICE, "device check failed (0x%x)", e);
    }
    return KD_OK;
}

// Build: multi-block levels, then the shared-memory subtree finish, which also produces the
// moments and walk records below the local roots; then the nodes above them.  Leaves the
// bodies in tree order in tid, thi and tlo (and tpos when FP64 records are wanted).
void enqueue_build(kd_ctx *c, bool want_d, bool want_f) {
    Plan &p = c->plan;
    const bool levels = !p.glevels.empty();
    // the last two levels (one when the root is the only multi-block segment) in one pass
    const size_t L = p.glevels.size();
    const size_t npair = L >= 2 && p.gmax[L - 2] <= kPairMax
                             ? 2
                             : (L >= 1 && p.gmax[L - 1] <= kPairMax ? 1 : 0);
    // a multi-block level 0 reads the bodies' positions in place (original order: the body id
    // is the position), so the first pass only reduces the root's bounding box
    const bool direct0 = L > npair && p.gmax[0] > kMultiMin;
    Work w0 = c->work;
    if (direct0) {
        w0.x[0] = c->bodies.x;
        w0.y[0] = c->bodies.y;
        w0.z[0] = c->bodies.z;
        w0.id[0] = nullptr;
    }
    launch_init_work(c->bodies, c->work, (uint32_t)c->n, levels ? c->scr.bmin[0] : nullptr,
                     levels ? c->scr.bmax[0] : nullptr, c->st, !direct0);
    c->launches += 3;  // init + local finish + upward pass
    int cur = 0;
    for (size_t l = 0; l + npair < L; ++l) {
        LevelArgs lv;
        lv.ids = c->d_glevels[l];
        lv.G = (uint32_t)p.glevels[l].size();
        lv.tiles = (p.gmax[l] + kTile - 1) / kTile;
        lv.multi = p.gmax[l] > kMultiMin;
        lv.rank = kMedianRank;
        lv.med_pos = nullptr;
        lv.max_iters = c->select_passes;
        const uint32_t G_next = l + 1 < p.glevels.size() ? (uint32_t)p.glevels[l + 1].size() : 0u;
        c->launches += launch_level(c->topo, lv, c->nout, l == 0 ? w0 : c->work, cur, c->scr,
                                    (int)l, G_next, c->st, true, p.gmax[l]);
        cur ^= 1;
    }
    if (npair) {
        const size_t l0 = L - npair;
        c->launches += launch_pair(c->topo, c->d_glevels[l0],
                                   npair == 2 ? c->d_glevels[l0 + 1] : nullptr,
                                   (uint32_t)p.glevels[l0].size(), p.gmax[l0],
                                   c->scr.bmin[l0 & 1], c->scr.bmax[l0 & 1], c->nout, c->work,
                                   cur, c->select_passes, c->scr.err, c->st);
        cur ^= 1;
    }
    LocalOut o;
    o.mass = c->bodies.m;
    o.tpos = want_d ? c->tpos : nullptr;  // FP64 positions: read by the FP64 walk only
    o.tid = c->tid;
    o.thi = c->thi;
    o.tlo = c->tlo;
    o.trel = c->trel;
    o.mo = c->mom;
    o.mof = c->momf;
    o.recd = want_d ? c->recd : nullptr;
    o.recp = c->recp;
    o.recf = want_f ? c->recf : nullptr;
    o.heavy = c->d_heavy;
    o.n_heavy = c->n_heavy;
    const uint32_t nr = (uint32_t)p.local_roots.size();
    launch_local(c->topo, c->d_local_roots, nr, c->nout, c->work, cur, o,
                 c->dev_err, c->st);
    launch_moments_top(c->topo, c->d_local_roots, nr, c->nout, o, c->st);
    c->final_buf = cur;
}

void enqueue_walk(kd_ctx *c) {
    unsigned long long *cnt = c->counting ? c->d_counts : nullptr;
    if (c->prm.precision == KD_PREC_MIXED) {
        c->launches += launch_walk_group(c->recf, c->thi, c->tlo, c->trel, c->tid, c->d_gstart,
                                         c->d_gsplit, c->n_groups, c->walk_stack(),
                                         c->prm.theta, c->bodies, c->d_heavy, c->n_heavy,
                                         c->acc, c->d_hpart, c->d_hcount, c->dev_err, cnt,
                                         c->st);
    } else {
        c->launches += 1;
        launch_walk_fp64(c->recd, c->recp, c->thi, c->tlo, c->tpos, c->tid, (uint32_t)c->n,
                         c->prm.theta, c->acc, c->dev_err, cnt, c->st,
                         c->stack_limit ? c->stack_limit : (uint32_t)kStackMax);
    }
}

int fetch_counts(kd_ctx *c) {
    if (!c->counting) return KD_OK;
    unsigned long long h[4];
    KD_CHECK(c, cudaMemcpyAsync(h, c->d_counts, sizeof h, cudaMemcpyDeviceToHost, c->st));
    KD_CHECK(c, cudaStreamSynchronize(c->st));
    for (int i = 0; i < 4; ++i) c->counts[i] = h[i];
    return KD_OK;
}

int reset_counts(kd_ctx *c) {
    if (c->counting) KD_CHECK(c, cudaMemsetAsync(c->d_counts, 0, 4 * sizeof(unsigned long long), c->st));
    return KD_OK;
}

float elapsed(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
}

}  // namespace

namespace {

// After new bodies landed in the master arrays: check the device error word (non-finite
// input), list the heavy bodies (m >= heavy_frac * total mass).
int accept_bodies(kd_ctx *c) {
    const size_t n = c->n;
    launch_find_heavy(c->bodies, (uint32_t)n, c->prm.heavy_frac > 0 ? c->prm.heavy_frac : 2.0,
                      c->d_total, c->d_heavy, c->d_nheavy, c->dev_err, c->st);
    uint32_t nh = 0;
    uint32_t ids[kMaxHeavy];
    KD_CHECK(c, cudaMemcpyAsync(&nh, c->d_nheavy, sizeof nh, cudaMemcpyDeviceToHost, c->st));
    KD_CHECK(c, cudaMemcpyAsync(ids, c->d_heavy, sizeof ids, cudaMemcpyDeviceToHost, c->st));
    int rc = check_device(c);
    c->has_tree = false;
    if (rc) {
        c->has_bodies = false;
        return rc;
    }
    c->heavy.assign(ids, ids + std::min<uint32_t>(nh, kMaxHeavy));
    std::sort(c->heavy.begin(), c->heavy.end());
    c->n_heavy = (int)c->heavy.size();
    if (nh > (uint32_t)kMaxHeavy) {
        c->n_heavy = 0;
        c->heavy.clear();
        if (c->prm.precision == KD_PREC_MIXED) {
            c->has_bodies = false;
            return c->fail(KD_EINVAL, "%u bodies exceed heavy_frac of the total mass; at most %d",
                           nh, kMaxHeavy);
        }
    }
    if (c->n_heavy)
        KD_CHECK(c, cudaMemcpyAsync(c->d_heavy, c->heavy.data(), c->n_heavy * sizeof(uint32_t),
                                    cudaMemcpyHostToDevice, c->st));
    c->has_bodies = true;
    return KD_OK;
}

}  // namespace

struct kd_tape_impl {
    kd_ctx *ctx;
    uint64_t gen;  // the context's tape number: names the owner of the segment buffer
    double dt;
    int64_t steps, every;
    std::vector<double *> ck;  // per checkpoint: x|y|z|vx|vy|vz (6n)
    double *final_state;       // 6n
};

int copy_state(kd_ctx *c, double *dst6, bool to_buffer) {
    const size_t n = c->n, b = n * sizeof(double);
    double *arr[6] = {c->bodies.x, c->bodies.y, c->bodies.z,
                      c->bodies.vx, c->bodies.vy, c->bodies.vz};
    for (int k = 0; k < 6; ++k) {
        if (to_buffer)
            KD_CHECK(c, cudaMemcpyAsync(dst6 + k * n, arr[k], b, cudaMemcpyDeviceToDevice, c->st));
        else
            KD_CHECK(c, cudaMemcpyAsync(arr[k], dst6 + k * n, b, cudaMemcpyDeviceToDevice, c->st));
    }
    return KD_OK;
}

int adj_alloc(kd_ctx *c, int64_t every) {
    if (c->adj_ready && c->adj_every >= every) return KD_OK;
    const size_t n = c->n;
    if (!c->adj_ready) {
        KD_CHECK(c, c->alloc(&c->lx, 3 * n));
        KD_CHECK(c, c->alloc(&c->lv, 3 * n));
        KD_CHECK(c, c->alloc(&c->amu, 3 * n));
        KD_CHECK(c, c->alloc(&c->ay, 3 * n));
        KD_CHECK(c, c->alloc(&c->ysink, 3 * n));
        KD_CHECK(c, c->alloc(&c->yheavy, 3 * kMaxHeavy));
        KD_CHECK(c, c->alloc(&c->aU, 3 * n));
        KD_CHECK(c, c->alloc(&c->aG, 3 * (size_t)c->plan.n_nodes));
    }
    if (c->segbuf) {
        cudaFree(c->segbuf);
        c->owned.erase(std::find(c->owned.begin(), c->owned.end(), (void *)c->segbuf));
        c->segbuf = nullptr;
    }
    KD_CHECK(c, c->alloc(&c->segbuf, 3 * n * (size_t)every));
    c->seg_owner = 0;
    c->adj_every = every;
    c->adj_ready = true;
    return KD_OK;
}

void enqueue_step(kd_ctx *c, double dt) {
    const bool mixed = c->prm.precision == KD_PREC_MIXED;
    enqueue_build(c, !mixed, mixed);
    enqueue_walk(c);
    launch_kick_drift(c->bodies, c->acc, (uint32_t)c->n, dt, c->dev_err, c->st);
    c->launches += 1;
}

// `steps` steps on the context's stream.  A step is a fixed launch sequence for a given n and
// precision, so it is captured once into a CUDA graph and relaunched: one host call per step
// instead of ~100.  The graph is recaptured when dt, the precision or the heavy-body count
// (kernel arguments) change; counting and timing modes launch directly.
void enqueue_steps(kd_ctx *c, double dt, int64_t steps) {
    if (steps <= 0) return;
    if (c->counting || c->timing || c->graph_off) {
        for (int64_t s = 0; s < steps; ++s) enqueue_step(c, dt);
        return;
    }
    if (!c->graph || c->graph_dt != dt || c->graph_prec != c->prm.precision ||
        c->graph_heavy != c->n_heavy) {
        if (c->graph) cudaGraphExecDestroy(c->graph);
        c->graph = nullptr;
        const uint64_t l0 = c->launches;
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(c->st, cudaStreamCaptureModeRelaxed);
        if (e == cudaSuccess) {
            enqueue_step(c, dt);
            e = cudaStreamEndCapture(c->st, &g);
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&c->graph, g, 0);
        if (g) cudaGraphDestroy(g);
        c->graph_launches = c->launches - l0;
        c->launches = l0;
        if (e != cudaSuccess || !c->graph) {
            cudaGetLastError();  // clear: fall back to direct launches
            c->graph = nullptr;
            c->graph_off = true;
            for (int64_t s = 0; s < steps; ++s) enqueue_step(c, dt);
            return;
        }
        c->graph_dt = dt;
        c->graph_prec = c->prm.precision;
        c->graph_heavy = c->n_heavy;
    }
    for (int64_t s = 0; s < steps; ++s) {
        cudaGraphLaunch(c->graph, c->st);
        c->launches += c->graph_launches;
    }
}

// One backward step over the bodies' current positions: rebuild the (mixed) tree and apply
// the transpose-Jacobian step.  Replayed from a CUDA graph like the forward step (recaptured
// when dt or the heavy-body count changes).
void enqueue_adj_step(kd_ctx *c, const AdjArgs &a) {
    auto direct = [&]() {
        enqueue_build(c, false, true);
        c->launches += launch_adjoint_step(a, c->st);
    };
    if (c->counting || c->timing || c->graph_off) {
        direct();
        return;
    }
    if (!c->adj_graph || c->adj_graph_dt != a.dt || c->adj_graph_heavy != c->n_heavy) {
        if (c->adj_graph) cudaGraphExecDestroy(c->adj_graph);
        c->adj_graph = nullptr;
        const uint64_t l0 = c->launches;
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(c->st, cudaStreamCaptureModeRelaxed);
        if (e == cudaSuccess) {
            direct();
            e = cudaStreamEndCapture(c->st, &g);
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&c->adj_graph, g, 0);
        if (g) cudaGraphDestroy(g);
        c->adj_graph_launches = c->launches - l0;
        c->launches = l0;
        if (e != cudaSuccess || !c->adj_graph) {
            cudaGetLastError();
            c->adj_graph = nullptr;
            c->graph_off = true;
            direct();
            return;
        }
        c->adj_graph_dt = a.dt;
        c->adj_graph_heavy = c->n_heavy;
    }
    cudaGraphLaunch(c->adj_graph, c->st);
    c->launches += c->adj_graph_launches;
}

namespace kd {
void set_thread_error(const char *msg) { g_create_error = msg ? msg : ""; }

int sm_count() {
    constexpr int kDevices = 64;
    static std::atomic<int> cache[kDevices];  // 0: not queried yet
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kDevices) {
        cudaGetLastError();
        dev = -1;
    }
    int v = dev >= 0 ? cache[dev].load(std::memory_order_relaxed) : 0;
    if (v > 0) return v;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev < 0 ? 0 : dev) !=
            cudaSuccess ||
        v <= 0) {
        cudaGetLastError();
        return 1;  // grid-stride kernels stay correct on any grid
    }
    if (dev >= 0) cache[dev].store(v, std::memory_order_relaxed);
    return v;
}
}  // namespace kd

// Rust's `{}` for f64: the shortest digits that round-trip, written positionally (never in
// exponent form); "NaN", "inf", "-inf", "-0".
std::string rust_f64(double v) {
    if (std::isnan(v)) return "NaN";
    if (std::isinf(v)) return v < 0 ? "-inf" : "inf";
    char buf[64];
    auto r = std::to_chars(buf, buf + sizeof buf, v, std::chars_format::scientific);
    std::string sci(buf, r.ptr);  // [-]d[.ddd]e(+|-)xx
    std::string out;
    size_t i = 0;
    if (sci[0] == '-') {
        out = "-";
        i = 1;
    }
    const size_t epos = sci.find('e');
    std::string digits;
    for (size_t k = i; k < epos; ++k)
        if (sci[k] != '.') digits += sci[k];
    const int e = std::stoi(sci.substr(epos + 1));  // value = d.ddd * 10^e
    const int nd = (int)digits.size();
    if (e >= nd - 1) {
        out += digits + std::string((size_t)(e - (nd - 1)), '0');
    } else if (e >= 0) {
        out += digits.substr(0, (size_t)e + 1) + "." + digits.substr((size_t)e + 1);
    } else {
        out += "0." + std::string((size_t)(-e - 1), '0') + digits;
    }
    return out;
}

// ====================================================================== C ABI

extern "C" {

void kd_default_params(kd_params *p) {
    if (!p) return;
    p->leaf_size = 7;
    p->layout = KD_LAYOUT_DFS;
    p->precision = KD_PREC_FP64;
    p->device = 0;
    p->theta = 0.3;
    p->dt = 1e-3;
    p->heavy_frac = 1e-3;
    p->seed = 0;
}

size_t kd_nodes_needed(size_t n, int32_t leaf_size, int32_t layout) {
    if (leaf_size < 2 || leaf_size > KD_MAX_LEAF) return 0;
    return layout == KD_LAYOUT_PAR4 ? (size_t)needed_par(n, (uint32_t)leaf_size)
                                    : (size_t)needed_seq(n, (uint32_t)leaf_size);
}

int kd_group_plan(size_t n, int32_t leaf_size, uint32_t *gstart, uint32_t *gsplit, size_t cap,
                  size_t *n_groups) {
    if (n < 1 || n >= (size_t)1 << 31 || leaf_size < 2 || leaf_size > KD_MAX_LEAF || !n_groups) {
        g_create_error = "kd_group_plan: need 1 <= n < 2^31, leaf_size in [2, 8], n_groups";
        return KD_EINVAL;
    }
    Plan p;
    std::string err;
    if (!make_plan((uint32_t)n, (uint32_t)leaf_size, p, err)) {
        g_create_error = "kd_group_plan: " + err;
        return KD_EINVAL;
    }
    const size_t ng = p.gstart.size() - 1;
    *n_groups = ng;
    if (!gstart || !gsplit || cap < ng + 1) {
        g_create_error = "kd_group_plan: gstart needs n_groups + 1 entries (gsplit n_groups)";
        return KD_EINVAL;
    }
    std::copy(p.gstart.begin(), p.gstart.end(), gstart);
    std::copy(p.gsplit.begin(), p.gsplit.end(), gsplit);
    return KD_OK;
}

const char *kd_last_error(const kd_ctx *ctx) {
    return ctx ? ctx->err.c_str() : g_create_error.c_str();
}

kd_ctx *kd_create(size_t n, const kd_params *params) {
    kd_params prm;
    if (params)
        prm = *params;
    else
        kd_default_params(&prm);
    if (n < 1 || n >= (1ull << 31)) {
        g_create_error = "n must be in [1, 2^31)";
        return nullptr;
    }
    if (prm.leaf_size < 2 || prm.leaf_size > KD_MAX_LEAF) {
        g_create_error = "leaf_size must be in [2, 8]";
        return nullptr;
    }
    if (prm.layout != KD_LAYOUT_DFS && prm.layout != KD_LAYOUT_PAR4) {
        g_create_error = "unknown layout";
        return nullptr;
    }
    if (prm.precision != KD_PREC_FP64 && prm.precision != KD_PREC_MIXED) {
        g_create_error = "unknown precision";
        return nullptr;
    }
    if (!(prm.theta >= 0.0) || !std::isfinite(prm.theta)) {
        g_create_error = "theta must be finite and >= 0";
        return nullptr;
    }
    kd_ctx *c = new (std::nothrow) kd_ctx();
    if (!c) {
        g_create_error = "out of host memory";
        return nullptr;
    }
    c->n = n;
    c->prm = prm;
    std::string perr;
    if (!make_plan((uint32_t)n, (uint32_t)prm.leaf_size, c->plan, perr)) {
        g_create_error = perr;
        delete c;
        return nullptr;
    }
    if (prm.layout == KD_LAYOUT_PAR4 && !c->plan.par4_ok) {
        g_create_error = "PAR4 node slots exhausted for this n (build_tree_par4 would panic)";
        delete c;
        return nullptr;
    }
    if (setup(c) != KD_OK) {
        g_create_error = c->err;
        kd_destroy(c);
        return nullptr;
    }
    return c;
}

void kd_destroy(kd_ctx *c) {
    if (!c) return;
    cudaSetDevice(c->prm.device);
    if (c->st) cudaStreamSynchronize(c->st);
    if (c->graph) cudaGraphExecDestroy(c->graph);
    if (c->adj_graph) cudaGraphExecDestroy(c->adj_graph);
    for (void *p : c->owned) cudaFree(p);
    for (auto &e : c->ev)
        if (e) cudaEventDestroy(e);
    for (auto &e : c->tev)
        if (e) cudaEventDestroy(e);
    if (c->st) cudaStreamDestroy(c->st);
    delete c;
}

// Device-accessible address of a page-locked host buffer (registered or allocated pinned),
// 16-byte aligned as the transfer kernels' vector accesses need; nullptr for pageable or
// device memory and for other alignments.
static void *pinned_device_view(const void *p) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();  // an address CUDA does not know: clear the (non-sticky) error
        return nullptr;
    }
    if (at.type != cudaMemoryTypeHost || !at.devicePointer) return nullptr;
    return (reinterpret_cast<uintptr_t>(at.devicePointer) & 15u) == 0 ? at.devicePointer
                                                                      : nullptr;
}

int kd_set_bodies(kd_ctx *c, const kd_particle_c *bodies, size_t n) {
    if (!c) return KD_EINVAL;
    if (!bodies || n != c->n) return c->fail(KD_EINVAL, "expected %zu bodies", c->n);
    KD_CHECK(c, cudaSetDevice(c->prm.device));
    // pinned records are read in place by the converting kernel; others are staged
    if (const void *view = pinned_device_view(bodies)) {
        launch_host_to_soa(view, c->bodies, (uint32_t)n, c->dev_err, c->st);
    } else {
        KD_CHECK(c, cudaMemcpyAsync(c->aos, bodies, n * sizeof(kd_particle_c),
                                    cudaMemcpyHostToDevice, c->st));
        launch_aos_to_soa(c->aos, c->bodies, (uint32_t)n, c->dev_err, c->st);
    }
    return accept_bodies(c);
}

int kd_generate(kd_ctx *c, int32_t kind, uint64_t seed) {
    if (!c) return KD_EINVAL;
    KD_CHECK(c, cudaSetDevice(c->prm.device));
    KD_CHECK(c, cudaMemsetAsync(c->dev_err, 0, sizeof(uint32_t), c->st));
    if (launch_generate(kind, c->bodies, (uint32_t)c->n, seed, c->gen_scratch, c->st) < 0)
        return c->fail(KD_EINVAL, "unknown generator %d", kind);
    KD_CHECK(c, cudaGetLastError());
    return accept_bodies(c);
}

int kd_get_bodies(kd_ctx *c, kd_particle_c *bodies, size_t n) {
    if (!c) return KD_EINVAL;
    if (!bodies || n != c->n) return c->fail(KD_EINVAL, "expected %zu bodies", c->n);
    if (!c->has_bodies) return c->fail(KD_ESTATE, "no bodies set");
    KD_CHECK(c, cudaSetDevice(c->prm.device));
    if (void *view = pinned_device_view(bodies)) {
        launch_soa_to_host(c->bodies, view, (uint32_t)n, c->st);
    } else {
        launch_soa_to_aos(c->bodies, c->aos, (uint32_t)n, c->st);
        KD_CHECK(c, cudaMemcpyAsync(bodies, c->aos, n * sizeof(kd_particle_c),
                                    cudaMemcpyDeviceToHost, c->st));
    }
    KD_CHECK(c, cudaStreamSynchronize(c->st));
    return KD_OK;
}

int kd_build_tree(kd_ctx *c, size_t *last_node) {
    if (!c) return KD_EINVAL;
    if (!c->has_bodies) return c->fail(KD_ESTATE, "no bodies set");
    KD_CHECK(c, cudaSetDevice(c->prm.device));
    c->has_tree = false;  // until this build has passed its device checks
    KD_CHECK(c, cudaEventRecord(c->ev[0], c->st));
    enqueue_build(c, true, true);
    KD_CHECK(c, cudaEventRecord(c->ev[1], c->st));
    KD_CHECK(c, cudaEventRecord(c->ev[2], c->st));
    KD_CHECK(c, cudaGetLastError());
    int rc = check_device(c);
    if (rc) return rc;
    c->stats = kd_stats{};
    c->stats.build_ms = elapsed(c->ev[0], c->ev[1]);
    c->stats.moments_ms = elapsed(c->ev[1], c->ev[2]);
    c->stats.total_ms = elapsed(c->ev[0], c->ev[2]);
    c->has_tree = true;
    c->tree_fp64 = true;
    c->tree_mixed = true;
    if (last_node)
        *last_node = c->prm.layout == KD_LAYOUT_PAR4 ? (size_t)c->plan.par4_last
                                                     : (size_t)c->plan.n_nodes - 1;
    return KD_OK;
}

int kd_get_nodes(kd_ctx *c, kd_node_c *out, size_t cap, size_t *count) {
    if (!c) return KD_EINVAL;
    if (!c->has_tree || !c->tree_fp64) return c->fail(KD_ESTATE, "no tree built");
    const Plan &p = c->plan;
    const size_t need = c->prm.layout == KD_LAYOUT_PAR4 ? p.par4_slots : p.n_nodes;
    if (!out || cap < need) return c->fail(KD_EINVAL, "need %zu node slots", need);
    KD_CHECK(c, cudaSetDevice(c->prm.device));
    const size_t nn = p.n_nodes;
    std::vector<uint8_t> sd(nn);
    std::vector<double> sv(nn), sz(nn), M(nn), S(3 * nn);
    std::vector<uint32_t> tid(c->n);
    KD_CHECK(c, cudaMemcpyAsync(sd.data(), c->nout.split_dim, nn, cudaMemcpyDeviceToHost, c->st));
    KD_CHECK(c, cudaMemcpyAsync(sv.data(), c->nout.split_val, nn * 8, cudaMemcpyDeviceToHost, c->st));
    KD_CHECK(c, cudaMemcpyAsync(sz.data(), c->nout.size, nn * 8, cudaMemcpyDeviceToHost, c->st));
    KD_CHECK(c, cudaMemcpyAsync(M.data(), c->mom.M, nn * 8, cudaMemcpyDeviceToHost, c->st));
    KD_CHECK(c, cudaMemcpyAsync(S.data(), c->mom.S, 3 * nn * 8, cudaMemcpyDeviceToHost, c->st));
    KD_CHECK(c, cudaMemcpyAsync(tid.data(), c->tid, c->n * 4, cudaMemcpyDeviceToHost, c->st));
    KD_CHECK(c, cudaStreamSynchronize(c->st));
    const bool par4 = c->prm.layout == KD_LAYOUT_PAR4;
    if (par4) {
        // unused slots stay as allocate_node_vec leaves them: Leaf{0, [usize::MAX; MAX]}
        for (size_t i = 0; i < need; ++i) {
            memset(&out[i], 0, sizeof(kd_node_c));
            for (int k = 0; k < KD_MAX_LEAF; ++k) out[i].particles[k] = ~0ull;
        }
    }
    auto slot = [&](uint32_t id) -> size_t { return par4 ? (size_t)p.par4[id] : (size_t)id; };
    for (uint32_t id = 0; id < nn; ++id) {
        kd_node_c &o = out[slot(id)];
        memset(&o, 0, sizeof o);
        if (p.count[id] > p.leaf) {
            o.num_parts = 0;
            o.split_dim = sd[id];
            o.split_val = sv[id];
            o.m = M[id];
            o.cm[0] = S[3 * id] / M[id];
            o.cm[1] = S[3 * id + 1] / M[id];
            o.cm[2] = S[3 * id + 2] / M[id];
            o.size = sz[id];
            o.left = slot(id + 1);
            o.right = slot(p.right[id]);
        } else {
            o.num_parts = p.count[id];
            for (uint32_t k = 0; k < p.count[id]; ++k) o.particles[k] = tid[p.start[id] + k];
        }
    }
    if (count) *count = need;
    return KD_OK;
}

int kd_quickstat_index(const double *vals, size_t n_vals, uint64_t *idx, size_t n, size_t goal,
                       int32_t device, double *gpu_ms) {
    if (!vals || !idx || n < 1 || n >= (1ull << 31) || goal >= n || n_vals < 1) {
        g_create_error = "kd_quickstat_index: need vals, idx, 1 <= n < 2^31 and goal < n";
        return KD_EINVAL;
    }
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) {
        g_create_error = cudaGetErrorString(e);
        return KD_ECUDA;
    }
    const uint32_t nn = (uint32_t)n;
    const uint32_t tiles = (nn + kTile - 1) / kTile;
    std::vector<void *> mem;
    auto get = [&](size_t bytes) -> void * {
        void *p = nullptr;
        if (e == cudaSuccess) e = cudaMalloc(&p, bytes ? bytes : 1);
        if (e == cudaSuccess) mem.push_back(p);
        return p;
    };
    double *d_vals = (double *)get(n_vals * sizeof(double));
    uint64_t *d_idx = (uint64_t *)get(n * sizeof(uint64_t));
    Work w{};
    Scratch sc{};
    for (int k = 0; k < 2; ++k) {
        w.x[k] = w.y[k] = w.z[k] = (double *)get(n * sizeof(double));
        w.id[k] = (uint32_t *)get(n * sizeof(uint32_t));
        sc.bmin[k] = (unsigned long long *)get(3 * sizeof(unsigned long long));
        sc.bmax[k] = (unsigned long long *)get(3 * sizeof(unsigned long long));
    }
    for (int k = 0; k < 3; ++k) {
        sc.ckey[k] = (unsigned long long *)get(n * sizeof(unsigned long long));
        sc.cpos[k] = (uint32_t *)get(n * sizeof(uint32_t));
    }
    sc.done = (uint32_t *)get(sizeof(uint32_t));
    sc.sel = (SegSel *)get(sizeof(SegSel));
    sc.hist = (uint32_t *)get(kHistBins * sizeof(uint32_t));
    sc.cand_cnt = (uint32_t *)get(sizeof(uint32_t));
    sc.tile_cnt = (uint32_t *)get(tiles * sizeof(uint32_t));
    sc.tile_off = (uint32_t *)get(tiles * sizeof(uint32_t));
    sc.err = (uint32_t *)get(sizeof(uint32_t));
    uint32_t *d_seg = (uint32_t *)get(3 * sizeof(uint32_t));  // start, count, node id
    uint32_t *d_med = (uint32_t *)get(sizeof(uint32_t));
    NodeOut no;
    no.split_dim = (uint8_t *)get(8);
    no.split_val = (double *)get(8);
    no.size = (double *)get(8);
    cudaStream_t st = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&ev[0]);
    if (e == cudaSuccess) e = cudaEventCreate(&ev[1]);
    const uint32_t seg_h[3] = {0u, nn, 0u};
    uint32_t err_h = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_vals, vals, n_vals * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_idx, idx, n * sizeof(uint64_t), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_seg, seg_h, sizeof seg_h, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(sc.err, 0, sizeof(uint32_t), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(sc.done, 0, sizeof(uint32_t), st);
    if (e == cudaSuccess) {
        // one segment [0, n): its start / count live where a tree's node arrays would
        Topology t{};
        t.n = nn;
        t.n_nodes = 1;
        t.start = d_seg;
        t.count = d_seg + 1;
        LevelArgs lv;
        lv.ids = d_seg + 2;
        lv.G = 1;
        lv.tiles = tiles;
        lv.multi = nn > kMultiMin;
        lv.rank = (uint32_t)goal;
        lv.med_pos = d_med;
        cudaEventRecord(ev[0], st);
        launch_gather_keys(d_vals, n_vals, d_idx, nn, w.x[0], w.id[0], sc.err, st);
        launch_level(t, lv, no, w, 0, sc, 0, 0, st);
        launch_place_selected(w.id[1], d_med, (uint32_t)goal, st);
        cudaEventRecord(ev[1], st);
        e = cudaGetLastError();
    }
    std::vector<uint32_t> out(n);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out.data(), w.id[1], n * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&err_h, sc.err, sizeof err_h, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    float ms = 0.f;
    if (e == cudaSuccess && gpu_ms) {
        cudaEventElapsedTime(&ms, ev[0], ev[1]);
        *gpu_ms = ms;
    }
    for (auto &x : ev)
        if (x) cudaEventDestroy(x);
    if (st) cudaStreamDestroy(st);
    for (void *p : mem) cudaFree(p);
    if (e != cudaSuccess) {
        g_create_error = std::string("kd_quickstat_index: ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? KD_ENOMEM : KD_ECUDA;
    }
    if (err_h & kErrNumeric) {
        g_create_error = "kd_quickstat_index: an index is out of range or a value is not finite";
        return KD_ENUMERIC;
    }
    if (err_h) {
        g_create_error = "kd_quickstat_index: select failed to converge";
        return KD_EDEVICE;
    }
    for (size_t i = 0; i < n; ++i) idx[i] = out[i];
    return KD_OK;
}

int kd_energy(kd_ctx *c, double out[2]) {
    if (!c) return KD_EINVAL;
    if (!out) return c->fail(KD_EINVAL, "out is NULL");
    if (!c->has_bodies) return c->fail(KD_ESTATE, "no bodies set");
    KD_CHECK(c, cudaSetDevice(c->prm.device));
    if (!c->phi) KD_CHECK(c, c->alloc(&c->phi, c->n));
    constexpr int kBlocks = 256;
    enqueue_build(c, false, true);
    launch_walk_group(c->recf, c->thi, c->tlo, c->trel, c->tid, c->d_gstart, c->d_gsplit,
                      c->n_groups, c->walk_stack(), c->prm.theta, c->bodies, c->d_heavy,
                      c->n_heavy, c->acc, c->d_hpart, c->d_hcount, c->dev_err, nullptr, c->st,
                      c->phi);
    launch_energy_partial(c->bodies, c->phi, (uint32_t)c->n, c->gen_scratch, kBlocks, c->st);
    double part[2 * kBlocks];
    KD_CHECK(c, cudaMemcpyAsync(part, c->gen_scratch, sizeof part, cudaMemcpyDeviceToHost,
                                c->st));
    int rc = check_device(c);
    c->has_tree = false;  // only the mixed records of this tree were built
    if (rc) return rc;
    double k = 0.0, p = 0.0;
    for (int i = 0; i < kBlocks; ++i) {
        k += part[2 * i];
        p += part[2 * i + 1];
    }
    out[0] = k;
    out[1] = p;
    return KD_OK;
}

int kd_print_tree(kd_ctx *c, const char *path) {
    if (!c) return KD_EINVAL;
    if (!path) return c->fail(KD_EINVAL, "path is NULL");
    const Plan &p = c->plan;
    const bool par4 = c->prm.layout == KD_LAYOUT_PAR4;
    const size_t slots = par4 ? (size_t)p.par4_slots : (size_t)p.n_nodes;
    std::vector<kd_node_c> nodes(slots);
    size_t count = 0;
    int rc = kd_get_nodes(c, nodes.data(), slots, &count);
    if (rc) return rc;
    std::vector<kd_particle_c> b(c->n);
    rc = kd_get_bodies(c, b.data(), c->n);
    if (rc) return rc;
    // the Vec the reference prints: allocate_node_vec(n) slots (grown on demand for DFS)
    const size_t len = par4 ? count
                            : std::max(count, (size_t)needed_seq(c->n, (uint32_t)c->prm.leaf_size));
    FILE *f = fopen(path, "w");
    if (!f) return c->fail(KD_EINVAL, "cannot open %s", path);
    std::string out = std::to_string(len) + "\n";
    for (size_t i = 0; i < len; ++i) {
        if (i >= count) {
            out += "L 0\n";
        } else if (nodes[i].num_parts > 0 || (nodes[i].left == 0 && nodes[i].right == 0)) {
            out += "L " + std::to_string(nodes[i].num_parts) + "\n";
            for (uint64_t k = 0; k < nodes[i].num_parts; ++k) {
                const kd_particle_c &q = b[nodes[i].particles[k]];
                out += rust_f64(q.p[0]) + " " + rust_f64(q.p[1]) + " " + rust_f64(q.p[2]) + "\n";
            }
        } else {
            out += "I " + std::to_string(nodes[i].split_dim) + " " + rust_f64(nodes[i].split_val) +
                   " " + std::to_string(nodes[i].left) + " " + std::to_string(nodes[i].right) +
                   "\n";
        }
        if (out.size() > (1u << 20)) {
            fputs(out.c_str(), f);
            out.clear();
        }
    }
    fputs(out.c_str(), f);
    const bool bad = ferror(f) != 0;
    fclose(f);
    if (bad) return c->fail(KD_EINVAL, "write to %s failed", path);
    return KD_OK;
}

int kd_calc_accel(kd_ctx *c, double *acc) {
    if (!c) return KD_EINVAL;
    if (!acc) return c->fail(KD_EINVAL, "acc is NULL");
    if (!c->has_tree) return c->fail(KD_ESTATE, "no tree built");
    KD_CHECK(c, cudaSetDevice(c->prm.device));
    int rc = reset_counts(c);
    if (rc) return rc;
    KD_CHECK(c, cudaEventRecord(c->ev[0], c->st));
    enqueue_walk(c);
    KD_CHECK(c, cudaEventRecord(c->ev[1], c->st));
    KD_CHECK(c, cudaGetLastError());
    KD_CHECK(c, cudaMemcpyAsync(acc, c->acc, 3 * c->n * sizeof(double), cudaMemcpyDeviceToHost,
                                c->st));
    rc = check_device(c);
    if (rc) return rc;
    c->stats = kd_stats{};
    c->stats.walk_ms = elapsed(c->ev[0], c->ev[1]);
    c->stats.total_ms = c->stats.walk_ms;
    return fetch_counts(c);
}

int kd_simple_sim(kd_ctx *c, double dt, int64_t steps) {
    if (!c) return KD_EINVAL;
    if (!c->has_bodies) return c->fail(KD_ESTATE, "no bodies set");
    if (steps < 0) return c->fail(KD_EINVAL, "steps must be >= 0");
    if (dt == 0.0) dt = c->prm.dt;
    KD_CHECK(c, cudaSetDevice(c->prm.device));
    const bool mixed = c->prm.precision == KD_PREC_MIXED;
    int rc = reset_counts(c);
    if (rc) return rc;
    const size_t nev = c->timing ? 5 * (size_t)steps : 0;
    while (c->tev.size() < nev) {
        cudaEvent_t e;
        KD_CHECK(c, cudaEventCreate(&e));
        c->tev.push_back(e);
    }
    c->launches = 0;
    KD_CHECK(c, cudaEventRecord(c->ev[0], c->st));
    if (!c->timing) enqueue_steps(c, dt, steps);
    for (int64_t s = 0; s < (c->timing ? steps : 0); ++s) {
        cudaEvent_t *e = c->timing ? &c->tev[5 * (size_t)s] : nullptr;
        if (e) KD_CHECK(c, cudaEventRecord(e[0], c->st));
        enqueue_build(c, !mixed, mixed);
        if (e) KD_CHECK(c, cudaEventRecord(e[1], c->st));
        if (e) KD_CHECK(c, cudaEventRecord(e[2], c->st));
        enqueue_walk(c);
        if (e) KD_CHECK(c, cudaEventRecord(e[3], c->st));
        launch_kick_drift(c->bodies, c->acc, (uint32_t)c->n, dt, c->dev_err, c->st);
        c->launches += 1;
        if (e) KD_CHECK(c, cudaEventRecord(e[4], c->st));
    }
    KD_CHECK(c, cudaEventRecord(c->ev[1], c->st));
    KD_CHECK(c, cudaGetLastError());
    rc = check_device(c);
    c->has_tree = false;  // the tree no longer matches the moved bodies
    if (rc) return rc;
    c->stats = kd_stats{};
    c->stats.total_ms = elapsed(c->ev[0], c->ev[1]);
    c->stats.steps = (uint64_t)steps;
    c->stats.launches = c->launches;
    for (int64_t s = 0; s < (c->timing ? steps : 0); ++s) {
        cudaEvent_t *e = &c->tev[5 * (size_t)s];
        c->stats.build_ms += elapsed(e[0], e[1]);
        c->stats.moments_ms += elapsed(e[1], e[2]);
        c->stats.walk_ms += elapsed(e[2], e[3]);
        c->stats.kick_ms += elapsed(e[3], e[4]);
    }
    return fetch_counts(c);
}

int kd_set_precision(kd_ctx *c, int32_t precision) {
    if (!c) return KD_EINVAL;
    if (precision != KD_PREC_FP64 && precision != KD_PREC_MIXED)
        return c->fail(KD_EINVAL, "unknown precision");
    c->prm.precision = precision;
    return KD_OK;
}

int kd_get_stats(const kd_ctx *c, kd_stats *out) {
    if (!c || !out) return KD_EINVAL;
    *out = c->stats;
    return KD_OK;
}

int kd_forward(kd_ctx *c, double dt, int64_t steps, int64_t ckpt_every, kd_tape **out) {
    if (!c) return KD_EINVAL;
    if (!out) return c->fail(KD_EINVAL, "tape pointer is NULL");
    *out = nullptr;
    if (!c->has_bodies) return c->fail(KD_ESTATE, "no bodies set");
    if (c->prm.precision != KD_PREC_MIXED)
        return c->fail(KD_EINVAL, "the adjoint is implemented for KD_PREC_MIXED contexts");
    if (c->plan.n_nodes >= 0x80000000u)
        return c->fail(KD_EINVAL, "the adjoint supports trees of fewer than 2^31 nodes");
    if (steps < 1 || ckpt_every < 1) return c->fail(KD_EINVAL, "steps and ckpt_every must be >= 1");
    if (dt == 0.0) dt = c->prm.dt;
    KD_CHECK(c, cudaSetDevice(c->prm.device));
    int rc = adj_alloc(c, ckpt_every);
    if (rc) return rc;
    kd_tape_impl *t = new (std::nothrow) kd_tape_impl();
    if (!t) return c->fail(KD_ENOMEM, "out of host memory");
    t->ctx = c;
    t->gen = ++c->tapes;
    t->dt = dt;
    t->steps = steps;
    t->every = ckpt_every;
    t->final_state = nullptr;
    const size_t nck = (size_t)((steps + ckpt_every - 1) / ckpt_every);
    cudaError_t e = cudaSuccess;
    auto take = [&]() -> double * {
        if (!c->ck_free.empty()) {
            double *p = c->ck_free.back();
            c->ck_free.pop_back();
            return p;
        }
        double *p = nullptr;
        e = c->alloc(&p, 6 * c->n);
        return e == cudaSuccess ? p : nullptr;
    };
    for (size_t k = 0; k < nck && e == cudaSuccess; ++k) {
        double *p = take();
        if (p) t->ck.push_back(p);
    }
    if (e == cudaSuccess) t->final_state = take();
    if (e != cudaSuccess) {
        kd_tape_free(reinterpret_cast<kd_tape *>(t));
        return c->cuda_fail(e, "checkpoint allocation");
    }
    c->launches = 0;
    // the last segment's positions stay in segbuf, so the backward sweep need not recompute
    // that segment (the forward is deterministic: they are the positions it would recompute)
    const int64_t last0 = ((steps - 1) / ckpt_every) * ckpt_every;
    const size_t n = c->n;
    double *pos[3] = {c->bodies.x, c->bodies.y, c->bodies.z};
    c->seg_owner = 0;
    KD_CHECK(c, cudaEventRecord(c->ev[0], c->st));
    for (int64_t s = 0; s < steps; ++s) {
        if (s % ckpt_every == 0) {
            rc = copy_state(c, t->ck[(size_t)(s / ckpt_every)], true);
            if (rc) break;
        }
        if (s >= last0) {
            double *dst = c->segbuf + 3 * n * (size_t)(s - last0);
            for (int k = 0; k < 3; ++k)
                KD_CHECK(c, cudaMemcpyAsync(dst + k * n, pos[k], n * sizeof(double),
                                            cudaMemcpyDeviceToDevice, c->st));
        }
        enqueue_steps(c, dt, 1);
    }
    if (!rc) rc = copy_state(c, t->final_state, true);
    KD_CHECK(c, cudaEventRecord(c->ev[1], c->st));
    if (!rc) rc = check_device(c);
    if (rc) {
        kd_tape_free(reinterpret_cast<kd_tape *>(t));
        return rc;
    }
    c->has_tree = false;
    c->seg_owner = t->gen;
    c->stats = kd_stats{};
    c->stats.total_ms = elapsed(c->ev[0], c->ev[1]);
    c->stats.steps = (uint64_t)steps;
    c->stats.launches = c->launches;
    *out = reinterpret_cast<kd_tape *>(t);
    return KD_OK;
}

int kd_backward(kd_tape *tape, const double *dL_dx, const double *dL_dv, double *g_x0,
                double *g_v0) {
    if (!tape) return KD_EINVAL;
    kd_tape_impl *t = reinterpret_cast<kd_tape_impl *>(tape);
    kd_ctx *c = t->ctx;
    if (!dL_dx || !g_x0 || !g_v0) return c->fail(KD_EINVAL, "NULL gradient buffer");
    if (c->prm.precision != KD_PREC_MIXED)
        return c->fail(KD_EINVAL, "the adjoint is implemented for KD_PREC_MIXED contexts");
    if (c->plan.n_nodes >= 0x80000000u)
        return c->fail(KD_EINVAL, "the adjoint supports trees of fewer than 2^31 nodes");
    KD_CHECK(c, cudaSetDevice(c->prm.device));
    int rc = adj_alloc(c, t->every);
    if (rc) return rc;
    const size_t n = c->n, b3 = 3 * n * sizeof(double);
    KD_CHECK(c, cudaMemcpyAsync(c->lx, dL_dx, b3, cudaMemcpyHostToDevice, c->st));
    if (dL_dv)
        KD_CHECK(c, cudaMemcpyAsync(c->lv, dL_dv, b3, cudaMemcpyHostToDevice, c->st));
    else
        KD_CHECK(c, cudaMemsetAsync(c->lv, 0, b3, c->st));
    AdjArgs a;
    a.topo = c->topo;
    a.recf = c->recf;
    a.thi = c->thi;
    a.tlo = c->tlo;
    a.trel = c->trel;
    a.tid = c->tid;
    a.n = (uint32_t)n;
    a.theta = c->prm.theta;
    a.dt = t->dt;
    a.bodies = c->bodies;
    a.heavy = c->d_heavy;
    a.n_heavy = c->n_heavy;
    a.lx = c->lx;
    a.lv = c->lv;
    a.mu = c->amu;
    a.y = c->ay;
    a.ysink = c->ysink;
    a.yheavy = c->yheavy;
    a.hpart = c->d_hpart;
    a.hcount = c->d_hcount;
    a.U = c->aU;
    a.G = c->aG;
    a.err = c->dev_err;
    a.gstart = c->d_gstart;
    a.gsplit = c->d_gsplit;
    a.n_groups = c->n_groups;
    a.stk_cap = c->walk_stack();
    c->launches = 0;
    KD_CHECK(c, cudaEventRecord(c->ev[0], c->st));
    const int64_t nseg = (t->steps + t->every - 1) / t->every;
    double *pos[3] = {c->bodies.x, c->bodies.y, c->bodies.z};
    for (int64_t seg = nseg - 1; seg >= 0 && !rc; --seg) {
        const int64_t n0 = seg * t->every, n1 = std::min(t->steps, n0 + t->every);
        const bool kept = seg == nseg - 1 && c->seg_owner == t->gen;
        if (!kept) {
            c->seg_owner = 0;
            rc = copy_state(c, t->ck[(size_t)seg], false);
            if (rc) break;
        }
        // recompute the segment forward, keeping the positions at the start of every step
        for (int64_t s = n0; s < n1 && !kept; ++s) {
            double *dst = c->segbuf + 3 * n * (size_t)(s - n0);
            for (int k = 0; k < 3; ++k)
                KD_CHECK(c, cudaMemcpyAsync(dst + k * n, pos[k], n * sizeof(double),
                                            cudaMemcpyDeviceToDevice, c->st));
            if (s + 1 < n1) enqueue_steps(c, t->dt, 1);
        }
        for (int64_t s = n1 - 1; s >= n0; --s) {
            const double *src = c->segbuf + 3 * n * (size_t)(s - n0);
            for (int k = 0; k < 3; ++k)
                KD_CHECK(c, cudaMemcpyAsync(pos[k], src + k * n, n * sizeof(double),
                                            cudaMemcpyDeviceToDevice, c->st));
            enqueue_adj_step(c, a);
        }
    }
    if (!rc) rc = copy_state(c, t->final_state, false);
    KD_CHECK(c, cudaEventRecord(c->ev[1], c->st));
    KD_CHECK(c, cudaGetLastError());
    if (rc) return rc;
    KD_CHECK(c, cudaMemcpyAsync(g_x0, c->lx, b3, cudaMemcpyDeviceToHost, c->st));
    KD_CHECK(c, cudaMemcpyAsync(g_v0, c->lv, b3, cudaMemcpyDeviceToHost, c->st));
    rc = check_device(c);
    if (rc) return rc;
    c->has_tree = false;
    c->stats = kd_stats{};
    c->stats.total_ms = elapsed(c->ev[0], c->ev[1]);
    c->stats.steps = (uint64_t)t->steps;
    c->stats.launches = c->launches;
    return KD_OK;
}

void kd_tape_free(kd_tape *tape) {
    if (!tape) return;
    kd_tape_impl *t = reinterpret_cast<kd_tape_impl *>(tape);
    // the checkpoint buffers belong to the context: back to its free list for the next
    // forward sweep (kd_destroy releases them)
    kd_ctx *c = t->ctx;
    for (double *p : t->ck) c->ck_free.push_back(p);
    if (t->final_state) c->ck_free.push_back(t->final_state);
    delete t;
}

int kd_set_timing(kd_ctx *c, int32_t on) {
    if (!c) return KD_EINVAL;
    c->timing = on != 0;
    return KD_OK;
}

int kd_direct_accel(kd_ctx *c, const uint64_t *sinks, size_t ns, double *acc) {
    if (!c) return KD_EINVAL;
    if (!c->has_bodies) return c->fail(KD_ESTATE, "no bodies set");
    if (!sinks || !acc || ns == 0 || ns > (1u << 24))
        return c->fail(KD_EINVAL, "need 1 <= ns <= 2^24 sinks and output storage");
    for (size_t k = 0; k < ns; ++k)
        if (sinks[k] >= c->n) return c->fail(KD_EINVAL, "sink %zu out of range", k);
    KD_CHECK(c, cudaSetDevice(c->prm.device));
    const size_t chunks = (c->n + kDirectChunk - 1) / kDirectChunk;
    uint64_t *d_sinks = nullptr;
    double *d_part = nullptr, *d_acc = nullptr;
    cudaError_t e = cudaMalloc((void **)&d_sinks, ns * sizeof(uint64_t));
    if (e == cudaSuccess) e = cudaMalloc((void **)&d_part, 3 * ns * chunks * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc((void **)&d_acc, 3 * ns * sizeof(double));
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_sinks, sinks, ns * sizeof(uint64_t), cudaMemcpyHostToDevice, c->st);
    if (e == cudaSuccess) {
        launch_direct(c->bodies, (uint32_t)c->n, d_sinks, (uint32_t)ns, d_part, d_acc, c->st);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(acc, d_acc, 3 * ns * sizeof(double), cudaMemcpyDeviceToHost, c->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    cudaFree(d_sinks);
    cudaFree(d_part);
    cudaFree(d_acc);
    if (e != cudaSuccess) return c->cuda_fail(e, "kd_direct_accel");
    return KD_OK;
}

int kd_set_device_limits(kd_ctx *c, int32_t stack_entries, int32_t select_passes) {
    if (!c) return KD_EINVAL;
    if ((stack_entries >= 0 && stack_entries < 2) || select_passes > kSelMaxIters)
        return c->fail(KD_EINVAL, "need stack_entries >= 2 and select_passes <= %d "
                       "(negative: the default)", kSelMaxIters);
    c->stack_limit = stack_entries < 0 ? 0u : (uint32_t)stack_entries;
    c->select_passes = select_passes < 0 ? kSelMaxIters : (int)select_passes;
    // the captured step graphs hold the old limits as kernel arguments
    KD_CHECK(c, cudaSetDevice(c->prm.device));
    KD_CHECK(c, cudaStreamSynchronize(c->st));
    if (c->graph) cudaGraphExecDestroy(c->graph);
    if (c->adj_graph) cudaGraphExecDestroy(c->adj_graph);
    c->graph = nullptr;
    c->adj_graph = nullptr;
    return KD_OK;
}

int kd_set_counting(kd_ctx *c, int32_t on) {
    if (!c) return KD_EINVAL;
    c->counting = on != 0;
    return KD_OK;
}

int kd_get_counts(const kd_ctx *c, uint64_t out[4]) {
    if (!c || !out) return KD_EINVAL;
    for (int i = 0; i < 4; ++i) out[i] = c->counts[i];
    return KD_OK;
}

}  // extern "C"
