/*
 * kdoracle.c -- CPU ORACLE for the kD-tree Barnes-Hut step.  TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, in plain C, the reference's Rust implementation of the hot path
 * (MarkCLewis/MultiLanguageKDTree, Parallel/RustVersion/src/array_kd_tree.rs,
 * quickstat.rs, array_particle.rs and the leaf-7 constants of
 * Sequential/RustVersion/src/array_kd_tree.rs).  It is the checker that the CUDA library
 * is compared against: only tests, the smoke check and the CPU-baseline leg of the bench
 * may load it.  Nothing in the product links or calls it.
 *
 * Parity pin: the restatement is validated against the reference's own C port
 * (Parallel/CVersion/src/kdtree.c), compiled from the reference sources into oracle/_ref
 * by oracle/build.py, on identical particle arrays (tests/test_oracle.py), and against
 * the quickstat known answer of quickstat.rs:191-197.
 *
 * Arithmetic: every floating-point expression keeps the reference's operation order and is
 * compiled with -ffp-contract=off, so no multiply-add is fused (Rust never fuses).
 * The pivot RNG (fastrand in the reference) is a seeded splitmix64 here: pivots only decide
 * the order of indices inside a node, never which bodies a node holds when keys differ.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_MAX_LEAF 8

/* Particle record: array_particle.rs:3-8 (p[3], v[3], r, m; 64 bytes). */
typedef struct {
    double p[3];
    double v[3];
    double r;
    double m;
} orc_particle;

/* Flat node record, field for field the C port's KDTree (Parallel/CVersion/src/kdtree.h:9-22)
 * widened to 8 leaf slots so both leaf sizes of the reference (7 and 8) fit. */
typedef struct {
    uint64_t num_parts;
    uint64_t particles[ORC_MAX_LEAF];
    uint64_t split_dim;
    double split_val;
    double m;
    double cm[3];
    double size;
    uint64_t left;
    uint64_t right;
} orc_node;

typedef struct {
    uint64_t s;
} orc_rng;

static uint64_t rng_next(orc_rng *r) {
    uint64_t z = (r->s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

/* uniform integer in [lo, hi) -- stands in for fastrand::usize(s..e) */
static size_t rng_range(orc_rng *r, size_t lo, size_t hi) {
    return lo + (size_t)(rng_next(r) % (uint64_t)(hi - lo));
}

/* ---------------------------------------------------------------- node counts */

/* nodes_needed_for_particles, Parallel/RustVersion/src/array_kd_tree.rs:45-53.
 * 2^ceil(log2(x)) is taken as the smallest power of two >= x, which equals the Rust
 * f64 expression for every x below 2^52. */
uint64_t orc_nodes_needed_par(uint64_t n, int leaf) {
    if (n <= (uint64_t)leaf) return 1;
    uint64_t min_leaves = n / (uint64_t)(leaf / 2);
    uint64_t leaves = 1;
    while (leaves < min_leaves) leaves <<= 1;
    return 2 * leaves - 1;
}

/* nodes_needed_for_particles, Sequential/RustVersion/src/array_kd_tree.rs:37-39 */
uint64_t orc_nodes_needed_seq(uint64_t n, int leaf) {
    return 2 * (n / (uint64_t)(leaf / 2) + 1);
}

/* ---------------------------------------------------------------- quickselect */

/* quickstat_index, Parallel/RustVersion/src/quickstat.rs:9-34, with the comparator
 * `lt(a, b) = keys[a] < keys[b]` (array_kd_tree.rs:561-562 passes p[split_dim]). */
static void quickstat_keys(uint64_t *idx, size_t len, size_t goal, const double *keys,
                           size_t stride, orc_rng *rng) {
    size_t s = 0, e = len;
    while (s + 1 < e) {
        size_t pivot = rng_range(rng, s, e);
        uint64_t t = idx[s]; idx[s] = idx[pivot]; idx[pivot] = t;
        size_t low = s + 1, high = e - 1;
        while (low <= high) {
            if (keys[idx[low] * stride] < keys[idx[s] * stride]) {
                low += 1;
            } else {
                t = idx[low]; idx[low] = idx[high]; idx[high] = t;
                high -= 1;
            }
        }
        t = idx[s]; idx[s] = idx[high]; idx[high] = t;
        if (high < goal) s = high + 1;
        else if (high > goal) e = high;
        else s = e;
    }
}

/* Public form used by the known-answer test: values are a plain array. */
void orc_quickstat_index(uint64_t *idx, size_t len, size_t goal, const double *vals,
                         uint64_t seed) {
    orc_rng rng = {seed};
    quickstat_keys(idx, len, goal, vals, 1, &rng);
}

/* ---------------------------------------------------------------- build */

/* Segment scan of array_kd_tree.rs:532-557 (par4) / :86-111 (DFS): mass, unnormalised
 * then normalised centre of mass, bounding box from +-1e100, split dimension by strict >
 * from dim 0, size = extent along the split dimension. */
static void scan_segment(const uint64_t *idx, size_t len, const orc_particle *P,
                         double *m_out, double cm[3], uint64_t *split_dim, double *size) {
    double mn[3] = {1e100, 1e100, 1e100};
    double mx[3] = {-1e100, -1e100, -1e100};
    double m = 0.0;
    cm[0] = cm[1] = cm[2] = 0.0;
    for (size_t i = 0; i < len; ++i) {
        const orc_particle *q = &P[idx[i]];
        m += q->m;
        cm[0] += q->m * q->p[0];
        cm[1] += q->m * q->p[1];
        cm[2] += q->m * q->p[2];
        for (int d = 0; d < 3; ++d) {
            mn[d] = fmin(mn[d], q->p[d]);
            mx[d] = fmax(mx[d], q->p[d]);
        }
    }
    cm[0] /= m;
    cm[1] /= m;
    cm[2] /= m;
    uint64_t sd = 0;
    for (int d = 1; d < 3; ++d)
        if (mx[d] - mn[d] > mx[sd] - mn[sd]) sd = (uint64_t)d;
    *m_out = m;
    *split_dim = sd;
    *size = mx[sd] - mn[sd];
}

typedef struct {
    orc_node *nodes;
    size_t cap;
    int leaf;
    int overflow;
    orc_rng rng;
} dfs_state;

static int ensure_cap(dfs_state *st, size_t node) {
    if (node < st->cap) return 1;
    st->overflow = 1; /* the reference grows its Vec here (array_kd_tree.rs:75-77) */
    return 0;
}

/* build_tree (DFS-packed numbering), Parallel/RustVersion/src/array_kd_tree.rs:63-130 and
 * Sequential/RustVersion/src/array_kd_tree.rs:49-138.  Returns the last node used. */
static size_t build_dfs(uint64_t *idx, size_t start, size_t end, const orc_particle *P,
                        size_t cur, dfs_state *st) {
    size_t np = end - start;
    if (np <= (size_t)st->leaf) {
        if (!ensure_cap(st, cur)) return cur;
        orc_node *n = &st->nodes[cur];
        memset(n, 0, sizeof(*n));
        n->num_parts = np;
        for (size_t i = 0; i < np; ++i) n->particles[i] = idx[start + i];
        return cur;
    }
    double m, cm[3], size;
    uint64_t sd;
    scan_segment(idx + start, np, P, &m, cm, &sd, &size);
    size_t mid = (start + end) / 2;
    quickstat_keys(idx + start, np, mid - start, &P[0].p[sd], sizeof(orc_particle) / 8,
                   &st->rng);
    double split_val = P[idx[mid]].p[sd];
    size_t left = build_dfs(idx, start, mid, P, cur + 1, st);
    size_t right = build_dfs(idx, mid, end, P, left + 1, st);
    if (!ensure_cap(st, cur)) return right;
    orc_node *n = &st->nodes[cur];
    memset(n, 0, sizeof(*n));
    n->split_dim = sd;
    n->split_val = split_val;
    n->m = m;
    n->cm[0] = cm[0]; n->cm[1] = cm[1]; n->cm[2] = cm[2];
    n->size = size;
    n->left = cur + 1;
    n->right = left + 1;
    return right;
}

/* Returns the last node index, or (uint64_t)-1 when `cap` slots were not enough. */
uint64_t orc_build_tree_dfs(uint64_t *idx, size_t n, const orc_particle *P, orc_node *nodes,
                            size_t cap, int leaf, uint64_t seed) {
    dfs_state st = {nodes, cap, leaf, 0, {seed}};
    size_t last = build_dfs(idx, 0, n, P, 0, &st);
    return st.overflow ? (uint64_t)-1 : (uint64_t)last;
}

typedef struct {
    int leaf;
    int max_threads;
    volatile int overflow;
} par4_cfg;

/* build_tree_par4, Parallel/RustVersion/src/array_kd_tree.rs:515-583.  `nodes`/`cap` is
 * the slice handed to this subtree; the left subtree gets nodes_needed(len/2) slots and the
 * right subtree whatever remains (:566-569).  rayon::join becomes an OpenMP task pair while
 * thread_cnt < the thread count (:571-578). */
static void build_par4(uint64_t *idx, size_t np, size_t cur, const orc_particle *P,
                       orc_node *nodes, size_t cap, size_t thread_cnt, par4_cfg *cfg,
                       uint64_t seed) {
    if (cap < 1) { cfg->overflow = 1; return; }
    if (np <= (size_t)cfg->leaf) {
        orc_node *n = &nodes[0];
        memset(n, 0, sizeof(*n));
        n->num_parts = np;
        for (size_t i = 0; i < np; ++i) n->particles[i] = idx[i];
        return;
    }
    double m, cm[3], size;
    uint64_t sd;
    scan_segment(idx, np, P, &m, cm, &sd, &size);
    size_t mid = np / 2;
    orc_rng rng = {seed};
    quickstat_keys(idx, np, mid, &P[0].p[sd], sizeof(orc_particle) / 8, &rng);
    double split_val = P[idx[mid]].p[sd];
    size_t num_nodes = (size_t)orc_nodes_needed_par(mid, cfg->leaf);
    if (1 + num_nodes > cap) { cfg->overflow = 1; return; }
    uint64_t sl = rng_next(&rng), sr = rng_next(&rng);
    if ((int)thread_cnt < cfg->max_threads) {
#pragma omp task shared(cfg)
        build_par4(idx, mid, cur + 1, P, nodes + 1, num_nodes, thread_cnt * 2, cfg, sl);
#pragma omp task shared(cfg)
        build_par4(idx + mid, np - mid, cur + 1 + num_nodes, P, nodes + 1 + num_nodes,
                   cap - 1 - num_nodes, thread_cnt * 2, cfg, sr);
#pragma omp taskwait
    } else {
        build_par4(idx, mid, cur + 1, P, nodes + 1, num_nodes, thread_cnt * 2, cfg, sl);
        build_par4(idx + mid, np - mid, cur + 1 + num_nodes, P, nodes + 1 + num_nodes,
                   cap - 1 - num_nodes, thread_cnt * 2, cfg, sr);
    }
    orc_node *n = &nodes[0];
    memset(n, 0, sizeof(*n));
    n->split_dim = sd;
    n->split_val = split_val;
    n->m = m;
    n->cm[0] = cm[0]; n->cm[1] = cm[1]; n->cm[2] = cm[2];
    n->size = size;
    n->left = cur + 1;
    n->right = cur + 1 + num_nodes;
}

static int max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Returns 0, or -1 when the node slice overflowed (the Rust code would panic). Unused slots
 * are left as empty leaves, as allocate_node_vec leaves them (array_kd_tree.rs:55-60). */
int orc_build_tree_par4(uint64_t *idx, size_t n, const orc_particle *P, orc_node *nodes,
                        size_t cap, int leaf, uint64_t seed) {
    par4_cfg cfg = {leaf, max_threads(), 0};
    memset(nodes, 0, cap * sizeof(orc_node));
#pragma omp parallel
#pragma omp single
    build_par4(idx, n, 0, P, nodes, cap, 1, &cfg, seed);
    return cfg.overflow ? -1 : 0;
}

/* ---------------------------------------------------------------- walk */

/* calc_pp_accel, array_particle.rs:67-76 */
static inline void pp_accel(const orc_particle *pi, const orc_particle *pj, double a[3]) {
    double dx = pi->p[0] - pj->p[0];
    double dy = pi->p[1] - pj->p[1];
    double dz = pi->p[2] - pj->p[2];
    double dp2 = dx * dx + dy * dy + dz * dz;
    double dist = sqrt(dp2);
    double magi = -pj->m / (dist * dist * dist);
    a[0] = magi * dx;
    a[1] = magi * dy;
    a[2] = magi * dz;
}

typedef struct {
    uint64_t p2p, opened, m2p, visits;
} orc_counts;

/* accel_recur, Parallel/RustVersion/src/array_kd_tree.rs:585-617: sequential sum inside a
 * leaf with self-exclusion by index, opening test size^2 < theta^2 |d|^2 (strict), and the
 * binary-tree sum left + right. */
static void accel_recur(size_t cur, size_t p, const orc_particle *P, const orc_node *nodes,
                        double theta2, double out[3], orc_counts *c, double *absum) {
    const orc_node *n = &nodes[cur];
    if (c) c->visits++;
    if (n->num_parts > 0) {
        double acc[3] = {0.0, 0.0, 0.0};
        for (uint64_t i = 0; i < n->num_parts; ++i) {
            if (n->particles[i] != p) {
                double pa[3];
                pp_accel(&P[p], &P[n->particles[i]], pa);
                if (absum) *absum += sqrt(pa[0] * pa[0] + pa[1] * pa[1] + pa[2] * pa[2]);
                acc[0] += pa[0];
                acc[1] += pa[1];
                acc[2] += pa[2];
                if (c) c->p2p++;
            }
        }
        out[0] = acc[0]; out[1] = acc[1]; out[2] = acc[2];
        return;
    }
    double dx = P[p].p[0] - n->cm[0];
    double dy = P[p].p[1] - n->cm[1];
    double dz = P[p].p[2] - n->cm[2];
    double dist_sqr = dx * dx + dy * dy + dz * dz;
    if (c) c->opened++;
    if (n->size * n->size < theta2 * dist_sqr) {
        double dist = sqrt(dist_sqr);
        double magi = -n->m / (dist_sqr * dist);
        out[0] = dx * magi; out[1] = dy * magi; out[2] = dz * magi;
        if (absum) *absum += sqrt(out[0] * out[0] + out[1] * out[1] + out[2] * out[2]);
        if (c) c->m2p++;
    } else {
        double l[3], r[3];
        accel_recur(n->left, p, P, nodes, theta2, l, c, absum);
        accel_recur(n->right, p, P, nodes, theta2, r, c, absum);
        out[0] = l[0] + r[0]; out[1] = l[1] + r[1]; out[2] = l[2] + r[2];
    }
}

/* calc_accel (array_kd_tree.rs:619-621) for every body, parallel over sinks like the
 * par_iter_mut of :647.  `theta` is THETA (:15); THETA*THETA is formed first (:606). */
void orc_calc_accel_all(const orc_particle *P, size_t n, const orc_node *nodes, double theta,
                        double *acc) {
    double theta2 = theta * theta;
#pragma omp parallel for schedule(dynamic, 256)
    for (size_t i = 0; i < n; ++i) accel_recur(0, i, P, nodes, theta2, &acc[3 * i], NULL, NULL);
}

/* Same walk, also returning per body the sum of the magnitudes of its interaction terms:
 * the scale that bounds the rounding error of any summation order of those terms. */
void orc_calc_accel_abs(const orc_particle *P, size_t n, const orc_node *nodes, double theta,
                        double *acc, double *absum) {
    double theta2 = theta * theta;
#pragma omp parallel for schedule(dynamic, 256)
    for (size_t i = 0; i < n; ++i) {
        absum[i] = 0.0;
        accel_recur(0, i, P, nodes, theta2, &acc[3 * i], NULL, &absum[i]);
    }
}

/* The walk for a list of sinks only (acc[3k..] and absum[k] for sinks[k]): the per-step
 * sampled checks of large runs, where walking every body each step would take minutes. */
void orc_calc_accel_sinks(const orc_particle *P, const orc_node *nodes, double theta,
                          const uint64_t *sinks, size_t ns, double *acc, double *absum) {
    double theta2 = theta * theta;
#pragma omp parallel for schedule(dynamic, 16)
    for (size_t k = 0; k < ns; ++k) {
        absum[k] = 0.0;
        accel_recur(0, (size_t)sinks[k], P, nodes, theta2, &acc[3 * k], NULL, &absum[k]);
    }
}

/* Instrumented walk over a list of sinks: interaction counts per the reference's walk. */
void orc_walk_counts(const orc_particle *P, const orc_node *nodes, double theta,
                     const uint64_t *sinks, size_t ns, uint64_t out[4]) {
    double theta2 = theta * theta;
    uint64_t p2p = 0, opened = 0, m2p = 0, visits = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : p2p, opened, m2p, visits)
    for (size_t k = 0; k < ns; ++k) {
        double a[3];
        orc_counts c = {0, 0, 0, 0};
        accel_recur(0, (size_t)sinks[k], P, nodes, theta2, a, &c, NULL);
        p2p += c.p2p; opened += c.opened; m2p += c.m2p; visits += c.visits;
    }
    out[0] = p2p; out[1] = opened; out[2] = m2p; out[3] = visits;
}

/* ---------------------------------------------------------------- grouped walk */

/* The sink groups of the GPU's grouped mixed walk: whole leaves in depth-first order
 * (left before right), packed greedily up to ORC_GROUP_MAX bodies.  A node is accepted for a whole
 * group when size^2 < theta^2 dmin^2, dmin the distance from the node's centre of mass to
 * the nearer of the group's two bounding boxes (Barnes 1990, J. Comput. Phys. 87:161); leaves
 * reached are summed pairwise, self excluded by index.  Everything in FP64, each sink's
 * terms added in traversal order. */
#define ORC_GROUP_MAX 64

static size_t dfs_leaves(const orc_node *nodes, size_t cur, size_t *out, size_t k) {
    if (nodes[cur].num_parts > 0) {
        out[k] = cur;
        return k + 1;
    }
    k = dfs_leaves(nodes, nodes[cur].left, out, k);
    return dfs_leaves(nodes, nodes[cur].right, out, k);
}

/* Squared distance from c to the box [lo, hi] (infinite for an empty box, lo > hi). */
static double box_dist2(const double c[3], const double lo[3], const double hi[3]) {
    if (lo[0] > hi[0]) return INFINITY;
    double e2 = 0.0;
    for (int d = 0; d < 3; ++d) {
        double e = lo[d] - c[d];
        if (c[d] - hi[d] > e) e = c[d] - hi[d];
        if (e > 0.0) e2 += e * e;
    }
    return e2;
}

static void group_recur(size_t cur, const orc_particle *P, const orc_node *nodes,
                        const uint64_t *sinks, size_t ns, const double lo[2][3],
                        const double hi[2][3], double theta2, double *acc, orc_counts *c) {
    const orc_node *nd = &nodes[cur];
    c->visits++;
    if (nd->num_parts > 0) {
        for (size_t k = 0; k < ns; ++k)
            for (uint64_t i = 0; i < nd->num_parts; ++i) {
                if (nd->particles[i] == sinks[k]) continue;
                double pa[3];
                pp_accel(&P[sinks[k]], &P[nd->particles[i]], pa);
                acc[3 * k] += pa[0];
                acc[3 * k + 1] += pa[1];
                acc[3 * k + 2] += pa[2];
                c->p2p++;
            }
        return;
    }
    double e2 = box_dist2(nd->cm, lo[0], hi[0]);
    const double f2 = box_dist2(nd->cm, lo[1], hi[1]);
    if (f2 < e2) e2 = f2;
    if (nd->size * nd->size < theta2 * e2) {
        for (size_t k = 0; k < ns; ++k) {
            const double *p = P[sinks[k]].p;
            double dx = p[0] - nd->cm[0], dy = p[1] - nd->cm[1], dz = p[2] - nd->cm[2];
            double dist_sqr = dx * dx + dy * dy + dz * dz;
            double dist = sqrt(dist_sqr);
            double magi = -nd->m / (dist_sqr * dist);
            acc[3 * k] += dx * magi;
            acc[3 * k + 1] += dy * magi;
            acc[3 * k + 2] += dz * magi;
            c->m2p++;
        }
        return;
    }
    c->opened++;
    group_recur(nd->left, P, nodes, sinks, ns, lo, hi, theta2, acc, c);
    group_recur(nd->right, P, nodes, sinks, ns, lo, hi, theta2, acc, c);
}

/* The group's bodies are boxed in two parts, split where the deepest node holding the whole
 * group splits (a node of c bodies at depth-first position st splits at st + c/2); the test
 * uses the nearer box. */
static size_t group_split(const orc_node *nodes, size_t n, size_t g0, size_t g1) {
    size_t cur = 0, st = 0, cn = n;
    while (nodes[cur].num_parts == 0) {
        const size_t mid = st + cn / 2;
        if (g1 <= mid) {
            cn = cn / 2;
            cur = nodes[cur].left;
        } else if (g0 >= mid) {
            st = mid;
            cn = cn - cn / 2;
            cur = nodes[cur].right;
        } else {
            return mid;
        }
    }
    return g1;
}

/* Groups of the tree: first body of every group in depth-first body order (`order`, n
 * entries) and group offsets (`gstart`, n_groups + 1).  Returns n_groups. */
static size_t make_groups(const orc_node *nodes, size_t n_nodes, uint64_t *order,
                          size_t *gstart) {
    size_t *lv = (size_t *)malloc(sizeof(size_t) * (n_nodes + 1));
    size_t nl = dfs_leaves(nodes, 0, lv, 0), pos = 0, ng = 0, fill = ORC_GROUP_MAX;
    for (size_t k = 0; k < nl; ++k) {
        const orc_node *nd = &nodes[lv[k]];
        if (fill + nd->num_parts > ORC_GROUP_MAX) {
            gstart[ng++] = pos;
            fill = 0;
        }
        for (uint64_t i = 0; i < nd->num_parts; ++i) order[pos++] = nd->particles[i];
        fill += nd->num_parts;
    }
    gstart[ng] = pos;
    free(lv);
    return ng;
}

/* The groups of make_groups and their split positions, for the tests: gstart (ng + 1
 * entries, depth-first body positions) and gsplit (ng entries, group_split).  Returns ng,
 * or (size_t)-1 when cap < ng + 1 or on allocation failure. */
size_t orc_groups(const orc_node *nodes, size_t n_nodes, size_t n, size_t *gstart_out,
                  size_t *gsplit_out, size_t cap) {
    uint64_t *order = (uint64_t *)malloc(sizeof(uint64_t) * (n ? n : 1));
    size_t *gs = (size_t *)malloc(sizeof(size_t) * (n + 1));
    size_t ng = (size_t)-1;
    if (order && gs) {
        ng = make_groups(nodes, n_nodes, order, gs);
        if (ng + 1 > cap) {
            ng = (size_t)-1;
        } else {
            for (size_t g = 0; g < ng; ++g) {
                gstart_out[g] = gs[g];
                gsplit_out[g] = group_split(nodes, n, gs[g], gs[g + 1]);
            }
            gstart_out[ng] = gs[ng];
        }
    }
    free(order);
    free(gs);
    return ng;
}

/* acc (n*3, original body order); counts: p2p and m2p per sink, node tests per group,
 * internal nodes opened per group. */
int orc_calc_accel_group(const orc_particle *P, size_t n, const orc_node *nodes, size_t n_nodes,
                         double theta, double *acc, uint64_t counts[4]) {
    uint64_t *order = (uint64_t *)malloc(sizeof(uint64_t) * n);
    size_t *gstart = (size_t *)malloc(sizeof(size_t) * (n + 1));
    if (!order || !gstart) {
        free(order);
        free(gstart);
        return -1;
    }
    const size_t ng = make_groups(nodes, n_nodes, order, gstart);
    const double theta2 = theta * theta;
    uint64_t p2p = 0, m2p = 0, tests = 0, opened = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : p2p, m2p, tests, opened)
    for (size_t g = 0; g < ng; ++g) {
        const uint64_t *sk = order + gstart[g];
        const size_t ns = gstart[g + 1] - gstart[g];
        const size_t sp = group_split(nodes, n, gstart[g], gstart[g + 1]) - gstart[g];
        double lo[2][3], hi[2][3], a[3 * ORC_GROUP_MAX];
        for (int h = 0; h < 2; ++h)
            for (int d = 0; d < 3; ++d) {
                lo[h][d] = INFINITY;
                hi[h][d] = -INFINITY;
            }
        for (size_t k = 0; k < ns; ++k) {
            const int h = k < sp ? 0 : 1;
            for (int d = 0; d < 3; ++d) {
                if (P[sk[k]].p[d] < lo[h][d]) lo[h][d] = P[sk[k]].p[d];
                if (P[sk[k]].p[d] > hi[h][d]) hi[h][d] = P[sk[k]].p[d];
            }
        }
        for (size_t k = 0; k < 3 * ns; ++k) a[k] = 0.0;
        orc_counts c = {0, 0, 0, 0};
        group_recur(0, P, nodes, sk, ns, lo, hi, theta2, a, &c);
        for (size_t k = 0; k < ns; ++k)
            for (int d = 0; d < 3; ++d) acc[3 * sk[k] + d] = a[3 * k + d];
        p2p += c.p2p;
        m2p += c.m2p;
        tests += c.visits;
        opened += c.opened;
    }
    if (counts) {
        counts[0] = p2p;
        counts[1] = tests;
        counts[2] = m2p;
        counts[3] = opened;
    }
    free(order);
    free(gstart);
    return 0;
}

/* ---------------------------------------------------------------- step loop */

/* simple_sim, Parallel/RustVersion/src/array_kd_tree.rs:623-664 (layout 1 = build_tree_par4)
 * and Sequential/RustVersion/src/array_kd_tree.rs:178-218 (layout 0 = DFS build_tree):
 * reset indices, build, accel for every body, then v += dt*a; p += dt*v.
 * `acc_trace`, when not NULL, receives every step's accelerations (steps*n*3). */
int orc_simple_sim(orc_particle *P, size_t n, double dt, int64_t steps, int leaf, int layout,
                   double theta, uint64_t seed, double *acc_trace) {
    size_t cap = layout == 1 ? (size_t)orc_nodes_needed_par(n, leaf) : 2 * n + 2;
    orc_node *nodes = (orc_node *)calloc(cap, sizeof(orc_node));
    uint64_t *idx = (uint64_t *)malloc(n * sizeof(uint64_t));
    double *acc = (double *)calloc(3 * n, sizeof(double));
    if (!nodes || !idx || !acc) { free(nodes); free(idx); free(acc); return -2; }
    int rc = 0;
    for (int64_t step = 0; step < steps; ++step) {
        for (size_t i = 0; i < n; ++i) idx[i] = i;
        uint64_t s = seed + 0x51ED27ULL * (uint64_t)step;
        if (layout == 1) {
            if (orc_build_tree_par4(idx, n, P, nodes, cap, leaf, s) != 0) { rc = -1; break; }
        } else {
            if (orc_build_tree_dfs(idx, n, P, nodes, cap, leaf, s) == (uint64_t)-1) { rc = -1; break; }
        }
        orc_calc_accel_all(P, n, nodes, theta, acc);
        if (acc_trace) memcpy(acc_trace + (size_t)step * 3 * n, acc, 3 * n * sizeof(double));
#pragma omp parallel for schedule(static)
        for (size_t i = 0; i < n; ++i) {
            orc_particle *b = &P[i];
            double *a = &acc[3 * i];
            b->v[0] += dt * a[0];
            b->v[1] += dt * a[1];
            b->v[2] += dt * a[2];
            double dx = dt * b->v[0];
            double dy = dt * b->v[1];
            double dz = dt * b->v[2];
            b->p[0] += dx;
            b->p[1] += dy;
            b->p[2] += dz;
            a[0] = 0.0; a[1] = 0.0; a[2] = 0.0;
        }
    }
    free(nodes); free(idx); free(acc);
    return rc;
}

/* One timing sample of a simple_sim step (array_kd_tree.rs:640-662) on all host threads:
 * the whole PAR4 build, the walk for the `ns` listed sinks only, and the kick-drift of every
 * body (the bodies that were not walked keep a zero acceleration and only drift).  t[0..2]
 * receive the wall seconds of the three parts; the caller scales the walk by n / ns.  Returns
 * 0, -1 when the node slice overflowed, -2 when out of memory. */
int orc_sampled_step(orc_particle *P, size_t n, double dt, int leaf, double theta,
                     uint64_t seed, const uint64_t *sinks, size_t ns, double t[3]) {
    size_t cap = (size_t)orc_nodes_needed_par(n, leaf);
    orc_node *nodes = (orc_node *)malloc(cap * sizeof(orc_node));
    uint64_t *idx = (uint64_t *)malloc(n * sizeof(uint64_t));
    double *acc = (double *)calloc(3 * n, sizeof(double));
    double *sa = (double *)malloc(3 * (ns ? ns : 1) * sizeof(double));
    if (!nodes || !idx || !acc || !sa) { free(nodes); free(idx); free(acc); free(sa); return -2; }
    double theta2 = theta * theta;
    double t0 = omp_get_wtime();
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < n; ++i) idx[i] = i;
    int rc = orc_build_tree_par4(idx, n, P, nodes, cap, leaf, seed);
    double t1 = omp_get_wtime();
#pragma omp parallel for schedule(dynamic, 16)
    for (size_t k = 0; k < ns; ++k)
        accel_recur(0, (size_t)sinks[k], P, nodes, theta2, &sa[3 * k], NULL, NULL);
    double t2 = omp_get_wtime();
    for (size_t k = 0; k < ns; ++k) memcpy(&acc[3 * (size_t)sinks[k]], &sa[3 * k], 24);
    double t3 = omp_get_wtime();
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < n; ++i) {
        orc_particle *b = &P[i];
        double *a = &acc[3 * i];
        b->v[0] += dt * a[0];
        b->v[1] += dt * a[1];
        b->v[2] += dt * a[2];
        b->p[0] += dt * b->v[0];
        b->p[1] += dt * b->v[1];
        b->p[2] += dt * b->v[2];
        a[0] = 0.0; a[1] = 0.0; a[2] = 0.0;
    }
    double t4 = omp_get_wtime();
    t[0] = t1 - t0;
    t[1] = t2 - t1;
    t[2] = t4 - t3;
    free(nodes); free(idx); free(acc); free(sa);
    return rc;
}

/* ---------------------------------------------------------------- direct sum */

/* FP64 direct sum for a set of sinks: one-sided form of the all-pairs kernel of
 * Sequential/RustVersion/src/simd_particle.rs:95-103, each pair evaluated like
 * calc_pp_accel (array_particle.rs:67-76).  Summed in source order. */
void orc_direct_accel(const orc_particle *P, size_t n, const uint64_t *sinks, size_t ns,
                      double *acc) {
#pragma omp parallel for schedule(dynamic, 4)
    for (size_t k = 0; k < ns; ++k) {
        size_t i = (size_t)sinks[k];
        double a0 = 0.0, a1 = 0.0, a2 = 0.0;
        for (size_t j = 0; j < n; ++j) {
            if (j == i) continue;
            double pa[3];
            pp_accel(&P[i], &P[j], pa);
            a0 += pa[0]; a1 += pa[1]; a2 += pa[2];
        }
        acc[3 * k] = a0; acc[3 * k + 1] = a1; acc[3 * k + 2] = a2;
    }
}

/* The same direct sum, also returning per sink the sum of the magnitudes of its terms (the
 * scale of the rounding error of any other summation order of the same terms). */
void orc_direct_accel_abs(const orc_particle *P, size_t n, const uint64_t *sinks, size_t ns,
                          double *acc, double *absum) {
#pragma omp parallel for schedule(dynamic, 4)
    for (size_t k = 0; k < ns; ++k) {
        size_t i = (size_t)sinks[k];
        double a0 = 0.0, a1 = 0.0, a2 = 0.0, s = 0.0;
        for (size_t j = 0; j < n; ++j) {
            if (j == i) continue;
            double pa[3];
            pp_accel(&P[i], &P[j], pa);
            a0 += pa[0]; a1 += pa[1]; a2 += pa[2];
            s += sqrt(pa[0] * pa[0] + pa[1] * pa[1] + pa[2] * pa[2]);
        }
        acc[3 * k] = a0; acc[3 * k + 1] = a1; acc[3 * k + 2] = a2;
        absum[k] = s;
    }
}

/* Direct-sum potential energy sum_{i<j} -m_i m_j / r_ij and kinetic energy (small N). */
void orc_energy(const orc_particle *P, size_t n, double out[2]) {
    double pe = 0.0, ke = 0.0;
#pragma omp parallel for reduction(+ : pe, ke) schedule(dynamic, 16)
    for (size_t i = 0; i < n; ++i) {
        const orc_particle *a = &P[i];
        ke += 0.5 * a->m * (a->v[0] * a->v[0] + a->v[1] * a->v[1] + a->v[2] * a->v[2]);
        for (size_t j = i + 1; j < n; ++j) {
            double dx = a->p[0] - P[j].p[0], dy = a->p[1] - P[j].p[1], dz = a->p[2] - P[j].p[2];
            pe -= a->m * P[j].m / sqrt(dx * dx + dy * dy + dz * dz);
        }
    }
    out[0] = ke;
    out[1] = pe;
}

/* ---------------------------------------------------------------- direct-sum adjoint */

/* Unit tidal product w = |d|^-3 (mu - 3 (d.mu) |d|^-2 d), d = xi - xj. */
static inline void tidal_w(const double d[3], const double mu[3], double w[3]) {
    double d2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    double inv2 = 1.0 / d2;
    double inv3 = inv2 / sqrt(d2);
    double dm = d[0] * mu[0] + d[1] * mu[1] + d[2] * mu[2];
    double c3 = 3.0 * dm * inv2;
    for (int k = 0; k < 3; ++k) w[k] = inv3 * (mu[k] - c3 * d[k]);
}

/* Direct-sum accelerations of all n bodies from positions x (3n), FP64. */
static void direct_all(const double *x, const double *m, size_t n, double *a) {
#pragma omp parallel for schedule(dynamic, 16)
    for (size_t i = 0; i < n; ++i) {
        double ax = 0, ay = 0, az = 0;
        for (size_t j = 0; j < n; ++j) {
            if (j == i) continue;
            double dx = x[3 * i] - x[3 * j], dy = x[3 * i + 1] - x[3 * j + 1],
                   dz = x[3 * i + 2] - x[3 * j + 2];
            double dp2 = dx * dx + dy * dy + dz * dz;
            double dist = sqrt(dp2);
            double magi = -m[j] / (dist * dist * dist);
            ax += magi * dx; ay += magi * dy; az += magi * dz;
        }
        a[3 * i] = ax; a[3 * i + 1] = ay; a[3 * i + 2] = az;
    }
}

/* FP64 direct-sum forward (semi-implicit Euler of array_kd_tree.rs:649-658 with all-pairs
 * forces) for `steps` steps, then the exact reverse sweep:
 *   mu = lv + dt lx;  lv = mu;  lx += dt J^T mu,
 *   (J^T mu)_i = sum_{j != i} [ -m_j w(x_i - x_j, mu_i) + m_i w(x_j - x_i, mu_j) ].
 * dL_dx / dL_dv: gradient at the final state (3n each; dL_dv may be NULL).  When
 * `loss_target` is not NULL, dL_dx is ignored and the loss (1/n) sum |x_T - target|^2 is
 * used instead; its value is stored in *loss.  Outputs the gradients at the initial state
 * and the final positions x_T (3n). */
int orc_adjoint_direct(const orc_particle *P, size_t n, double dt, int64_t steps,
                       const double *dL_dx, const double *dL_dv, const double *loss_target,
                       double *loss, double *g_x0, double *g_v0, double *xT) {
    double *xs = (double *)malloc((size_t)(steps + 1) * 3 * n * sizeof(double));
    double *v = (double *)malloc(3 * n * sizeof(double));
    double *m = (double *)malloc(n * sizeof(double));
    double *a = (double *)malloc(3 * n * sizeof(double));
    double *lx = (double *)malloc(3 * n * sizeof(double));
    double *lv = (double *)malloc(3 * n * sizeof(double));
    double *mu = (double *)malloc(3 * n * sizeof(double));
    double *y = (double *)malloc(3 * n * sizeof(double));
    if (!xs || !v || !m || !a || !lx || !lv || !mu || !y) {
        free(xs); free(v); free(m); free(a); free(lx); free(lv); free(mu); free(y);
        return -2;
    }
    for (size_t i = 0; i < n; ++i) {
        for (int k = 0; k < 3; ++k) { xs[3 * i + k] = P[i].p[k]; v[3 * i + k] = P[i].v[k]; }
        m[i] = P[i].m;
    }
    for (int64_t s = 0; s < steps; ++s) {
        double *x0 = xs + (size_t)s * 3 * n, *x1 = x0 + 3 * n;
        direct_all(x0, m, n, a);
        for (size_t k = 0; k < 3 * n; ++k) {
            v[k] += dt * a[k];
            x1[k] = x0[k] + dt * v[k];
        }
    }
    double *xe = xs + (size_t)steps * 3 * n;
    memcpy(xT, xe, 3 * n * sizeof(double));
    if (loss_target) {
        double L = 0.0;
        for (size_t k = 0; k < 3 * n; ++k) {
            double e = xe[k] - loss_target[k];
            L += e * e;
            lx[k] = 2.0 * e / (double)n;
        }
        *loss = L / (double)n;
    } else {
        memcpy(lx, dL_dx, 3 * n * sizeof(double));
    }
    if (dL_dv) memcpy(lv, dL_dv, 3 * n * sizeof(double));
    else memset(lv, 0, 3 * n * sizeof(double));
    for (int64_t s = steps - 1; s >= 0; --s) {
        const double *x = xs + (size_t)s * 3 * n;
        for (size_t k = 0; k < 3 * n; ++k) mu[k] = lv[k] + dt * lx[k];
#pragma omp parallel for schedule(dynamic, 16)
        for (size_t i = 0; i < n; ++i) {
            double yi[3] = {0, 0, 0};
            for (size_t j = 0; j < n; ++j) {
                if (j == i) continue;
                double d[3] = {x[3 * i] - x[3 * j], x[3 * i + 1] - x[3 * j + 1],
                               x[3 * i + 2] - x[3 * j + 2]};
                double w[3], e[3] = {-d[0], -d[1], -d[2]};
                tidal_w(d, &mu[3 * i], w);
                for (int k = 0; k < 3; ++k) yi[k] -= m[j] * w[k];
                tidal_w(e, &mu[3 * j], w);
                for (int k = 0; k < 3; ++k) yi[k] += m[i] * w[k];
            }
            for (int k = 0; k < 3; ++k) y[3 * i + k] = yi[k];
        }
        for (size_t k = 0; k < 3 * n; ++k) {
            lx[k] += dt * y[k];
            lv[k] = mu[k];
        }
    }
    memcpy(g_x0, lx, 3 * n * sizeof(double));
    memcpy(g_v0, lv, 3 * n * sizeof(double));
    free(xs); free(v); free(m); free(a); free(lx); free(lv); free(mu); free(y);
    return 0;
}

/* Transpose Jacobian product of one Barnes-Hut evaluation, y = J^T mu, over the interaction
 * set of accel_recur (array_kd_tree.rs:585-617): for every sink i and interaction with a
 * source of mass m at c, w = w(x_i - c, mu_i):  y_i -= m w;  a pair source j gets m_j w; a
 * node K passes w down to each of its bodies l as m_l w. */
static void jt_recur(size_t cur, size_t p, const orc_particle *P, const orc_node *nodes,
                     double theta2, const double *mu, double *ys, double *y, double *Gn) {
    const orc_node *n = &nodes[cur];
    if (n->num_parts > 0) {
        for (uint64_t k = 0; k < n->num_parts; ++k) {
            size_t j = (size_t)n->particles[k];
            if (j == p) continue;
            double d[3] = {P[p].p[0] - P[j].p[0], P[p].p[1] - P[j].p[1], P[p].p[2] - P[j].p[2]};
            double w[3];
            tidal_w(d, &mu[3 * p], w);
            for (int q = 0; q < 3; ++q) {
                ys[q] -= P[j].m * w[q];
#pragma omp atomic
                y[3 * j + q] += P[j].m * w[q];
            }
        }
        return;
    }
    double d[3] = {P[p].p[0] - n->cm[0], P[p].p[1] - n->cm[1], P[p].p[2] - n->cm[2]};
    double d2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    if (n->size * n->size < theta2 * d2) {
        double w[3];
        tidal_w(d, &mu[3 * p], w);
        for (int q = 0; q < 3; ++q) {
            ys[q] -= n->m * w[q];
#pragma omp atomic
            Gn[3 * cur + q] += w[q];
        }
    } else {
        jt_recur(n->left, p, P, nodes, theta2, mu, ys, y, Gn);
        jt_recur(n->right, p, P, nodes, theta2, mu, ys, y, Gn);
    }
}

static void jt_down(size_t cur, const orc_particle *P, const orc_node *nodes, const double *Gn,
                    double acc0, double acc1, double acc2, double *y) {
    const orc_node *n = &nodes[cur];
    if (n->num_parts > 0) {
        for (uint64_t k = 0; k < n->num_parts; ++k) {
            size_t l = (size_t)n->particles[k];
            y[3 * l] += P[l].m * acc0;
            y[3 * l + 1] += P[l].m * acc1;
            y[3 * l + 2] += P[l].m * acc2;
        }
        return;
    }
    acc0 += Gn[3 * cur]; acc1 += Gn[3 * cur + 1]; acc2 += Gn[3 * cur + 2];
    jt_down(n->left, P, nodes, Gn, acc0, acc1, acc2, y);
    jt_down(n->right, P, nodes, Gn, acc0, acc1, acc2, y);
}

int orc_tree_jt(const orc_particle *P, size_t n, const orc_node *nodes, size_t n_nodes,
                double theta, const double *mu, double *y) {
    double *Gn = (double *)calloc(3 * n_nodes, sizeof(double));
    if (!Gn) return -2;
    memset(y, 0, 3 * n * sizeof(double));
    double theta2 = theta * theta;
#pragma omp parallel for schedule(dynamic, 64)
    for (size_t i = 0; i < n; ++i) {
        double ys[3] = {0.0, 0.0, 0.0};
        jt_recur(0, i, P, nodes, theta2, mu, ys, y, Gn);
        for (int q = 0; q < 3; ++q) {
#pragma omp atomic
            y[3 * i + q] += ys[q];
        }
    }
    jt_down(0, P, nodes, Gn, 0.0, 0.0, 0.0, y);
    free(Gn);
    return 0;
}

/* J^T mu over the grouped interaction set of the mixed path (the decisions of group_recur):
 * per sink s and source c of mass m, w = T(x_s - c) mu_s; the sink gets -m w, a pair source
 * j gets +m_j w, an accepted node's bodies get m_i w through Gn and jt_down. */
static void jt_group_recur(size_t cur, const orc_particle *P, const orc_node *nodes,
                           const uint64_t *sinks, size_t ns, const double lo[2][3],
                           const double hi[2][3], double theta2, const double *mu, double *ys,
                           double *y, double *Gn) {
    const orc_node *nd = &nodes[cur];
    if (nd->num_parts > 0) {
        for (size_t k = 0; k < ns; ++k) {
            const size_t p = (size_t)sinks[k];
            for (uint64_t i = 0; i < nd->num_parts; ++i) {
                const size_t j = (size_t)nd->particles[i];
                if (j == p) continue;
                double d[3] = {P[p].p[0] - P[j].p[0], P[p].p[1] - P[j].p[1],
                               P[p].p[2] - P[j].p[2]};
                double w[3];
                tidal_w(d, &mu[3 * p], w);
                for (int q = 0; q < 3; ++q) {
                    ys[3 * k + q] -= P[j].m * w[q];
#pragma omp atomic
                    y[3 * j + q] += P[j].m * w[q];
                }
            }
        }
        return;
    }
    double e2 = box_dist2(nd->cm, lo[0], hi[0]);
    const double f2 = box_dist2(nd->cm, lo[1], hi[1]);
    if (f2 < e2) e2 = f2;
    if (nd->size * nd->size < theta2 * e2) {
        for (size_t k = 0; k < ns; ++k) {
            const size_t p = (size_t)sinks[k];
            double d[3] = {P[p].p[0] - nd->cm[0], P[p].p[1] - nd->cm[1], P[p].p[2] - nd->cm[2]};
            double w[3];
            tidal_w(d, &mu[3 * p], w);
            for (int q = 0; q < 3; ++q) {
                ys[3 * k + q] -= nd->m * w[q];
#pragma omp atomic
                Gn[3 * cur + q] += w[q];
            }
        }
        return;
    }
    jt_group_recur(nd->left, P, nodes, sinks, ns, lo, hi, theta2, mu, ys, y, Gn);
    jt_group_recur(nd->right, P, nodes, sinks, ns, lo, hi, theta2, mu, ys, y, Gn);
}

int orc_tree_jt_group(const orc_particle *P, size_t n, const orc_node *nodes, size_t n_nodes,
                      double theta, const double *mu, double *y) {
    double *Gn = (double *)calloc(3 * n_nodes, sizeof(double));
    uint64_t *order = (uint64_t *)malloc(sizeof(uint64_t) * n);
    size_t *gstart = (size_t *)malloc(sizeof(size_t) * (n + 1));
    if (!Gn || !order || !gstart) {
        free(Gn);
        free(order);
        free(gstart);
        return -2;
    }
    memset(y, 0, 3 * n * sizeof(double));
    const size_t ng = make_groups(nodes, n_nodes, order, gstart);
    const double theta2 = theta * theta;
#pragma omp parallel for schedule(dynamic, 16)
    for (size_t g = 0; g < ng; ++g) {
        const uint64_t *sk = order + gstart[g];
        const size_t ns = gstart[g + 1] - gstart[g];
        const size_t sp = group_split(nodes, n, gstart[g], gstart[g + 1]) - gstart[g];
        double lo[2][3], hi[2][3], ys[3 * ORC_GROUP_MAX];
        for (int h = 0; h < 2; ++h)
            for (int d = 0; d < 3; ++d) {
                lo[h][d] = INFINITY;
                hi[h][d] = -INFINITY;
            }
        for (size_t k = 0; k < ns; ++k) {
            const int h = k < sp ? 0 : 1;
            for (int d = 0; d < 3; ++d) {
                if (P[sk[k]].p[d] < lo[h][d]) lo[h][d] = P[sk[k]].p[d];
                if (P[sk[k]].p[d] > hi[h][d]) hi[h][d] = P[sk[k]].p[d];
            }
        }
        for (size_t k = 0; k < 3 * ns; ++k) ys[k] = 0.0;
        jt_group_recur(0, P, nodes, sk, ns, lo, hi, theta2, mu, ys, y, Gn);
        for (size_t k = 0; k < ns; ++k)
            for (int q = 0; q < 3; ++q) {
#pragma omp atomic
                y[3 * sk[k] + q] += ys[3 * k + q];
            }
    }
    jt_down(0, P, nodes, Gn, 0.0, 0.0, 0.0, y);
    free(Gn);
    free(order);
    free(gstart);
    return 0;
}

int orc_omp_threads(void) { return max_threads(); }

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
