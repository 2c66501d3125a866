/*
 * kdnbody.h -- C ABI of libkdnbody.so, the GB300 kD-tree Barnes-Hut step.
 *
 * The reference (MarkCLewis/MultiLanguageKDTree) exposes this path as the Rust module
 * surface of Parallel/RustVersion (src/lib.rs:1-3: array_kd_tree, array_particle,
 * quickstat).  Each entry point below names the reference function it stands in for.
 * Conventions:
 *   - every call returns 0 (KD_OK) or a negative KD_E* code; nothing aborts or throws
 *     across this boundary, and kd_last_error() holds a one-line message;
 *   - the caller owns every host buffer; the library owns all device memory of a context;
 *   - one context = one CUDA stream on one device; a context is not thread-safe, a
 *     process may hold several;
 *   - body indices are 0..n-1 in the order of the array given to kd_set_bodies.
 */
#ifndef KDNBODY_H
#define KDNBODY_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KD_OK 0
#define KD_EINVAL (-1)    /* bad argument: size, leaf size, layout, NULL pointer */
#define KD_ENOMEM (-2)    /* device or host allocation failed */
#define KD_ECUDA (-3)     /* a CUDA runtime call failed */
#define KD_ESTATE (-4)    /* call out of order (no bodies yet, no tree yet, no tape) */
#define KD_ENUMERIC (-5)  /* non-finite position/velocity/mass, or a negative mass */
#define KD_EOVERFLOW (-6) /* node slots exhausted: the reference would panic here */
#define KD_EDEVICE (-7)   /* a device-side check failed (stack depth, iteration cap) */

#define KD_MAX_LEAF 8

/* Body record: Particle of Parallel/RustVersion/src/array_particle.rs:3-8 (and
 * Parallel/CVersion/src/particle.h:13-18): position, velocity, radius (unused by the
 * dynamics, carried through), mass.  64 bytes, #[repr(C)]-compatible. */
typedef struct {
    double p[3];
    double v[3];
    double r;
    double m;
} kd_particle_c;

/* Node record: the flat KDTree struct of Parallel/CVersion/src/kdtree.h:9-22, with 8 leaf
 * slots so that both reference leaf sizes (7: sequential Rust and C; 8: parallel Rust) fit.
 * A leaf has num_parts > 0 (or is an unused PAR4 slot with num_parts == 0 and left ==
 * right == 0); an internal node has num_parts == 0 and the fields of the Rust
 * KDTree::Internal variant (array_kd_tree.rs:25-33).  particles[] holds body indices. */
typedef struct {
    uint64_t num_parts;
    uint64_t particles[KD_MAX_LEAF];
    uint64_t split_dim;
    double split_val;
    double m;
    double cm[3];
    double size;
    uint64_t left;
    uint64_t right;
} kd_node_c;

/* Node numbering.  DFS: left = cur+1, right = last node of left + 1 -- build_tree of
 * array_kd_tree.rs:63-130.  PAR4: left = cur+1, right = cur+1+nodes_needed(len/2) --
 * build_tree_par4 of array_kd_tree.rs:515-583 (the one simple_sim uses, :643). */
enum { KD_LAYOUT_DFS = 0, KD_LAYOUT_PAR4 = 1 };

/* FP64: the reference's arithmetic, every interaction of every body as the Rust walk makes
 * it.  MIXED: FP32 pairwise and multipole terms on split (hi+lo) coordinates with
 * compensated sums; FP64 for storage, tree splits, kick-drift and the heavy bodies (their
 * pull on every body, and their own accelerations as direct sums over all bodies). */
enum { KD_PREC_FP64 = 0, KD_PREC_MIXED = 1 };

typedef struct {
    int32_t leaf_size;  /* MAX_PARTS: 7 (Sequential Rust, C) or 8 (Parallel Rust); 2..8 */
    int32_t layout;     /* KD_LAYOUT_* numbering reported by kd_get_nodes */
    int32_t precision;  /* KD_PREC_* */
    int32_t device;     /* CUDA device ordinal */
    double theta;       /* THETA, array_kd_tree.rs:15 (0.3) */
    double dt;          /* time step used by kd_simple_sim when its dt argument is 0 */
    double heavy_frac;  /* MIXED: bodies with m >= heavy_frac * total mass (at most 8) are
                           summed directly in FP64 (the central-mass term), and their own
                           accelerations are FP64 direct sums over all bodies; <= 0
                           disables */
    uint64_t seed;      /* reserved for generators; the build itself is deterministic */
} kd_params;

typedef struct kd_ctx kd_ctx;
typedef struct kd_tape kd_tape;

/* Per-phase device times of the last kd_simple_sim / kd_calc_accel call, milliseconds,
 * and the walk's interaction counts when counting was requested. */
typedef struct {
    double build_ms;    /* per-phase sums; filled only while kd_set_timing(ctx, 1) */
    double moments_ms;
    double walk_ms;
    double kick_ms;
    double total_ms;    /* whole call, always */
    uint64_t steps;
    uint64_t launches;  /* kernels launched by the call */
} kd_stats;

/* Fill defaults: leaf 7, DFS, FP64, device 0, theta 0.3, dt 1e-3, heavy_frac 1e-3. */
void kd_default_params(kd_params *params);

/* allocate_node_vec / nodes_needed_for_particles: number of node slots the reference
 * allocates for n bodies.  PAR4: Parallel/RustVersion/src/array_kd_tree.rs:45-60;
 * DFS: Sequential/RustVersion/src/array_kd_tree.rs:37-46 (that Vec grows on demand;
 * kd_build_tree reports the nodes actually used). */
size_t kd_nodes_needed(size_t n, int32_t leaf_size, int32_t layout);

/* The sink groups of the mixed (grouped) walk for n bodies (host computation, no device):
 * whole leaves in tree order packed greedily up to 64 bodies; gstart[0..g] = first tree
 * position of each group and n at the end, gsplit[0..g-1] = the split position of the
 * deepest node holding each group (its end for a one-leaf group).  cap is the capacity of
 * gstart (g + 1 entries needed; gsplit needs cap - 1).  *n_groups = g is set even when
 * cap < g + 1 (then KD_EINVAL, nothing is written, and kd_last_error(NULL) says why). */
int kd_group_plan(size_t n, int32_t leaf_size, uint32_t *gstart, uint32_t *gsplit, size_t cap,
                  size_t *n_groups);

/* Create a context for n bodies (1 <= n < 2^31).  Replaces the set-up half of
 * simple_sim (array_kd_tree.rs:624-630): node storage, index vector, accelerations.
 * Returns NULL on failure; kd_last_error(NULL) then says why. */
kd_ctx *kd_create(size_t n, const kd_params *params);
void kd_destroy(kd_ctx *ctx);

/* Last error message of ctx (or of the calling thread's last failed kd_create,
 * kd_group_plan, kd_quickstat_index or kd_direct_accel_noalloc when ctx is NULL).  Never
 * NULL. */
const char *kd_last_error(const kd_ctx *ctx);

/* Copy n bodies host -> device (Vec<Particle> handed to simple_sim/build_tree).  Checks
 * that every p, v, m is finite and m >= 0.  A page-locked (pinned) 16-byte-aligned array is
 * read in place by the converting kernel at the host link's rate; any other array is first
 * copied to a device staging buffer.  Returns after the bodies are on the device. */
int kd_set_bodies(kd_ctx *ctx, const kd_particle_c *bodies, size_t n);
/* Generate n bodies on the device, straight into the context (no host arrays): the
 * initial conditions of array_particle.rs without the host-to-device copy.  KD_GEN_RING: body
 * 0 of mass 1 at rest at the origin, bodies 1..n-1 of mass 1e-14 with r ~ U[0.8, 1.2],
 * phi ~ U[0, 2 pi), z ~ Normal(0, 1e-4), circular speed sqrt(1/r).  KD_GEN_PLUMMER: Plummer
 * sphere (G = M = a = 1, equal masses, radii below 20, speeds from the distribution
 * function), centre of mass at rest at the origin.  KD_GEN_CIRCULAR: circular_orbits(n-1) of
 * array_particle.rs:19-44.  Each body draws from its own counter-based stream, so the result
 * depends on (n, seed) only. */
enum { KD_GEN_RING = 0, KD_GEN_PLUMMER = 1, KD_GEN_CIRCULAR = 2 };
int kd_generate(kd_ctx *ctx, int32_t kind, uint64_t seed);

/* Copy the bodies device -> host (the &mut Vec<Particle> after simple_sim returns); a
 * page-locked 16-byte-aligned array is written in place, any other through a staging
 * buffer.  Returns after the copy is complete. */
int kd_get_bodies(kd_ctx *ctx, kd_particle_c *bodies, size_t n);

/* build_tree (array_kd_tree.rs:63-130) / build_tree_par4 (:515-583) over the current
 * bodies, on the device.  *last_node (may be NULL) receives the index of the last node
 * used in the context's layout: build_tree's return value for DFS, the highest occupied
 * slot for PAR4. */
int kd_build_tree(kd_ctx *ctx, size_t *last_node);

/* Copy the tree built by the last kd_build_tree to the host in the context's layout.
 * cap must be >= the node count (kd_nodes_needed for PAR4, last_node+1 for DFS);
 * *count receives the number of records written. */
int kd_get_nodes(kd_ctx *ctx, kd_node_c *out, size_t cap, size_t *count);

/* quickstat_index (Parallel/RustVersion/src/quickstat.rs:9-34) on the GPU, no context:
 * reorders the index vector idx[0..n) (host, values < n_vals, into vals[0..n_vals), host)
 * so that vals[idx[i]] < vals[idx[goal]] for i < goal and vals[idx[i]] >= vals[idx[goal]]
 * for i >= goal -- the post-condition of quickstat.rs:211-216.  Equal values are ordered by
 * index value (the reference's order among equal values depends on its random pivots).
 * Non-finite values and out-of-range indices are rejected (KD_ENUMERIC).  *gpu_ms (may be
 * NULL) receives the device time of the selection and partition, transfers excluded.
 * Allocates and frees its own device memory; kd_last_error(NULL) reports failures. */
int kd_quickstat_index(const double *vals, size_t n_vals, uint64_t *idx, size_t n, size_t goal,
                       int32_t device, double *gpu_ms);

/* print_tree (array_kd_tree.rs:666-692) of the last kd_build_tree, written to `path` (the
 * reference writes tree{step}.txt): the node-vector length on the first line, then in slot
 * order "L num_parts" followed by one "x y z" line per body, or
 * "I split_dim split_val left right"; numbers as Rust's `{}` prints them (shortest
 * round-trip digits, no exponent).  The length is allocate_node_vec(n) for PAR4 and the
 * grown sequential Vec for DFS, whose unused slots print as "L 0". */
int kd_print_tree(kd_ctx *ctx, const char *path);

/* calc_accel (array_kd_tree.rs:619-621) for every body at once, over the tree of the last
 * kd_build_tree: acc[3*i+d] = d-th component of the acceleration of body i. */
int kd_calc_accel(kd_ctx *ctx, double *acc);

/* simple_sim (array_kd_tree.rs:623-664): `steps` steps of build -> accel -> kick-drift
 * (v += dt*a; p += dt*v), bodies resident on the device between calls.  dt == 0 uses
 * params.dt. */
int kd_simple_sim(kd_ctx *ctx, double dt, int64_t steps);

/* Energies of the current bodies: out[0] = sum of m v^2 / 2, out[1] = sum of m phi / 2 with
 * each body's potential phi from a mixed-precision walk over a tree built for this call
 * (theta of the context; heavy bodies in FP64).  Used for energy-drift reports; the
 * reference has no energy diagnostic.  Invalidates the tree of the last kd_build_tree. */
int kd_energy(kd_ctx *ctx, double out[2]);

/* Switch the arithmetic of later walks (KD_PREC_*). */
int kd_set_precision(kd_ctx *ctx, int32_t precision);

/* Device timings of the last call. */
int kd_get_stats(const kd_ctx *ctx, kd_stats *out);

/* Record CUDA events around every phase of every step (build, moments, walk, kick) so
 * kd_get_stats reports per-phase device time.  Off by default. */
int kd_set_timing(kd_ctx *ctx, int32_t on);

/* FP64 direct sum (no tree) for a list of sink bodies over all n bodies, pair kernel of
 * array_particle.rs:67-76 -- the all-pairs form of Sequential/RustVersion/src/
 * simd_particle.rs:95-103, one-sided.  acc[3*k+d] for sinks[k].  An error yardstick for the
 * tree walks; O(ns * n). */
int kd_direct_accel(kd_ctx *ctx, const uint64_t *sinks, size_t ns, double *acc);

/* Adjoint (reverse mode) of the step loop, autograd.Function style: kd_forward runs
 * `steps` steps like kd_simple_sim (the context must use KD_PREC_MIXED) and keeps a
 * checkpoint of (x, v) every `ckpt_every` steps in device memory; kd_backward takes the
 * gradient of a loss with respect to the final positions and velocities (host, 3*n each,
 * dL_dv may be NULL for zero) and returns the gradients with respect to the initial ones
 * (host, 3*n each).  Each checkpoint segment is recomputed forward (except the last, whose
 * positions the forward sweep leaves in the context while no later sweep has replaced them),
 * then walked back step by step: mu = lv + dt*lx; lv = mu; lx += dt * J(x_n)^T mu,
 * J = da/dx over the interaction set of the forward walk (tidal tensors; node sources pushed
 * down to their bodies with weight m_i/M).  Device memory: 48 B per body per checkpoint
 * plus 24 B per body per step of one segment.  The bodies are left at the final state.  A
 * tape may be consumed by
 * several kd_backward calls; kd_tape_free releases it (before its context is destroyed).  The
 * checkpoint buffers stay with the context and are reused by later kd_forward calls once
 * their tape is freed; kd_destroy releases them.  No counterpart in the reference
 * (which has no derivatives); it differentiates simple_sim (array_kd_tree.rs:623-664). */
int kd_forward(kd_ctx *ctx, double dt, int64_t steps, int64_t ckpt_every, kd_tape **tape);
int kd_backward(kd_tape *tape, const double *dL_dx, const double *dL_dv, double *g_x0,
                double *g_v0);
void kd_tape_free(kd_tape *tape);

/* kd_direct_accel without a context and without allocating device memory, for callers that
 * cannot allocate: a host whose device memory is fully committed to its own simulation
 * state, or one that measures accuracy inside its step loop, where the device-wide
 * synchronisation of cudaMalloc/cudaFree would stall its other streams.  No counterpart in
 * the reference.  All pointers are device pointers of the current device: positions x, y,
 * z and masses m of n bodies (FP64, n < 2^31), ns sink indices, and acc (3*ns doubles,
 * acc[3k+d] for sinks[k]); an out-of-range sink index yields NaN.  Work is queued on
 * `stream` (a cudaStream_t; NULL = default stream) and not waited for.
 * Limit: ns <= 43690 -- the partial sums live in one 1 MiB __device__ array of the library
 * (131072 doubles, 3 per sink and source chunk), which every GPU that loads the library holds
 * until exit.  The sources are cut into min(ceil(n / 4096), floor(131072 / (3 ns))) chunks,
 * one grid column each, so a large ns with a large n makes one long launch on a grid of only
 * ceil(ns / 128) x (1 or 2) blocks: callers sampling accuracy inside a step loop should keep
 * ns small (a few thousand sinks give 10 or more chunks); larger ns returns KD_EINVAL and
 * kd_last_error(NULL) says why.  The first call on a device looks up that array's address
 * (cudaGetSymbolAddress) with the device current; make that first call before any stream
 * capture.  Every call overwrites all the partials it reads, so no clearing is needed, but
 * all calls share the one array: calls that overlap on the GPU (other streams, other host
 * threads) race and must be serialised by the caller. */
int kd_direct_accel_noalloc(const double *x, const double *y, const double *z,
                            const double *m, size_t n, const uint64_t *sinks, size_t ns,
                            double *acc, void *stream);

/* Device-side guards, lowered for testing the failure path: the traversal stack of both
 * walks is cut to stack_entries (at most 32 for the FP64 walk, whose stack is one entry per
 * lane; at most 32 * (tree depth + 2) + 64 for the grouped walk and its adjoint) and the
 * radix refinement passes of the block median selects (segments above 4,096 bodies, and the
 * shared-memory selects of the last two levels above the subtree finish) to select_passes
 * (at most 16).  A negative value restores the default.  A walk or select that
 * runs out stops, sets a device flag, and the call returns KD_EDEVICE ("traversal stack
 * overflow" / "median select failed to converge"); nothing traps or waits, the step's
 * kick-drift is skipped (the bodies stay at the start of the failed step), and the context
 * stays usable.  No counterpart in the reference, whose walk and quickselect panic on a
 * bad index instead. */
int kd_set_device_limits(kd_ctx *ctx, int32_t stack_entries, int32_t select_passes);

/* Measured FP32 multiply-add rate of a device, TFLOP/s (2 flops per multiply-add): out[0]
 * with scalar fma.rn.f32, out[1] with packed fma.rn.f32x2 (the form of the mixed walk's pair
 * sums); every SM busy for a few milliseconds.  A measurement helper for roofline figures,
 * with no counterpart in the reference; kd_last_error(NULL) reports failures. */
int kd_fp32_peak(int32_t device, double out[2]);

/* Interaction counts of the last walk, summed over bodies: out[0] = pair (P2P)
 * interactions, out[2] = accepted multipole (M2P) interactions.  FP64 walk: out[1] =
 * opening tests at internal nodes, out[3] = node visits, both per body.  Mixed (grouped)
 * walk: out[1] = node tests, each made once for a group of up to 64 bodies, out[3] = the
 * same tests counted once per body of the group.  Counting is enabled by
 * kd_set_counting(ctx, 1) (it costs a few percent). */
int kd_set_counting(kd_ctx *ctx, int32_t on);
int kd_get_counts(const kd_ctx *ctx, uint64_t out[4]);

#ifdef __cplusplus
}
#endif

#endif /* KDNBODY_H */
