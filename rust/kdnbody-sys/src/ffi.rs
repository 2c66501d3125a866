//! Raw declarations of include/kdnbody.h, the C ABI of libkdnbody.so.  Every type is
//! `#[repr(C)]` with the header's field order; every function returns 0 (KD_OK) or a negative
//! KD_E* status, except the few the header declares otherwise.  Safe wrappers live in the
//! other modules of the crate.
#![allow(non_camel_case_types)]

use std::os::raw::{c_char, c_int, c_void};

pub const KD_OK: c_int = 0;
pub const KD_EINVAL: c_int = -1;
pub const KD_ENOMEM: c_int = -2;
pub const KD_ECUDA: c_int = -3;
pub const KD_ESTATE: c_int = -4;
pub const KD_ENUMERIC: c_int = -5;
pub const KD_EOVERFLOW: c_int = -6;
pub const KD_EDEVICE: c_int = -7;

pub const KD_MAX_LEAF: usize = 8;

pub const KD_LAYOUT_DFS: i32 = 0;
pub const KD_LAYOUT_PAR4: i32 = 1;
pub const KD_PREC_FP64: i32 = 0;
pub const KD_PREC_MIXED: i32 = 1;
pub const KD_GEN_RING: i32 = 0;
pub const KD_GEN_PLUMMER: i32 = 1;
pub const KD_GEN_CIRCULAR: i32 = 2;

/// kd_particle_c: the reference's `Particle` (array_particle.rs:3-8), 64 bytes.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default, PartialEq)]
pub struct KdParticle {
    pub p: [f64; 3],
    pub v: [f64; 3],
    pub r: f64,
    pub m: f64,
}

/// kd_node_c: the flat KDTree record of Parallel/CVersion/src/kdtree.h:9-22, 8 leaf slots.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default, PartialEq)]
pub struct KdNode {
    pub num_parts: u64,
    pub particles: [u64; KD_MAX_LEAF],
    pub split_dim: u64,
    pub split_val: f64,
    pub m: f64,
    pub cm: [f64; 3],
    pub size: f64,
    pub left: u64,
    pub right: u64,
}

/// kd_params.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default, PartialEq)]
pub struct KdParams {
    pub leaf_size: i32,
    pub layout: i32,
    pub precision: i32,
    pub device: i32,
    pub theta: f64,
    pub dt: f64,
    pub heavy_frac: f64,
    pub seed: u64,
}

/// kd_stats.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default, PartialEq)]
pub struct KdStats {
    pub build_ms: f64,
    pub moments_ms: f64,
    pub walk_ms: f64,
    pub kick_ms: f64,
    pub total_ms: f64,
    pub steps: u64,
    pub launches: u64,
}

/// Opaque kd_ctx and kd_tape.
#[repr(C)]
pub struct KdCtx {
    _private: [u8; 0],
}
#[repr(C)]
pub struct KdTape {
    _private: [u8; 0],
}

#[link(name = "kdnbody")]
extern "C" {
    pub fn kd_default_params(params: *mut KdParams);
    pub fn kd_nodes_needed(n: usize, leaf_size: i32, layout: i32) -> usize;
    pub fn kd_group_plan(n: usize, leaf_size: i32, gstart: *mut u32, gsplit: *mut u32, cap: usize,
                         n_groups: *mut usize) -> c_int;
    pub fn kd_create(n: usize, params: *const KdParams) -> *mut KdCtx;
    pub fn kd_destroy(ctx: *mut KdCtx);
    pub fn kd_last_error(ctx: *const KdCtx) -> *const c_char;
    pub fn kd_set_bodies(ctx: *mut KdCtx, bodies: *const KdParticle, n: usize) -> c_int;
    pub fn kd_generate(ctx: *mut KdCtx, kind: i32, seed: u64) -> c_int;
    pub fn kd_get_bodies(ctx: *mut KdCtx, bodies: *mut KdParticle, n: usize) -> c_int;
    pub fn kd_build_tree(ctx: *mut KdCtx, last_node: *mut usize) -> c_int;
    pub fn kd_get_nodes(ctx: *mut KdCtx, out: *mut KdNode, cap: usize, count: *mut usize) -> c_int;
    pub fn kd_quickstat_index(vals: *const f64, n_vals: usize, idx: *mut u64, n: usize,
                              goal: usize, device: i32, gpu_ms: *mut f64) -> c_int;
    pub fn kd_print_tree(ctx: *mut KdCtx, path: *const c_char) -> c_int;
    pub fn kd_calc_accel(ctx: *mut KdCtx, acc: *mut f64) -> c_int;
    pub fn kd_simple_sim(ctx: *mut KdCtx, dt: f64, steps: i64) -> c_int;
    pub fn kd_energy(ctx: *mut KdCtx, out: *mut f64) -> c_int;
    pub fn kd_set_precision(ctx: *mut KdCtx, precision: i32) -> c_int;
    pub fn kd_get_stats(ctx: *const KdCtx, out: *mut KdStats) -> c_int;
    pub fn kd_set_timing(ctx: *mut KdCtx, on: i32) -> c_int;
    pub fn kd_direct_accel(ctx: *mut KdCtx, sinks: *const u64, ns: usize, acc: *mut f64) -> c_int;
    pub fn kd_forward(ctx: *mut KdCtx, dt: f64, steps: i64, ckpt_every: i64,
                      tape: *mut *mut KdTape) -> c_int;
    pub fn kd_backward(tape: *mut KdTape, dl_dx: *const f64, dl_dv: *const f64, g_x0: *mut f64,
                       g_v0: *mut f64) -> c_int;
    pub fn kd_tape_free(tape: *mut KdTape);
    pub fn kd_direct_accel_noalloc(x: *const f64, y: *const f64, z: *const f64, m: *const f64,
                                   n: usize, sinks: *const u64, ns: usize, acc: *mut f64,
                                   stream: *mut c_void) -> c_int;
    pub fn kd_set_device_limits(ctx: *mut KdCtx, stack_entries: i32, select_passes: i32) -> c_int;
    pub fn kd_fp32_peak(device: i32, out: *mut f64) -> c_int;
    pub fn kd_set_counting(ctx: *mut KdCtx, on: i32) -> c_int;
    pub fn kd_get_counts(ctx: *const KdCtx, out: *mut u64) -> c_int;
}
