//! kdnbody: the GB300 kD-tree Barnes-Hut step of libkdnbody.so (include/kdnbody.h) behind the
//! module surface of the reference crate `rust_kdtree_nbody`
//! (MarkCLewis/MultiLanguageKDTree Parallel/RustVersion/src/lib.rs:1-3:
//! `array_kd_tree`, `array_particle`, `quickstat`), so that a caller swaps the crate name and
//! keeps its call sites:
//!
//! | reference (`rust_kdtree_nbody`)                    | here (`kdnbody`)                       |
//! |----------------------------------------------------|----------------------------------------|
//! | `array_particle::Particle`, `two_bodies`, `circular_orbits` | same names (`Particle` is `#[repr(C)]`) |
//! | `array_kd_tree::allocate_node_vec(n)` :55-60       | same                                   |
//! | `array_kd_tree::build_tree(...)` :63-130 (DFS)     | same arguments, built on the GPU       |
//! | `array_kd_tree::build_tree_par4(...)` :515-583     | same arguments, built on the GPU       |
//! | `array_kd_tree::calc_accel(p, ...)` :619-621       | same (one GPU walk of all bodies per call; use `Sim::calc_accel`) |
//! | `array_kd_tree::simple_sim(&mut bodies, dt, steps)` :623-664 | same, bodies resident on the GPU |
//! | `quickstat::quickstat_index(idx, goal, lt)` :9-34  | `quickstat_index(idx, goal, keys)` (the comparator's keys) |
//! | (none: the reference has no derivatives)           | `adjoint`: `Sim::forward` / `Tape::backward` |
//!
//! The reference-shaped functions panic on failure, as the reference does on a bad index;
//! `array_kd_tree::Sim` (one device context, bodies resident in HBM) returns `Result`.
//! Every computation runs in libkdnbody.so on the GPU; this crate computes nothing itself.

pub mod ffi;

pub mod error {
    //! Status codes of the C ABI as a Rust error.
    use crate::ffi;
    use std::ffi::CStr;
    use std::os::raw::c_int;

    /// A negative KD_E* status and the library's one-line message (kd_last_error).
    #[derive(Clone, Debug, PartialEq)]
    pub struct KdError {
        pub code: i32,
        pub message: String,
    }

    impl std::fmt::Display for KdError {
        fn fmt(&self, f: &mut std::fmt::Formatter<'_>) -> std::fmt::Result {
            let name = match self.code {
                ffi::KD_EINVAL => "KD_EINVAL",
                ffi::KD_ENOMEM => "KD_ENOMEM",
                ffi::KD_ECUDA => "KD_ECUDA",
                ffi::KD_ESTATE => "KD_ESTATE",
                ffi::KD_ENUMERIC => "KD_ENUMERIC",
                ffi::KD_EOVERFLOW => "KD_EOVERFLOW",
                ffi::KD_EDEVICE => "KD_EDEVICE",
                _ => "KD_E?",
            };
            write!(f, "{}: {}", name, self.message)
        }
    }

    impl std::error::Error for KdError {}

    pub type Result<T> = std::result::Result<T, KdError>;

    /// The message kd_last_error reports for `ctx` (NULL: the calling thread's last
    /// context-free failure).
    pub fn last_error(ctx: *const ffi::KdCtx) -> String {
        // SAFETY: kd_last_error never returns NULL and the string lives until the next call
        // on the same context or thread.
        unsafe { CStr::from_ptr(ffi::kd_last_error(ctx)).to_string_lossy().into_owned() }
    }

    pub(crate) fn check(rc: c_int, ctx: *const ffi::KdCtx) -> Result<()> {
        if rc == ffi::KD_OK {
            Ok(())
        } else {
            Err(KdError { code: rc, message: last_error(ctx) })
        }
    }
}

pub mod array_particle {
    //! Bodies: `Particle` of Parallel/RustVersion/src/array_particle.rs:3-8 and its generators.

    /// Position, velocity, radius (carried, unused by the dynamics), mass.  `#[repr(C)]` with
    /// the layout of kd_particle_c, so a `Vec<Particle>` is handed to the library in place.
    #[repr(C)]
    #[derive(Clone, Copy, Debug, Default, PartialEq)]
    pub struct Particle {
        pub p: [f64; 3],
        pub v: [f64; 3],
        pub r: f64,
        pub m: f64,
    }

    /// two_bodies (array_particle.rs:10-17): a unit mass at the origin and a light body at
    /// distance 1 moving at unit speed.
    pub fn two_bodies() -> Vec<Particle> {
        vec![
            Particle { p: [0.0, 0.0, 0.0], v: [0.0, 0.0, 0.0], r: 1.0, m: 1.0 },
            Particle { p: [1.0, 0.0, 0.0], v: [0.0, 1.0, 0.0], r: 1e-4, m: 1e-20 },
        ]
    }

    /// SplitMix64: the generators' uniform stream (the reference draws from fastrand,
    /// unseeded, so its angles cannot be reproduced; here they depend on the seed only).
    struct Stream(u64);

    impl Stream {
        fn next_f64(&mut self) -> f64 {
            self.0 = self.0.wrapping_add(0x9E37_79B9_7F4A_7C15);
            let mut z = self.0;
            z = (z ^ (z >> 30)).wrapping_mul(0xBF58_476D_1CE4_E5B9);
            z = (z ^ (z >> 27)).wrapping_mul(0x94D0_49BB_1331_11EB);
            z ^= z >> 31;
            (z >> 11) as f64 * (1.0 / (1u64 << 53) as f64)
        }
    }

    /// circular_orbits (array_particle.rs:19-44): a unit central mass and n bodies of mass
    /// 1e-14 on circular orbits at radii 0.1 + 5 i / n, angles uniform in [0, 6.28); n + 1
    /// bodies in all.  The angles come from a stream seeded by `seed`.
    pub fn circular_orbits_seeded(n: usize, seed: u64) -> Vec<Particle> {
        let mut s = Stream(seed);
        let mut out = Vec::with_capacity(n + 1);
        out.push(Particle { p: [0.0; 3], v: [0.0; 3], r: 0.00465047, m: 1.0 });
        for i in 0..n {
            let d = 0.1 + (i as f64) * 5.0 / (n as f64);
            let v = (1.0 / d).sqrt();
            let theta = s.next_f64() * 6.28;
            out.push(Particle {
                p: [d * theta.cos(), d * theta.sin(), 0.0],
                v: [-v * theta.sin(), v * theta.cos(), 0.0],
                r: 1e-7,
                m: 1e-14,
            });
        }
        out
    }

    /// circular_orbits with a fixed seed (the reference's signature).
    pub fn circular_orbits(n: usize) -> Vec<Particle> {
        circular_orbits_seeded(n, 1)
    }
}

pub mod array_kd_tree {
    //! The tree and the step: the reference's `array_kd_tree` functions, run on the GPU.
    use crate::array_particle::Particle;
    use crate::error::{check, last_error, KdError, Result};
    use crate::ffi;
    use std::ffi::CString;
    use std::ptr;

    /// MAX_PARTS of Parallel/RustVersion/src/array_kd_tree.rs:14 (the sequential versions
    /// use 7; `Params::leaf_size` takes either).
    pub const MAX_PARTS: usize = 8;
    /// THETA of array_kd_tree.rs:15.
    pub const THETA: f64 = 0.3;
    const NEGS: [usize; MAX_PARTS] = [usize::MAX; MAX_PARTS];

    /// The reference's node enum (array_kd_tree.rs:18-43).
    #[derive(Clone, Copy, Debug, PartialEq)]
    pub enum KDTree {
        Leaf { num_parts: usize, leaf_parts: [usize; MAX_PARTS] },
        Internal {
            split_dim: usize,
            split_val: f64,
            m: f64,
            cm: [f64; 3],
            size: f64,
            left: usize,
            right: usize,
        },
    }

    impl KDTree {
        pub fn leaf(num_parts: usize, particles: [usize; MAX_PARTS]) -> KDTree {
            KDTree::Leaf { num_parts, leaf_parts: particles }
        }

        fn from_node(n: &ffi::KdNode, index_of: &dyn Fn(u64) -> usize, offset: usize) -> KDTree {
            if n.num_parts > 0 || (n.left == 0 && n.right == 0) {
                let mut parts = NEGS;
                for k in 0..n.num_parts as usize {
                    parts[k] = index_of(n.particles[k]);
                }
                KDTree::Leaf { num_parts: n.num_parts as usize, leaf_parts: parts }
            } else {
                KDTree::Internal {
                    split_dim: n.split_dim as usize,
                    split_val: n.split_val,
                    m: n.m,
                    cm: n.cm,
                    size: n.size,
                    left: n.left as usize + offset,
                    right: n.right as usize + offset,
                }
            }
        }
    }

    /// Layout of the node numbering (KD_LAYOUT_*).
    #[derive(Clone, Copy, Debug, PartialEq)]
    pub enum Layout {
        /// build_tree: left = cur + 1, right = last node of the left subtree + 1.
        Dfs,
        /// build_tree_par4: left = cur + 1, right = cur + 1 + nodes_needed(len / 2).
        Par4,
    }

    /// Arithmetic of the walk (KD_PREC_*).
    #[derive(Clone, Copy, Debug, PartialEq)]
    pub enum Precision {
        /// The reference's FP64 arithmetic and interaction set.
        Fp64,
        /// FP32 pair and node terms on split coordinates, FP64 storage and heavy bodies.
        Mixed,
    }

    /// kd_params with the reference's defaults (leaf 8 and PAR4 as the parallel crate).
    #[derive(Clone, Copy, Debug)]
    pub struct Params {
        pub leaf_size: usize,
        pub layout: Layout,
        pub precision: Precision,
        pub device: i32,
        pub theta: f64,
        pub dt: f64,
        pub heavy_frac: f64,
    }

    impl Default for Params {
        fn default() -> Self {
            Params {
                leaf_size: MAX_PARTS,
                layout: Layout::Par4,
                precision: Precision::Fp64,
                device: 0,
                theta: THETA,
                dt: 1e-3,
                heavy_frac: 1e-3,
            }
        }
    }

    impl Params {
        fn raw(&self) -> ffi::KdParams {
            let mut p = ffi::KdParams::default();
            // SAFETY: p is a valid, writable kd_params.
            unsafe { ffi::kd_default_params(&mut p) };
            p.leaf_size = self.leaf_size as i32;
            p.layout = match self.layout {
                Layout::Dfs => ffi::KD_LAYOUT_DFS,
                Layout::Par4 => ffi::KD_LAYOUT_PAR4,
            };
            p.precision = match self.precision {
                Precision::Fp64 => ffi::KD_PREC_FP64,
                Precision::Mixed => ffi::KD_PREC_MIXED,
            };
            p.device = self.device;
            p.theta = self.theta;
            p.dt = self.dt;
            p.heavy_frac = self.heavy_frac;
            p
        }
    }

    fn as_raw(b: &[Particle]) -> *const ffi::KdParticle {
        // Particle and KdParticle are both #[repr(C)] { [f64; 3], [f64; 3], f64, f64 }
        b.as_ptr() as *const ffi::KdParticle
    }

    /// One device context: n bodies resident in HBM, their tree, accelerations and step loop.
    pub struct Sim {
        pub(crate) ctx: *mut ffi::KdCtx,
        n: usize,
        params: Params,
    }

    impl Sim {
        pub fn new(n: usize, params: Params) -> Result<Sim> {
            let raw = params.raw();
            // SAFETY: raw is a valid kd_params; a NULL return is checked.
            let ctx = unsafe { ffi::kd_create(n, &raw) };
            if ctx.is_null() {
                return Err(KdError { code: ffi::KD_EINVAL, message: last_error(ptr::null()) });
            }
            Ok(Sim { ctx, n, params })
        }

        pub fn len(&self) -> usize {
            self.n
        }

        pub fn is_empty(&self) -> bool {
            self.n == 0
        }

        pub fn params(&self) -> Params {
            self.params
        }

        /// Copy the bodies to the device (checks p, v, m finite and m >= 0).
        pub fn set_bodies(&mut self, bodies: &[Particle]) -> Result<()> {
            // SAFETY: bodies holds bodies.len() records of the kd_particle_c layout.
            check(unsafe { ffi::kd_set_bodies(self.ctx, as_raw(bodies), bodies.len()) }, self.ctx)
        }

        /// Copy the bodies back to the host.
        pub fn get_bodies(&mut self, bodies: &mut [Particle]) -> Result<()> {
            let p = bodies.as_mut_ptr() as *mut ffi::KdParticle;
            // SAFETY: bodies has room for bodies.len() records.
            check(unsafe { ffi::kd_get_bodies(self.ctx, p, bodies.len()) }, self.ctx)
        }

        /// Generate bodies on the device (ffi::KD_GEN_RING, _PLUMMER, _CIRCULAR).
        pub fn generate(&mut self, kind: i32, seed: u64) -> Result<()> {
            check(unsafe { ffi::kd_generate(self.ctx, kind, seed) }, self.ctx)
        }

        /// Build the tree of the current bodies; returns the last node used (build_tree's
        /// return value for DFS, the highest occupied slot for PAR4).
        pub fn build_tree(&mut self) -> Result<usize> {
            let mut last = 0usize;
            check(unsafe { ffi::kd_build_tree(self.ctx, &mut last) }, self.ctx)?;
            Ok(last)
        }

        /// The flat node records of the last build, in the context's numbering.
        pub fn raw_nodes(&mut self) -> Result<Vec<ffi::KdNode>> {
            let layout = self.params.raw().layout;
            let leaf = self.params.leaf_size as i32;
            let cap = match self.params.layout {
                Layout::Par4 => unsafe { ffi::kd_nodes_needed(self.n, leaf, layout) },
                Layout::Dfs => 2 * self.n + 2,
            };
            let mut out = vec![ffi::KdNode::default(); cap.max(1)];
            let mut count = 0usize;
            check(unsafe { ffi::kd_get_nodes(self.ctx, out.as_mut_ptr(), out.len(), &mut count) },
                  self.ctx)?;
            out.truncate(count);
            Ok(out)
        }

        /// The last build as the reference's node vector.
        pub fn nodes(&mut self) -> Result<Vec<KDTree>> {
            let raw = self.raw_nodes()?;
            Ok(raw.iter().map(|n| KDTree::from_node(n, &|i| i as usize, 0)).collect())
        }

        /// calc_accel for every body over the last build.
        pub fn calc_accel(&mut self) -> Result<Vec<[f64; 3]>> {
            let mut acc = vec![[0.0f64; 3]; self.n];
            check(unsafe { ffi::kd_calc_accel(self.ctx, acc.as_mut_ptr() as *mut f64) },
                  self.ctx)?;
            Ok(acc)
        }

        /// `steps` steps of build, walk and kick-drift (dt == 0: the context's dt).
        pub fn simple_sim(&mut self, dt: f64, steps: i64) -> Result<()> {
            check(unsafe { ffi::kd_simple_sim(self.ctx, dt, steps) }, self.ctx)
        }

        /// (kinetic, potential) energy of the current bodies.
        pub fn energy(&mut self) -> Result<(f64, f64)> {
            let mut e = [0.0f64; 2];
            check(unsafe { ffi::kd_energy(self.ctx, e.as_mut_ptr()) }, self.ctx)?;
            Ok((e[0], e[1]))
        }

        /// FP64 direct-sum accelerations of the listed bodies (an error yardstick).
        pub fn direct_accel(&mut self, sinks: &[u64]) -> Result<Vec<[f64; 3]>> {
            let mut acc = vec![[0.0f64; 3]; sinks.len()];
            check(unsafe {
                ffi::kd_direct_accel(self.ctx, sinks.as_ptr(), sinks.len(),
                                     acc.as_mut_ptr() as *mut f64)
            }, self.ctx)?;
            Ok(acc)
        }

        pub fn set_precision(&mut self, precision: Precision) -> Result<()> {
            self.params.precision = precision;
            let p = self.params.raw().precision;
            check(unsafe { ffi::kd_set_precision(self.ctx, p) }, self.ctx)
        }

        /// print_tree (array_kd_tree.rs:666-692) of the last build into `path`.
        pub fn print_tree(&mut self, path: &str) -> Result<()> {
            let c = CString::new(path).map_err(|_| KdError {
                code: ffi::KD_EINVAL,
                message: "path holds a NUL byte".to_string(),
            })?;
            check(unsafe { ffi::kd_print_tree(self.ctx, c.as_ptr()) }, self.ctx)
        }

        /// Device times and launch count of the last call.
        pub fn stats(&self) -> Result<ffi::KdStats> {
            let mut s = ffi::KdStats::default();
            check(unsafe { ffi::kd_get_stats(self.ctx, &mut s) }, self.ctx)?;
            Ok(s)
        }
    }

    impl Drop for Sim {
        fn drop(&mut self) {
            // SAFETY: ctx came from kd_create and is destroyed once.
            unsafe { ffi::kd_destroy(self.ctx) };
        }
    }

    fn expect<T>(r: Result<T>) -> T {
        match r {
            Ok(v) => v,
            Err(e) => panic!("{}", e),
        }
    }

    fn nodes_needed(n: usize, layout: Layout) -> usize {
        let l = match layout {
            Layout::Dfs => ffi::KD_LAYOUT_DFS,
            Layout::Par4 => ffi::KD_LAYOUT_PAR4,
        };
        // SAFETY: a pure function of its arguments.
        unsafe { ffi::kd_nodes_needed(n, MAX_PARTS as i32, l) }
    }

    /// allocate_node_vec (array_kd_tree.rs:55-60): nodes_needed_for_particles(n) empty leaves.
    pub fn allocate_node_vec(num_parts: usize) -> Vec<KDTree> {
        vec![KDTree::leaf(0, NEGS); nodes_needed(num_parts, Layout::Par4)]
    }

    /// Builds the tree of particles[indices[start..end]] on the GPU into nodes[cur_node..]
    /// with `layout`'s numbering; leaves name bodies by their index in `particles`, and
    /// indices[start..end] is rewritten in tree order.  Returns the last node written.
    fn build_into(indices: &mut [usize], particles: &[Particle], cur_node: usize,
                  nodes: &mut Vec<KDTree>, layout: Layout) -> usize {
        let sub: Vec<Particle> = indices.iter().map(|&i| particles[i]).collect();
        let params = Params { layout, ..Params::default() };
        let mut sim = expect(Sim::new(sub.len(), params));
        expect(sim.set_bodies(&sub));
        expect(sim.build_tree());
        let raw = expect(sim.raw_nodes());
        let map: Vec<usize> = indices.to_vec();
        let index_of = |i: u64| map[i as usize];
        if nodes.len() < cur_node + raw.len() {
            nodes.resize(cur_node + raw.len(), KDTree::leaf(0, NEGS));
        }
        let mut k = 0usize;
        for (j, n) in raw.iter().enumerate() {
            nodes[cur_node + j] = KDTree::from_node(n, &index_of, cur_node);
            for q in 0..n.num_parts as usize {
                indices[k] = index_of(n.particles[q]);
                k += 1;
            }
        }
        let used = raw
            .iter()
            .rposition(|n| n.num_parts > 0 || n.left != 0 || n.right != 0)
            .unwrap_or(0);
        cur_node + used
    }

    /// build_tree (array_kd_tree.rs:63-130, DFS numbering): the tree of
    /// particles[indices[start..end]] at nodes[cur_node..]; returns the index of the last node
    /// used.  The nodes Vec grows when it is too short (as the sequential version's does).
    pub fn build_tree(indices: &mut Vec<usize>, start: usize, end: usize,
                      particles: &Vec<Particle>, cur_node: usize, nodes: &mut Vec<KDTree>)
                      -> usize {
        build_into(&mut indices[start..end], particles, cur_node, nodes, Layout::Dfs)
    }

    /// build_tree_par4 (array_kd_tree.rs:515-583, PAR4 numbering) of particles[indices] into
    /// nodes[cur_node..].  `thread_cnt` is accepted for the call shape; the build runs on the
    /// GPU.
    pub fn build_tree_par4(indices: &mut [usize], cur_node: usize, particles: &Vec<Particle>,
                           nodes: &mut [KDTree], thread_cnt: usize) {
        let _ = thread_cnt;
        let mut v = nodes.to_vec();
        build_into(indices, particles, cur_node, &mut v, Layout::Par4);
        assert!(v.len() <= nodes.len(), "node slice too short for build_tree_par4");
        nodes.copy_from_slice(&v[..nodes.len()]);
    }

    /// calc_accel (array_kd_tree.rs:619-621) of body p.  `nodes` must be the tree of
    /// `particles` (as built above); the GPU rebuilds that same tree (membership is
    /// bit-exact) and walks every body, so calling this per body costs a whole walk each
    /// time: use `Sim::calc_accel` (all bodies at once) in a loop.
    pub fn calc_accel(p: usize, particles: &Vec<Particle>, nodes: &Vec<KDTree>) -> [f64; 3] {
        let _ = nodes;
        let mut sim = expect(Sim::new(particles.len(), Params::default()));
        expect(sim.set_bodies(particles));
        expect(sim.build_tree());
        expect(sim.calc_accel())[p]
    }

    /// simple_sim (array_kd_tree.rs:623-664): `steps` steps of the bodies in place, resident
    /// on the GPU for the whole run.
    pub fn simple_sim(bodies: &mut Vec<Particle>, dt: f64, steps: i64) {
        let mut sim = expect(Sim::new(bodies.len(), Params::default()));
        expect(sim.set_bodies(bodies));
        expect(sim.simple_sim(dt, steps));
        expect(sim.get_bodies(bodies));
    }

    /// print_tree (array_kd_tree.rs:666-692) of the bodies' tree, written to tree{step}.txt.
    pub fn print_tree(step: i64, particles: &Vec<Particle>) -> std::io::Result<()> {
        let mut sim = Sim::new(particles.len(), Params::default())
            .map_err(|e| std::io::Error::new(std::io::ErrorKind::Other, e))?;
        let io = |e: KdError| std::io::Error::new(std::io::ErrorKind::Other, e);
        sim.set_bodies(particles).map_err(io)?;
        sim.build_tree().map_err(io)?;
        sim.print_tree(&format!("tree{}.txt", step)).map_err(io)
    }
}

pub mod quickstat {
    //! quickstat_index (Parallel/RustVersion/src/quickstat.rs:9-34) on the GPU.
    use crate::error::{check, Result};
    use crate::ffi;
    use std::ptr;

    /// Reorders `indices` so that keys[indices[i]] < keys[indices[goal]] for i < goal and
    /// keys[indices[i]] >= keys[indices[goal]] for i >= goal (the post-condition of
    /// quickstat.rs:211-216).  The reference takes a comparator `lt(i1, i2)`; its build
    /// compares one coordinate of two bodies, so here the caller passes those keys.  Equal
    /// keys are ordered by index.
    pub fn quickstat_index(indices: &mut [usize], goal: usize, keys: &[f64]) -> Result<()> {
        let mut idx: Vec<u64> = indices.iter().map(|&i| i as u64).collect();
        check(unsafe {
            ffi::kd_quickstat_index(keys.as_ptr(), keys.len(), idx.as_mut_ptr(), idx.len(), goal,
                                    0, ptr::null_mut())
        }, ptr::null())?;
        for (d, s) in indices.iter_mut().zip(idx) {
            *d = s as usize;
        }
        Ok(())
    }
}

pub mod adjoint {
    //! Reverse mode of the step loop with the autograd.Function contract: `Sim::forward` runs
    //! the steps and saves checkpoints; `Tape::backward` takes the gradient of a loss with
    //! respect to the final positions and velocities and returns it with respect to the
    //! initial ones.  The reference has no derivatives; this differentiates simple_sim
    //! (array_kd_tree.rs:623-664) over the mixed-precision walk's interaction set.
    use crate::array_kd_tree::Sim;
    use crate::error::{check, Result};
    use crate::ffi;
    use std::ptr;

    /// The saved state of one forward sweep; it borrows its context, which it drives.
    pub struct Tape<'a> {
        sim: &'a mut Sim,
        tape: *mut ffi::KdTape,
    }

    impl Sim {
        /// forward: `steps` steps like simple_sim (the context must use Precision::Mixed),
        /// keeping a checkpoint of (x, v) every `ckpt_every` steps.
        pub fn forward(&mut self, dt: f64, steps: i64, ckpt_every: i64) -> Result<Tape<'_>> {
            let mut t: *mut ffi::KdTape = ptr::null_mut();
            check(unsafe { ffi::kd_forward(self.ctx, dt, steps, ckpt_every, &mut t) },
                  self.ctx)?;
            Ok(Tape { sim: self, tape: t })
        }
    }

    impl<'a> Tape<'a> {
        /// The context (its bodies are the forward sweep's final state).
        pub fn sim(&mut self) -> &mut Sim {
            &mut *self.sim
        }

        /// backward: (dL/dx_0, dL/dv_0) from dL/dx_T and dL/dv_T (None: zero).  May be called
        /// again with other gradients.
        pub fn backward(&mut self, dl_dx: &[[f64; 3]], dl_dv: Option<&[[f64; 3]]>)
                        -> Result<(Vec<[f64; 3]>, Vec<[f64; 3]>)> {
            let n = self.sim.len();
            assert_eq!(dl_dx.len(), n, "dl_dx must hold one row per body");
            if let Some(v) = dl_dv {
                assert_eq!(v.len(), n, "dl_dv must hold one row per body");
            }
            let mut gx = vec![[0.0f64; 3]; n];
            let mut gv = vec![[0.0f64; 3]; n];
            let dv = dl_dv.map_or(ptr::null(), |v| v.as_ptr() as *const f64);
            check(unsafe {
                ffi::kd_backward(self.tape, dl_dx.as_ptr() as *const f64, dv,
                                 gx.as_mut_ptr() as *mut f64, gv.as_mut_ptr() as *mut f64)
            }, self.sim.ctx)?;
            Ok((gx, gv))
        }
    }

    impl<'a> Drop for Tape<'a> {
        fn drop(&mut self) {
            // SAFETY: the tape came from kd_forward on a context that outlives it (borrow).
            unsafe { ffi::kd_tape_free(self.tape) };
        }
    }

    /// The pair as free functions: forward(sim, ...) saves, backward(tape, ...) consumes.
    pub fn forward(sim: &mut Sim, dt: f64, steps: i64, ckpt_every: i64) -> Result<Tape<'_>> {
        sim.forward(dt, steps, ckpt_every)
    }

    pub fn backward(tape: &mut Tape<'_>, dl_dx: &[[f64; 3]], dl_dv: Option<&[[f64; 3]]>)
                    -> Result<(Vec<[f64; 3]>, Vec<[f64; 3]>)> {
        tape.backward(dl_dx, dl_dv)
    }
}
