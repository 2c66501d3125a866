"""The kD-tree Barnes-Hut step on the GPU, with the reference's call shape.

Mirror of ``array_kd_tree`` of MarkCLewis/MultiLanguageKDTree
(Parallel/RustVersion/src/array_kd_tree.rs and Sequential/RustVersion/src/array_kd_tree.rs):

=====================================  =========================================
reference                              here
=====================================  =========================================
``allocate_node_vec(n)`` :55-60        ``allocate_node_vec(n, leaf_size, layout)``
``build_tree(...) -> usize`` :63-130   ``build_tree(bodies, ...)`` / ``KDTreeSim.build_tree``
``build_tree_par4(...)`` :515-583      ``build_tree(bodies, layout="par4")``
``calc_accel(p, ...)`` :619-621        ``calc_accel(bodies, ...)`` (all bodies at once)
``simple_sim(&mut bodies, dt, steps)`` ``simple_sim(bodies, dt, steps)`` (updates in place)
=====================================  =========================================

``KDTreeSim`` holds one device context (bodies resident in HBM between calls); the module
functions create a context for one call.  Every computation runs in libkdnbody.so on the
GPU; nothing here computes on the CPU.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import NODE_DTYPE, PARTICLE_DTYPE, KDError

__all__ = ["KDTreeSim", "Tape", "allocate_node_vec", "nodes_needed", "build_tree", "calc_accel",
           "simple_sim", "fp32_peak", "KDError", "NODE_DTYPE", "LAYOUTS", "PRECISIONS"]

LAYOUTS = {"dfs": _lib.KD_LAYOUT_DFS, "par4": _lib.KD_LAYOUT_PAR4}
PRECISIONS = {"fp64": _lib.KD_PREC_FP64, "mixed": _lib.KD_PREC_MIXED}


def _layout(v) -> int:
    return LAYOUTS[v] if isinstance(v, str) else int(v)


def _precision(v) -> int:
    return PRECISIONS[v] if isinstance(v, str) else int(v)


def group_plan(n: int, leaf_size: int = 7):
    """Sink groups of the mixed walk for n bodies (host computation): (gstart, gsplit) in tree
    positions, see kd_group_plan."""
    lib = _lib.load()
    ng = C.c_size_t(0)
    lib.kd_group_plan(n, leaf_size, None, None, 0, C.byref(ng))
    if ng.value == 0:
        raise ValueError("n must be >= 1 and leaf_size in [2, 8]")
    gstart = np.zeros(ng.value + 1, dtype=np.uint32)
    gsplit = np.zeros(ng.value, dtype=np.uint32)
    rc = lib.kd_group_plan(n, leaf_size, gstart.ctypes.data_as(C.POINTER(C.c_uint32)),
                           gsplit.ctypes.data_as(C.POINTER(C.c_uint32)), ng.value + 1,
                           C.byref(ng))
    if rc != 0:
        raise ValueError(f"kd_group_plan failed ({rc})")
    return gstart, gsplit


def fp32_peak(device: int = 0) -> dict:
    """Measured FP32 multiply-add rate of a device in TFLOP/s (kd_fp32_peak): scalar
    fma.rn.f32 and packed fma.rn.f32x2."""
    lib = _lib.load()
    out = (C.c_double * 2)()
    rc = lib.kd_fp32_peak(device, out)
    if rc != 0:
        raise KDError(rc, lib.kd_last_error(None).decode())
    return {"scalar": float(out[0]), "packed": float(out[1])}


def nodes_needed(n: int, leaf_size: int = 8, layout="par4") -> int:
    """nodes_needed_for_particles: PAR4 array_kd_tree.rs:45-53 (Parallel), DFS
    Sequential/RustVersion/src/array_kd_tree.rs:37-39."""
    v = _lib.load().kd_nodes_needed(n, leaf_size, _layout(layout))
    if v == 0:
        raise ValueError("leaf_size must be in [2, 8]")
    return int(v)


def allocate_node_vec(n: int, leaf_size: int = 8, layout="par4") -> np.ndarray:
    """allocate_node_vec (array_kd_tree.rs:55-60): nodes_needed(n) empty leaves, each with
    num_parts 0 and leaf slots set to usize::MAX (the NEGS constant, :16)."""
    out = np.zeros(nodes_needed(n, leaf_size, layout), dtype=NODE_DTYPE)
    out["particles"] = np.iinfo(np.uint64).max
    return out


class KDTreeSim:
    """One device context: ``n`` bodies, their tree, accelerations and step loop."""

    def __init__(self, n: int, leaf_size: int = 7, layout="dfs", precision="fp64",
                 theta: float = 0.3, dt: float = 1e-3, heavy_frac: float = 1e-3,
                 device: int = 0):
        lib = _lib.load()
        p = _lib.KdParams()
        lib.kd_default_params(C.byref(p))
        p.leaf_size = leaf_size
        p.layout = _layout(layout)
        p.precision = _precision(precision)
        p.device = device
        p.theta = theta
        p.dt = dt
        p.heavy_frac = heavy_frac
        self._lib = lib
        self.n = int(n)
        self.leaf_size = leaf_size
        self.layout = p.layout
        self._ctx = lib.kd_create(self.n, C.byref(p))
        if not self._ctx:
            raise KDError(_lib.KD_EINVAL, lib.kd_last_error(None).decode())

    # ------------------------------------------------------------- lifetime
    def close(self) -> None:
        if getattr(self, "_ctx", None):
            self._lib.kd_destroy(self._ctx)
            self._ctx = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int) -> None:
        _lib.check(rc, self._ctx)

    # ------------------------------------------------------------- bodies
    def set_bodies(self, bodies: np.ndarray) -> None:
        b = np.ascontiguousarray(bodies, dtype=PARTICLE_DTYPE)
        self._check(self._lib.kd_set_bodies(self._ctx, _lib.ptr(b), b.shape[0]))

    def generate(self, kind: str = "ring", seed: int = 0) -> None:
        """Generate the bodies on the device: "ring", "plummer" or "circular"
        (circular_orbits(n-1))."""
        kinds = {"ring": _lib.KD_GEN_RING, "plummer": _lib.KD_GEN_PLUMMER,
                 "circular": _lib.KD_GEN_CIRCULAR}
        self._check(self._lib.kd_generate(self._ctx, kinds[kind], int(seed)))

    def get_bodies(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(self.n, dtype=PARTICLE_DTYPE)
        if out.dtype != PARTICLE_DTYPE or not out.flags.c_contiguous or out.shape[0] != self.n:
            raise ValueError("out must be a contiguous PARTICLE_DTYPE array of length n")
        self._check(self._lib.kd_get_bodies(self._ctx, _lib.ptr(out), self.n))
        return out

    # ------------------------------------------------------------- tree
    def build_tree(self) -> int:
        """Build over the current bodies; returns the last node index (DFS: build_tree's
        return value; PAR4: the highest occupied slot)."""
        last = C.c_size_t(0)
        self._check(self._lib.kd_build_tree(self._ctx, C.byref(last)))
        return int(last.value)

    def nodes(self) -> np.ndarray:
        """The last built tree in the context's layout, as NODE_DTYPE records."""
        cap = max(nodes_needed(self.n, self.leaf_size, self.layout), 2 * self.n + 2)
        out = np.zeros(cap, dtype=NODE_DTYPE)
        cnt = C.c_size_t(0)
        self._check(self._lib.kd_get_nodes(self._ctx, _lib.ptr(out), cap, C.byref(cnt)))
        return out[: cnt.value]

    def print_tree(self, step: int | None = None, path: str | None = None) -> str:
        """print_tree (array_kd_tree.rs:666-692): write the last built tree to `path`, or to
        tree{step}.txt as the reference names it.  Returns the path."""
        if path is None:
            path = f"tree{0 if step is None else int(step)}.txt"
        self._check(self._lib.kd_print_tree(self._ctx, str(path).encode()))
        return str(path)

    # ------------------------------------------------------------- forces and steps
    def calc_accel(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty((self.n, 3), dtype=np.float64)
        self._check(self._lib.kd_calc_accel(self._ctx, _lib.ptr(out)))
        return out

    def simple_sim(self, dt: float, steps: int) -> None:
        self._check(self._lib.kd_simple_sim(self._ctx, float(dt), int(steps)))

    def energy(self) -> tuple[float, float]:
        """(kinetic, potential) energy of the current bodies (potential from a tree walk)."""
        out = (C.c_double * 2)()
        self._check(self._lib.kd_energy(self._ctx, out))
        return float(out[0]), float(out[1])

    def set_precision(self, precision) -> None:
        self._check(self._lib.kd_set_precision(self._ctx, _precision(precision)))

    def forward(self, dt: float, steps: int, ckpt_every: int = 32) -> "Tape":
        """Run `steps` steps like simple_sim, keeping checkpoints for backward()."""
        t = C.c_void_p()
        self._check(self._lib.kd_forward(self._ctx, float(dt), int(steps), int(ckpt_every),
                                         C.byref(t)))
        return Tape(self, t)

    def set_timing(self, on: bool) -> None:
        self._check(self._lib.kd_set_timing(self._ctx, 1 if on else 0))

    def direct_accel(self, sinks) -> np.ndarray:
        """FP64 direct-sum accelerations of the given bodies (an error yardstick)."""
        s = np.ascontiguousarray(sinks, dtype=np.uint64)
        out = np.empty((len(s), 3), dtype=np.float64)
        self._check(self._lib.kd_direct_accel(self._ctx, _lib.ptr(s), len(s), _lib.ptr(out)))
        return out

    def set_device_limits(self, stack_entries: int = -1, select_passes: int = -1) -> None:
        """Lower the device-side guards (kd_set_device_limits; negative = the default)."""
        self._check(self._lib.kd_set_device_limits(self._ctx, stack_entries, select_passes))

    def set_counting(self, on: bool) -> None:
        self._check(self._lib.kd_set_counting(self._ctx, 1 if on else 0))

    def counts(self) -> dict:
        a = (C.c_uint64 * 4)()
        self._check(self._lib.kd_get_counts(self._ctx, a))
        return {"p2p": a[0], "opened": a[1], "m2p": a[2], "visits": a[3]}

    def stats(self) -> dict:
        s = _lib.KdStats()
        self._check(self._lib.kd_get_stats(self._ctx, C.byref(s)))
        return {k: getattr(s, k) for k, _ in s._fields_}


class Tape:
    """Checkpoints of one forward sweep; backward() maps the gradient at the final state to
    the gradient at the initial state (the autograd.Function contract: forward saves,
    backward consumes grad-outputs and returns grad-inputs)."""

    def __init__(self, sim: KDTreeSim, handle: C.c_void_p):
        self._sim = sim
        self._h = handle

    def backward(self, dL_dx: np.ndarray, dL_dv: np.ndarray | None = None):
        n = self._sim.n
        gx = np.ascontiguousarray(dL_dx, dtype=np.float64).reshape(n, 3)
        gv = None if dL_dv is None else np.ascontiguousarray(dL_dv, dtype=np.float64).reshape(n, 3)
        ox = np.empty((n, 3))
        ov = np.empty((n, 3))
        self._sim._check(self._sim._lib.kd_backward(
            self._h, _lib.ptr(gx), _lib.ptr(gv) if gv is not None else None, _lib.ptr(ox),
            _lib.ptr(ov)))
        return ox, ov

    def close(self) -> None:
        if self._h:
            self._sim._lib.kd_tape_free(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def build_tree(bodies: np.ndarray, leaf_size: int = 7, layout="dfs", device: int = 0):
    """Build the tree of ``bodies`` on the GPU; returns (nodes, last_node) in the chosen
    layout's numbering (build_tree / build_tree_par4)."""
    with KDTreeSim(len(bodies), leaf_size=leaf_size, layout=layout, device=device) as s:
        s.set_bodies(bodies)
        last = s.build_tree()
        return s.nodes(), last


def calc_accel(bodies: np.ndarray, leaf_size: int = 7, theta: float = 0.3, precision="fp64",
               device: int = 0) -> np.ndarray:
    """calc_accel for every body (array_kd_tree.rs:619-621 applied to 0..n)."""
    with KDTreeSim(len(bodies), leaf_size=leaf_size, theta=theta, precision=precision,
                   device=device) as s:
        s.set_bodies(bodies)
        s.build_tree()
        return s.calc_accel()


def simple_sim(bodies: np.ndarray, dt: float, steps: int, leaf_size: int = 7,
               theta: float = 0.3, precision="fp64", device: int = 0) -> None:
    """simple_sim (array_kd_tree.rs:623-664): advances ``bodies`` in place."""
    with KDTreeSim(len(bodies), leaf_size=leaf_size, theta=theta, precision=precision,
                   device=device) as s:
        s.set_bodies(bodies)
        s.simple_sim(dt, steps)
        s.get_bodies(out=bodies)
