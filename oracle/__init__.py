"""CPU oracle of the kD-tree Barnes-Hut step -- TEST INFRASTRUCTURE ONLY.

Loaded only by tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py, as
the checker.  The product (multilanguagekdtree_gb300, libkdnbody.so) never imports it.

``Oracle`` wraps liboracle.so, the C restatement of the reference's Rust code
(kdoracle.c).  ``RefC`` wraps oracle/_ref/libkdref.so, the reference's own C port
(Parallel/CVersion/src/kdtree.c, particle.c) compiled from the reference checkout by
oracle/build.py; it exists only where the reference is mounted.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

HERE = Path(__file__).resolve().parent

# Particle record (array_particle.rs:3-8), 64 bytes
PARTICLE = np.dtype([("p", "<f8", (3,)), ("v", "<f8", (3,)), ("r", "<f8"), ("m", "<f8")])
# orc_node: the C port's flat KDTree (kdtree.h:9-22) with 8 leaf slots
NODE = np.dtype([
    ("num_parts", "<u8"), ("particles", "<u8", (8,)), ("split_dim", "<u8"),
    ("split_val", "<f8"), ("m", "<f8"), ("cm", "<f8", (3,)), ("size", "<f8"),
    ("left", "<u8"), ("right", "<u8"),
])
# the reference C port's KDTree with MAX_PARTS = 7 (kdtree.h:6, :9-22)
REF_NODE = np.dtype([
    ("num_parts", "<u8"), ("particles", "<u8", (7,)), ("split_dim", "<u8"),
    ("split_val", "<f8"), ("m", "<f8"), ("cm", "<f8", (3,)), ("size", "<f8"),
    ("left", "<u8"), ("right", "<u8"),
])

_vp = C.c_void_p


def _p(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


class Oracle:
    """The C restatement (liboracle.so)."""

    def __init__(self, build: bool = True):
        path = _build.build_oracle() if build else _build.ORACLE_LIB
        lib = C.CDLL(str(path))
        sig = {
            "orc_nodes_needed_par": (C.c_uint64, [C.c_uint64, C.c_int]),
            "orc_nodes_needed_seq": (C.c_uint64, [C.c_uint64, C.c_int]),
            "orc_quickstat_index": (None, [_vp, C.c_size_t, C.c_size_t, _vp, C.c_uint64]),
            "orc_build_tree_dfs": (C.c_uint64, [_vp, C.c_size_t, _vp, _vp, C.c_size_t, C.c_int,
                                                C.c_uint64]),
            "orc_build_tree_par4": (C.c_int, [_vp, C.c_size_t, _vp, _vp, C.c_size_t, C.c_int,
                                              C.c_uint64]),
            "orc_calc_accel_all": (None, [_vp, C.c_size_t, _vp, C.c_double, _vp]),
            "orc_calc_accel_abs": (None, [_vp, C.c_size_t, _vp, C.c_double, _vp, _vp]),
            "orc_walk_counts": (None, [_vp, _vp, C.c_double, _vp, C.c_size_t, _vp]),
            "orc_calc_accel_sinks": (None, [_vp, _vp, C.c_double, _vp, C.c_size_t, _vp, _vp]),
            "orc_direct_accel_abs": (None, [_vp, C.c_size_t, _vp, C.c_size_t, _vp, _vp]),
            "orc_sampled_step": (C.c_int, [_vp, C.c_size_t, C.c_double, C.c_int, C.c_double,
                                           C.c_uint64, _vp, C.c_size_t, _vp]),
            "orc_simple_sim": (C.c_int, [_vp, C.c_size_t, C.c_double, C.c_int64, C.c_int, C.c_int,
                                         C.c_double, C.c_uint64, _vp]),
            "orc_direct_accel": (None, [_vp, C.c_size_t, _vp, C.c_size_t, _vp]),
            "orc_energy": (None, [_vp, C.c_size_t, _vp]),
            "orc_adjoint_direct": (C.c_int, [_vp, C.c_size_t, C.c_double, C.c_int64, _vp, _vp,
                                             _vp, _vp, _vp, _vp, _vp]),
            "orc_tree_jt": (C.c_int, [_vp, C.c_size_t, _vp, C.c_size_t, C.c_double, _vp, _vp]),
            "orc_tree_jt_group": (C.c_int, [_vp, C.c_size_t, _vp, C.c_size_t, C.c_double, _vp,
                                            _vp]),
            "orc_calc_accel_group": (C.c_int, [_vp, C.c_size_t, _vp, C.c_size_t, C.c_double, _vp,
                                               _vp]),
            "orc_groups": (C.c_size_t, [_vp, C.c_size_t, C.c_size_t, _vp, _vp, C.c_size_t]),
            "orc_omp_threads": (C.c_int, []),
            "orc_set_threads": (None, [C.c_int]),
        }
        for name, (res, args) in sig.items():
            f = getattr(lib, name)
            f.restype, f.argtypes = res, args
        self.lib = lib

    @staticmethod
    def _bodies(b):
        b = np.ascontiguousarray(b)
        if b.dtype.itemsize != 64:
            raise ValueError("bodies must be 64-byte Particle records")
        return b.view(PARTICLE)

    def threads(self) -> int:
        return self.lib.orc_omp_threads()

    def set_threads(self, n: int) -> None:
        self.lib.orc_set_threads(n)

    def nodes_needed_par(self, n: int, leaf: int) -> int:
        return int(self.lib.orc_nodes_needed_par(n, leaf))

    def nodes_needed_seq(self, n: int, leaf: int) -> int:
        return int(self.lib.orc_nodes_needed_seq(n, leaf))

    def quickstat_index(self, vals, goal: int, idx=None, seed: int = 1) -> np.ndarray:
        vals = np.ascontiguousarray(vals, dtype=np.float64)
        idx = np.arange(len(vals), dtype=np.uint64) if idx is None else np.ascontiguousarray(
            idx, dtype=np.uint64)
        self.lib.orc_quickstat_index(_p(idx), len(idx), goal, _p(vals), seed)
        return idx

    def build_tree_dfs(self, bodies, leaf: int = 7, seed: int = 1):
        b = self._bodies(bodies)
        n = len(b)
        cap = 2 * n + 2
        nodes = np.zeros(cap, dtype=NODE)
        idx = np.arange(n, dtype=np.uint64)
        last = self.lib.orc_build_tree_dfs(_p(idx), n, _p(b), _p(nodes), cap, leaf, seed)
        if last == 2 ** 64 - 1:
            raise RuntimeError("node capacity exceeded")
        return nodes[: last + 1], int(last)

    def build_tree_par4(self, bodies, leaf: int = 8, seed: int = 1):
        b = self._bodies(bodies)
        n = len(b)
        cap = self.nodes_needed_par(n, leaf)
        nodes = np.zeros(cap, dtype=NODE)
        idx = np.arange(n, dtype=np.uint64)
        if self.lib.orc_build_tree_par4(_p(idx), n, _p(b), _p(nodes), cap, leaf, seed) != 0:
            raise RuntimeError("PAR4 node slots exhausted")
        return nodes

    def calc_accel(self, bodies, nodes, theta: float = 0.3) -> np.ndarray:
        b = self._bodies(bodies)
        nodes = np.ascontiguousarray(nodes, dtype=NODE)
        acc = np.zeros((len(b), 3))
        self.lib.orc_calc_accel_all(_p(b), len(b), _p(nodes), theta, _p(acc))
        return acc

    def calc_accel_abs(self, bodies, nodes, theta: float = 0.3):
        """(acc, sum over terms of |term|) per body."""
        b = self._bodies(bodies)
        nodes = np.ascontiguousarray(nodes, dtype=NODE)
        acc = np.zeros((len(b), 3))
        ab = np.zeros(len(b))
        self.lib.orc_calc_accel_abs(_p(b), len(b), _p(nodes), theta, _p(acc), _p(ab))
        return acc, ab

    def calc_accel_sinks(self, bodies, nodes, sinks, theta: float = 0.3):
        """The reference walk for the listed sinks only: (acc, sum of |term|) per sink."""
        b = self._bodies(bodies)
        nodes = np.ascontiguousarray(nodes, dtype=NODE)
        s = np.ascontiguousarray(sinks, dtype=np.uint64)
        acc = np.zeros((len(s), 3))
        ab = np.zeros(len(s))
        self.lib.orc_calc_accel_sinks(_p(b), _p(nodes), theta, _p(s), len(s), _p(acc), _p(ab))
        return acc, ab

    def walk_counts(self, bodies, nodes, sinks, theta: float = 0.3) -> dict:
        b = self._bodies(bodies)
        nodes = np.ascontiguousarray(nodes, dtype=NODE)
        s = np.ascontiguousarray(sinks, dtype=np.uint64)
        out = np.zeros(4, dtype=np.uint64)
        self.lib.orc_walk_counts(_p(b), _p(nodes), theta, _p(s), len(s), _p(out))
        return {"p2p": int(out[0]), "opened": int(out[1]), "m2p": int(out[2]),
                "visits": int(out[3])}

    def groups(self, nodes, n: int):
        """The grouped walk's sink groups over a DFS tree of n bodies: (gstart, gsplit),
        depth-first body positions (make_groups / group_split of kdoracle.c)."""
        nodes = np.ascontiguousarray(nodes, dtype=NODE)
        gstart = np.zeros(n + 1, dtype=np.uint64)
        gsplit = np.zeros(n + 1, dtype=np.uint64)
        ng = self.lib.orc_groups(_p(nodes), len(nodes), n, _p(gstart), _p(gsplit), n + 1)
        if ng == 2 ** 64 - 1:
            raise RuntimeError("orc_groups failed")
        return gstart[: ng + 1], gsplit[:ng]

    def calc_accel_group(self, bodies, nodes, theta: float = 0.3):
        """FP64 restatement of the grouped walk of the mixed path: sinks in groups of whole
        leaves (depth-first, <= 64 bodies), node accepted for a group when
        size^2 < theta^2 dmin^2 to the group's bounding box.  Returns (acc, counts)."""
        b = self._bodies(bodies)
        nodes = np.ascontiguousarray(nodes, dtype=NODE)
        acc = np.zeros((len(b), 3))
        out = np.zeros(4, dtype=np.uint64)
        if self.lib.orc_calc_accel_group(_p(b), len(b), _p(nodes), len(nodes), theta, _p(acc),
                                         _p(out)):
            raise RuntimeError("orc_calc_accel_group: out of memory")
        return acc, {"p2p": int(out[0]), "tests": int(out[1]), "m2p": int(out[2]),
                     "opened": int(out[3])}

    def simple_sim(self, bodies, dt: float, steps: int, leaf: int = 7, layout: str = "dfs",
                   theta: float = 0.3, seed: int = 1, trace: bool = False):
        """Advance ``bodies`` (a 64-byte record array) in place; with trace=True also return
        every step's accelerations, shape (steps, n, 3)."""
        b = bodies.view(PARTICLE)
        if not b.flags.c_contiguous:
            raise ValueError("bodies must be contiguous")
        n = len(b)
        tr = np.zeros((steps, n, 3)) if trace else None
        rc = self.lib.orc_simple_sim(_p(b), n, dt, steps, leaf, 1 if layout == "par4" else 0,
                                     theta, seed, _p(tr) if trace else None)
        if rc != 0:
            raise RuntimeError(f"orc_simple_sim failed ({rc})")
        return tr

    def direct_accel(self, bodies, sinks) -> np.ndarray:
        b = self._bodies(bodies)
        s = np.ascontiguousarray(sinks, dtype=np.uint64)
        acc = np.zeros((len(s), 3))
        self.lib.orc_direct_accel(_p(b), len(b), _p(s), len(s), _p(acc))
        return acc

    def sampled_step(self, bodies, dt: float, sinks, leaf: int = 7, theta: float = 0.3,
                     seed: int = 1):
        """One timing sample of a simple_sim step on all host threads (advances ``bodies``
        in place): the whole PAR4 build, the walk for ``sinks`` only, the kick-drift of every
        body.  Returns the wall seconds (build, sampled walk, kick-drift)."""
        b = bodies.view(PARTICLE)
        if not b.flags.c_contiguous:
            raise ValueError("bodies must be contiguous")
        s = np.ascontiguousarray(sinks, dtype=np.uint64)
        t = np.zeros(3)
        rc = self.lib.orc_sampled_step(_p(b), len(b), dt, leaf, theta, seed, _p(s), len(s),
                                       _p(t))
        if rc != 0:
            raise RuntimeError(f"orc_sampled_step failed ({rc})")
        return float(t[0]), float(t[1]), float(t[2])

    def direct_accel_abs(self, bodies, sinks):
        """FP64 direct sum for the sinks and, per sink, the sum of its terms' magnitudes."""
        b = self._bodies(bodies)
        s = np.ascontiguousarray(sinks, dtype=np.uint64)
        acc = np.zeros((len(s), 3))
        ab = np.zeros(len(s))
        self.lib.orc_direct_accel_abs(_p(b), len(b), _p(s), len(s), _p(acc), _p(ab))
        return acc, ab

    def adjoint_direct(self, bodies, dt: float, steps: int, target=None, dL_dx=None,
                       dL_dv=None):
        """FP64 direct-sum forward + exact reverse sweep.  With `target` (n,3) the loss is
        (1/n) sum |x_T - target|^2.  Returns dict(g_x0, g_v0, xT, loss)."""
        b = self._bodies(bodies)
        n = len(b)
        gx = np.zeros((n, 3))
        gv = np.zeros((n, 3))
        xT = np.zeros((n, 3))
        loss = np.zeros(1)
        tgt = None if target is None else np.ascontiguousarray(target, dtype=np.float64)
        ldx = None if dL_dx is None else np.ascontiguousarray(dL_dx, dtype=np.float64)
        ldv = None if dL_dv is None else np.ascontiguousarray(dL_dv, dtype=np.float64)
        rc = self.lib.orc_adjoint_direct(_p(b), n, dt, steps, _p(ldx) if ldx is not None else None,
                                         _p(ldv) if ldv is not None else None,
                                         _p(tgt) if tgt is not None else None, _p(loss),
                                         _p(gx), _p(gv), _p(xT))
        if rc != 0:
            raise RuntimeError("orc_adjoint_direct failed")
        return {"g_x0": gx, "g_v0": gv, "xT": xT, "loss": float(loss[0])}

    def tree_jt(self, bodies, nodes, mu, theta: float = 0.3) -> np.ndarray:
        """y = J^T mu over the Barnes-Hut interaction set of the given tree (FP64)."""
        b = self._bodies(bodies)
        nodes = np.ascontiguousarray(nodes, dtype=NODE)
        mu = np.ascontiguousarray(mu, dtype=np.float64)
        y = np.zeros((len(b), 3))
        if self.lib.orc_tree_jt(_p(b), len(b), _p(nodes), len(nodes), theta, _p(mu), _p(y)):
            raise RuntimeError("orc_tree_jt failed")
        return y

    def tree_jt_group(self, bodies, nodes, mu, theta: float = 0.3) -> np.ndarray:
        """y = J^T mu over the grouped interaction set of the mixed path (FP64)."""
        b = self._bodies(bodies)
        nodes = np.ascontiguousarray(nodes, dtype=NODE)
        mu = np.ascontiguousarray(mu, dtype=np.float64)
        y = np.zeros((len(b), 3))
        if self.lib.orc_tree_jt_group(_p(b), len(b), _p(nodes), len(nodes), theta, _p(mu),
                                      _p(y)):
            raise RuntimeError("orc_tree_jt_group failed")
        return y

    def energy(self, bodies):
        b = self._bodies(bodies)
        out = np.zeros(2)
        self.lib.orc_energy(_p(b), len(b), _p(out))
        return float(out[0]), float(out[1])


class _Arr(C.Structure):
    _fields_ = [("size", C.c_size_t), ("ptr", C.c_void_p)]


class RefC:
    """The reference's own C port, compiled from the reference sources (leaf 7, DFS
    numbering, sequential build with rand() pivots, OpenMP walk)."""

    MAX_PARTS = 7

    def __init__(self):
        path = _build.build_ref()
        if path is None or not Path(path).exists():
            raise FileNotFoundError("reference C port not built (reference checkout absent)")
        lib = C.CDLL(str(path))
        lib.build_tree.restype = C.c_size_t
        lib.build_tree.argtypes = [C.POINTER(_Arr), C.c_size_t, C.c_size_t, C.POINTER(_Arr),
                                   C.c_size_t, C.POINTER(_Arr)]
        lib.calc_accel.restype = None
        lib.calc_accel.argtypes = [C.c_size_t, C.POINTER(_Arr), C.POINTER(_Arr), _vp]
        lib.simple_sim.restype = None
        lib.simple_sim.argtypes = [C.POINTER(_Arr), C.c_double, C.c_int]
        lib.allocate_node_vec.restype = _Arr
        lib.allocate_node_vec.argtypes = [C.c_size_t]
        self.lib = lib
        self.libc = C.CDLL(None)
        self.libc.srand.argtypes = [C.c_uint]

    def allocate_node_vec_len(self, n: int) -> int:
        a = self.lib.allocate_node_vec(n)
        size = a.size
        self.libc.free(C.c_void_p(a.ptr))
        return int(size)

    def build_tree(self, bodies, seed: int = 1):
        """Returns (nodes as REF_NODE, last node index, index vector)."""
        b = np.ascontiguousarray(bodies).view(PARTICLE)
        n = len(b)
        self.libc.srand(seed)
        # the C port reallocs its node array on demand (KDTree_resize); give it malloc memory
        nodes_arr = self.lib.allocate_node_vec(n)
        idx = np.arange(n, dtype=np.uint64)
        parts = _Arr(n, b.ctypes.data)
        ind = _Arr(n, idx.ctypes.data)
        last = self.lib.build_tree(C.byref(ind), 0, n, C.byref(parts), 0, C.byref(nodes_arr))
        cnt = last + 1
        buf = (C.c_char * (cnt * REF_NODE.itemsize)).from_address(nodes_arr.ptr)
        nodes = np.frombuffer(bytes(buf), dtype=REF_NODE).copy()
        self.libc.free(C.c_void_p(nodes_arr.ptr))
        return nodes, int(last), idx

    def calc_accel(self, bodies, nodes) -> np.ndarray:
        b = np.ascontiguousarray(bodies).view(PARTICLE)
        nodes = np.ascontiguousarray(nodes, dtype=REF_NODE)
        parts = _Arr(len(b), b.ctypes.data)
        narr = _Arr(len(nodes), nodes.ctypes.data)
        acc = np.zeros((len(b), 3))
        for i in range(len(b)):
            self.lib.calc_accel(i, C.byref(parts), C.byref(narr),
                                C.c_void_p(acc.ctypes.data + 24 * i))
        return acc

    def simple_sim(self, bodies, dt: float, steps: int, seed: int = 1) -> None:
        b = bodies.view(PARTICLE)
        if not b.flags.c_contiguous:
            raise ValueError("bodies must be contiguous")
        self.libc.srand(seed)
        parts = _Arr(len(b), b.ctypes.data)
        self.lib.simple_sim(C.byref(parts), dt, steps)
