"""ctypes binding of libkdnbody.so (declared in include/kdnbody.h).

Loading fails loudly when the library is missing: there is no CPU fallback anywhere in this
package.  Build it with ``python -m multilanguagekdtree_gb300.build_ext`` or
``__graft_entry__.build()``.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libkdnbody.so"

KD_OK = 0
KD_EINVAL = -1
KD_ENOMEM = -2
KD_ECUDA = -3
KD_ESTATE = -4
KD_ENUMERIC = -5
KD_EOVERFLOW = -6
KD_EDEVICE = -7
KD_MAX_LEAF = 8
KD_LAYOUT_DFS = 0
KD_LAYOUT_PAR4 = 1
KD_PREC_FP64 = 0
KD_PREC_MIXED = 1
KD_GEN_RING = 0
KD_GEN_PLUMMER = 1
KD_GEN_CIRCULAR = 2

ERROR_NAMES = {
    KD_EINVAL: "KD_EINVAL", KD_ENOMEM: "KD_ENOMEM", KD_ECUDA: "KD_ECUDA",
    KD_ESTATE: "KD_ESTATE", KD_ENUMERIC: "KD_ENUMERIC", KD_EOVERFLOW: "KD_EOVERFLOW",
    KD_EDEVICE: "KD_EDEVICE",
}

# kd_particle_c: Particle of Parallel/RustVersion/src/array_particle.rs:3-8
PARTICLE_DTYPE = np.dtype([("p", "<f8", (3,)), ("v", "<f8", (3,)), ("r", "<f8"), ("m", "<f8")])
assert PARTICLE_DTYPE.itemsize == 64

# kd_node_c: KDTree of Parallel/CVersion/src/kdtree.h:9-22 with 8 leaf slots
NODE_DTYPE = np.dtype([
    ("num_parts", "<u8"), ("particles", "<u8", (KD_MAX_LEAF,)), ("split_dim", "<u8"),
    ("split_val", "<f8"), ("m", "<f8"), ("cm", "<f8", (3,)), ("size", "<f8"),
    ("left", "<u8"), ("right", "<u8"),
])


class KdParams(C.Structure):
    _fields_ = [("leaf_size", C.c_int32), ("layout", C.c_int32), ("precision", C.c_int32),
                ("device", C.c_int32), ("theta", C.c_double), ("dt", C.c_double),
                ("heavy_frac", C.c_double), ("seed", C.c_uint64)]


class KdStats(C.Structure):
    _fields_ = [("build_ms", C.c_double), ("moments_ms", C.c_double), ("walk_ms", C.c_double),
                ("kick_ms", C.c_double), ("total_ms", C.c_double), ("steps", C.c_uint64),
                ("launches", C.c_uint64)]


class KDError(RuntimeError):
    """A libkdnbody call returned a negative status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERROR_NAMES.get(code, code)}: {msg}")
        self.code = code


# name -> (restype, argtypes)
SIGNATURES = {
    "kd_default_params": (None, [C.POINTER(KdParams)]),
    "kd_nodes_needed": (C.c_size_t, [C.c_size_t, C.c_int32, C.c_int32]),
    "kd_group_plan": (C.c_int, [C.c_size_t, C.c_int32, C.POINTER(C.c_uint32),
                                C.POINTER(C.c_uint32), C.c_size_t, C.POINTER(C.c_size_t)]),
    "kd_create": (C.c_void_p, [C.c_size_t, C.POINTER(KdParams)]),
    "kd_destroy": (None, [C.c_void_p]),
    "kd_last_error": (C.c_char_p, [C.c_void_p]),
    "kd_set_bodies": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "kd_get_bodies": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "kd_generate": (C.c_int, [C.c_void_p, C.c_int32, C.c_uint64]),
    "kd_build_tree": (C.c_int, [C.c_void_p, C.POINTER(C.c_size_t)]),
    "kd_get_nodes": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t)]),
    "kd_calc_accel": (C.c_int, [C.c_void_p, C.c_void_p]),
    "kd_print_tree": (C.c_int, [C.c_void_p, C.c_char_p]),
    "kd_quickstat_index": (C.c_int, [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_size_t,
                                     C.c_int32, C.POINTER(C.c_double)]),
    "kd_simple_sim": (C.c_int, [C.c_void_p, C.c_double, C.c_int64]),
    "kd_set_precision": (C.c_int, [C.c_void_p, C.c_int32]),
    "kd_energy": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "kd_get_stats": (C.c_int, [C.c_void_p, C.POINTER(KdStats)]),
    "kd_set_timing": (C.c_int, [C.c_void_p, C.c_int32]),
    "kd_direct_accel": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]),
    "kd_forward": (C.c_int, [C.c_void_p, C.c_double, C.c_int64, C.c_int64,
                             C.POINTER(C.c_void_p)]),
    "kd_backward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "kd_tape_free": (None, [C.c_void_p]),
    "kd_direct_accel_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_size_t, C.c_void_p, C.c_size_t, C.c_void_p,
                                          C.c_void_p]),
    "kd_set_device_limits": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "kd_fp32_peak": (C.c_int, [C.c_int32, C.POINTER(C.c_double)]),
    "kd_set_counting": (C.c_int, [C.c_void_p, C.c_int32]),
    "kd_get_counts": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64)]),
}

_lib = None


def load() -> C.CDLL:
    """Load libkdnbody.so (once).  Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build it first "
                               "(python -m multilanguagekdtree_gb300.build_ext)")
        lib = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def check(rc: int, ctx) -> None:
    if rc != KD_OK:
        msg = load().kd_last_error(ctx)
        raise KDError(rc, msg.decode() if msg else "")


def ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)
