"""GPU selection with the post-condition of the reference's quickstat_index
(MarkCLewis/MultiLanguageKDTree Parallel/RustVersion/src/quickstat.rs:9-34).

``quickstat_index(vals, goal, indices=None)`` returns the index vector reordered so that
``vals[idx[i]] < vals[idx[goal]]`` for ``i < goal`` and ``>=`` for ``i >= goal`` (the
comparator ``|i1, i2| vals[i1] < vals[i2]`` of the reference's tests and benchmark).  The
selection runs on the GPU (libkdnbody.so); equal values are ordered by index value.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

__all__ = ["quickstat_index"]


def quickstat_index(vals, goal: int, indices=None, device: int = 0, timing: bool = False):
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    idx = (np.arange(len(vals), dtype=np.uint64) if indices is None
           else np.array(indices, dtype=np.uint64, copy=True))
    ms = C.c_double(0.0)
    lib = _lib.load()
    rc = lib.kd_quickstat_index(_lib.ptr(vals), len(vals), _lib.ptr(idx), len(idx), int(goal),
                                device, C.byref(ms))
    _lib.check(rc, None)
    return (idx, ms.value) if timing else idx
