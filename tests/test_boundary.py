"""CPU tests of the drop-in boundary: libkdnbody.so builds for sm_103a, loads, exports every
entry point include/kdnbody.h declares, and its host-only calls behave (no GPU needed)."""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "kdnbody.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w \*]*?\b(kd_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from multilanguagekdtree_gb300 import _lib, build_ext
    build_ext.build()
    return _lib.load()


def test_header_declares_the_reference_call_shape():
    names = declared_functions()
    for must in ["kd_create", "kd_destroy", "kd_set_bodies", "kd_get_bodies", "kd_build_tree",
                 "kd_get_nodes", "kd_calc_accel", "kd_simple_sim", "kd_nodes_needed",
                 "kd_last_error"]:
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_python_binding_covers_every_symbol():
    from multilanguagekdtree_gb300 import _lib
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_library_is_sm103a():
    # the fat binary must carry sm_103a code (checked through the build flags we pass)
    from multilanguagekdtree_gb300 import build_ext
    assert "arch=compute_103a,code=sm_103a" in build_ext.ARCH


def test_nodes_needed_matches_oracle(lib, oracle):
    for n in [1, 2, 7, 8, 9, 12, 100, 1000, 5001, 65537, 1_000_000, 10_000_000]:
        for leaf in (7, 8):
            assert lib.kd_nodes_needed(n, leaf, 1) == oracle.nodes_needed_par(n, leaf)
            assert lib.kd_nodes_needed(n, leaf, 0) == oracle.nodes_needed_seq(n, leaf)
    assert lib.kd_nodes_needed(10, 1, 0) == 0  # leaf size out of range


def test_create_rejects_bad_arguments_without_a_gpu(lib):
    from multilanguagekdtree_gb300 import _lib
    p = _lib.KdParams()
    lib.kd_default_params(C.byref(p))
    assert p.leaf_size == 7 and p.theta == 0.3 and p.dt == 1e-3
    assert lib.kd_create(0, C.byref(p)) is None
    assert b"n must be" in lib.kd_last_error(None)
    p.leaf_size = 9
    assert lib.kd_create(10, C.byref(p)) is None
    assert b"leaf_size" in lib.kd_last_error(None)
    p.leaf_size = 7
    p.layout = 5
    assert lib.kd_create(10, C.byref(p)) is None
    # NULL context arguments are rejected, never dereferenced
    assert lib.kd_set_bodies(None, None, 0) == _lib.KD_EINVAL
    assert lib.kd_build_tree(None, None) == _lib.KD_EINVAL
    assert lib.kd_simple_sim(None, 0.0, 1) == _lib.KD_EINVAL


def test_python_api_raises_kderror():
    import multilanguagekdtree_gb300 as kd
    with pytest.raises(kd.KDError):
        kd.KDTreeSim(0)
