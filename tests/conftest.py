"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on a CPU-only box."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libkdnbody.so")


@pytest.fixture(scope="session")
def oracle():
    from oracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def refc():
    from oracle import RefC
    try:
        return RefC()
    except FileNotFoundError as e:
        pytest.skip(str(e))


@pytest.fixture(scope="session")
def golden():
    z = np.load(GOLDEN / "ring1000.npz")
    from oracle import PARTICLE
    d = {k: z[k] for k in z.files}
    d["init"] = d["init"].view(PARTICLE)
    d["final"] = d["final"].view(PARTICLE)
    d["ref_simple_sim_final"] = d["ref_simple_sim_final"].view(PARTICLE)
    return d


@pytest.fixture(scope="session")
def kd():
    """The GPU library (built if stale).  Only GPU tests use this fixture."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from multilanguagekdtree_gb300 import build_ext
    build_ext.build()
    import multilanguagekdtree_gb300 as kd
    return kd


def replay_positions(golden):
    """Bodies at the start of every golden step: the reference's kick-drift (IEEE order,
    kdtree.c:296-305) applied to the recorded accelerations."""
    b = golden["init"].copy()
    out = []
    dt = float(golden["dt"])
    for k in range(int(golden["steps"])):
        out.append(b.copy())
        b["v"] = b["v"] + dt * golden["acc"][k]
        b["p"] = b["p"] + dt * b["v"]
    return out


def leaf_map(nodes, n):
    leaf_of = np.full(n, -1, dtype=np.int64)
    for i, nd in enumerate(nodes):
        k = int(nd["num_parts"])
        if k > 0:
            leaf_of[nd["particles"][:k].astype(np.int64)] = i
    return leaf_of


def leaf_sets(nodes):
    """Canonical membership: the sorted member list of every leaf, keyed by node index."""
    out = {}
    for i, nd in enumerate(nodes):
        k = int(nd["num_parts"])
        if k > 0:
            out[i] = tuple(sorted(int(x) for x in nd["particles"][:k]))
    return out


def rel_err(a, b):
    """Per-body |a-b| / |b| (b the reference)."""
    num = np.linalg.norm(a - b, axis=-1)
    den = np.linalg.norm(b, axis=-1)
    return num / np.where(den > 0, den, 1.0)


def assert_accel_close(acc, ref, absum, rtol=1e-12, kappa=100.0):
    """FP64 acceleration parity.  Different summation orders of the same terms differ by
    rounding proportional to the sum of the terms' magnitudes (absum), so:
    |da| <= rtol * |a| for every body whose sum is well conditioned (absum <= kappa |a|), and
    |da| <= rtol * absum for every body (e.g. a central mass whose pulls nearly cancel)."""
    d = np.linalg.norm(acc - ref, axis=-1)
    a = np.linalg.norm(ref, axis=-1)
    well = absum <= kappa * a
    assert well.mean() > 0.5, "too few well-conditioned bodies for a relative check"
    rel = d[well] / a[well]
    assert rel.max() <= rtol, f"max relative error {rel.max():.3e} > {rtol}"
    scaled = d / np.where(absum > 0, absum, 1.0)
    assert scaled.max() <= rtol, f"max error / sum|terms| {scaled.max():.3e} > {rtol}"
    return rel.max(), scaled.max()


def check_split_invariant(nodes, bodies, root=0):
    """The reference's recur_test_tree_struct (array_kd_tree.rs:834-877), on all three
    dimensions: every body under the left child is < split_val, every body under the right
    child is >= split_val, along that node's split_dim."""
    p = bodies["p"]
    stack = [(root, np.full(3, -np.inf), np.full(3, np.inf))]
    while stack:
        i, lo, hi = stack.pop()
        nd = nodes[i]
        k = int(nd["num_parts"])
        if k > 0:
            q = p[nd["particles"][:k].astype(np.int64)]
            assert (q >= lo).all() and (q < hi).all(), (i, q, lo, hi)
        else:
            d = int(nd["split_dim"])
            sv = float(nd["split_val"])
            h2 = hi.copy(); h2[d] = sv
            l2 = lo.copy(); l2[d] = sv
            stack.append((int(nd["left"]), lo, h2))
            stack.append((int(nd["right"]), l2, hi))
