"""GPU adjoint (kd_forward / kd_backward) against the oracle and finite differences.

* The transpose-Jacobian product of one step: with steps=1, dt=1 and dL/dv=0, the backward
  sweep returns g_x0 = r + J(x0)^T r for dL/dx = r, which is compared with the oracle's FP64
  J^T r over the grouped interaction set of the mixed walk (the oracle's J^T is pinned at
  theta=0 against the direct-sum adjoint in tests/test_oracle_adjoint.py).
* Whole sweeps: against the oracle's FP64 direct-sum adjoint, and against central finite
  differences (h = 1e-6) of the GPU forward on seeded coordinates of v0.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rot_z(p, ang=1.0):
    c, s = np.cos(ang), np.sin(ang)
    R = np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]])
    return p @ R.T


def rel_rows(a, b):
    return np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)


def gpu_grad(kd, bodies, dt, steps, target, theta=0.3, ckpt=32):
    n = len(bodies)
    with kd.KDTreeSim(n, leaf_size=7, precision="mixed", theta=theta) as s:
        s.set_bodies(bodies)
        with s.forward(dt, steps, ckpt) as tape:
            xT = s.get_bodies()["p"].copy()
            dLdx = 2.0 * (xT - target) / n
            gx, gv = tape.backward(dLdx)
            gx2, gv2 = tape.backward(dLdx)
            after = s.get_bodies()["p"].copy()
    # the source-side sums are FP64 atomics in no fixed order: repeated sweeps agree to their
    # rounding, not bit for bit
    assert np.allclose(gv, gv2, rtol=1e-6, atol=1e-6 * np.abs(gv).max())
    assert np.allclose(gx, gx2, rtol=1e-6, atol=1e-6 * np.abs(gx).max())
    assert np.array_equal(after, xT), "backward must leave the final state in place"
    return gx, gv, xT


@pytest.mark.parametrize("theta", [0.3, 0.5])
def test_one_step_jt_matches_oracle_tree(kd, oracle, theta):
    n = 20_000
    b = kd.plummer(n, seed=5)
    rng = np.random.default_rng(2)
    r = rng.normal(size=(n, 3))
    with kd.KDTreeSim(n, leaf_size=7, precision="mixed", theta=theta) as s:
        s.set_bodies(b)
        with s.forward(1.0, 1, 1) as tape:
            gx, gv = tape.backward(r)
    assert np.array_equal(gv, r)
    jt = gx - r
    nodes, _ = oracle.build_tree_dfs(b, leaf=7)
    ref = oracle.tree_jt_group(b, nodes, r, theta)
    e = rel_rows(jt, ref)
    # FP32 arithmetic, and the rare node whose FP32 group test differs from FP64
    assert np.sqrt(np.mean(e ** 2)) <= 1e-4, np.sqrt(np.mean(e ** 2))
    assert np.median(e) <= 1e-5, np.median(e)


def test_theta_zero_sweep_matches_direct_sum_adjoint(kd, oracle):
    n = 3000
    b = kd.plummer(n, seed=6)
    tgt = rot_z(b["p"])
    gx, gv, xT = gpu_grad(kd, b, 1e-3, 20, tgt, theta=0.0, ckpt=8)
    ref = oracle.adjoint_direct(b, 1e-3, 20, target=tgt)
    assert np.abs(xT - ref["xT"]).max() < 1e-8  # FP32 pair forces in the forward
    assert rel_rows(gv, ref["g_v0"]).max() <= 1e-5
    assert rel_rows(gx, ref["g_x0"]).max() <= 1e-5


def test_ring_sweep_matches_direct_sum_adjoint(kd, oracle):
    """2,000-body ring, theta 0.3, 100 steps, checkpoints every 32 steps."""
    n = 2000
    b = kd.ring(n, seed=7)
    tgt = rot_z(b["p"])
    gx, gv, xT = gpu_grad(kd, b, 1e-3, 100, tgt)
    ref = oracle.adjoint_direct(b, 1e-3, 100, target=tgt)
    e = rel_rows(gv, ref["g_v0"])
    assert e.max() <= 1e-5, e.max()
    assert rel_rows(gx, ref["g_x0"]).max() <= 1e-5


def test_long_ring_sweep_matches_direct_sum_adjoint(kd, oracle):
    """2,000-body ring, theta 0.3, 1,000 steps, checkpoints every 32 steps: the sweep length
    of the 100,000-body gradient check, at a size the FP64 direct-sum adjoint finishes."""
    n = 2000
    b = kd.ring(n, seed=11)
    tgt = rot_z(b["p"])
    gx, gv, xT = gpu_grad(kd, b, 1e-3, 1000, tgt)
    ref = oracle.adjoint_direct(b, 1e-3, 1000, target=tgt)
    assert rel_rows(gv, ref["g_v0"]).max() <= 1e-4
    assert np.median(rel_rows(gv, ref["g_v0"])) <= 1e-5
    assert rel_rows(gx, ref["g_x0"]).max() <= 1e-4


def test_ring_sweep_matches_finite_differences(kd):
    """Central differences (h = 1e-6) of the GPU forward on 16 seeded coordinates of v0.  The
    loss difference is summed per body so that the bodies the perturbation does not reach
    cancel exactly."""
    n, steps, dt, h = 2000, 100, 1e-3, 1e-6
    b = kd.ring(n, seed=8)
    tgt = rot_z(b["p"])
    gx, gv, _ = gpu_grad(kd, b, dt, steps, tgt)
    rng = np.random.default_rng(9)
    coords = [(int(i), int(d)) for i, d in zip(rng.choice(np.arange(1, n), 16, replace=False),
                                             rng.integers(0, 2, 16))]
    with kd.KDTreeSim(n, leaf_size=7, precision="mixed") as s:
        def final(bb):
            s.set_bodies(bb)
            s.simple_sim(dt, steps)
            return s.get_bodies()["p"].copy()
        for i, d in coords:
            bp = b.copy(); bp["v"][i, d] += h
            bm = b.copy(); bm["v"][i, d] -= h
            xp, xm = final(bp), final(bm)
            lp = np.sum((xp - tgt) ** 2, axis=1)
            lm = np.sum((xm - tgt) ** 2, axis=1)
            fd = np.sum(lp - lm) / n / (2 * h)
            assert abs(fd - gv[i, d]) <= 1e-5 * abs(gv[i, d]) + 1e-12, (i, d, fd, gv[i, d])


def test_adjoint_needs_mixed_precision(kd):
    b = kd.ring(100, seed=1)
    with kd.KDTreeSim(100, precision="fp64") as s:
        s.set_bodies(b)
        with pytest.raises(kd.KDError):
            s.forward(1e-3, 2, 1)


def test_kept_last_segment_matches_recompute(kd):
    """The forward sweep leaves its last segment's positions for the backward sweep; once
    another sweep has replaced them the segment is recomputed, with the same gradients."""
    n = 3000
    b = kd.plummer(n, seed=12)
    r = np.random.default_rng(3).normal(size=(n, 3))
    with kd.KDTreeSim(n, leaf_size=7, precision="mixed", theta=0.5) as s:
        s.set_bodies(b)
        with s.forward(1e-3, 10, 32) as ta:
            gx1, gv1 = ta.backward(r)           # last segment kept from the forward
            with s.forward(1e-3, 10, 32):       # replaces the kept positions
                pass
            gx2, gv2 = ta.backward(r)           # recomputed from the checkpoint
    assert np.allclose(gx1, gx2, rtol=1e-9, atol=1e-12 * np.abs(gx1).max())
    assert np.allclose(gv1, gv2, rtol=1e-9, atol=1e-12 * np.abs(gv1).max())
