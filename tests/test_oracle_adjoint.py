"""CPU tests pinning the oracle's adjoints: the direct-sum reverse sweep against central
finite differences, and the Barnes-Hut transpose-Jacobian product against the direct sum
at theta = 0 (where the tree walk makes every pair interaction)."""
from __future__ import annotations

import numpy as np

from multilanguagekdtree_gb300.array_particle import plummer, ring


def rot_z(p, ang=1.0):
    c, s = np.cos(ang), np.sin(ang)
    return p @ np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]]).T


def test_direct_adjoint_matches_finite_differences(oracle):
    b = ring(300, seed=3)
    dt, steps, h = 1e-3, 30, 1e-6
    tgt = rot_z(b["p"])
    g = oracle.adjoint_direct(b, dt, steps, target=tgt)

    def per_body_loss(bb):
        return np.sum((oracle.adjoint_direct(bb, dt, steps, target=tgt)["xT"] - tgt) ** 2, axis=1)

    for i, d in [(5, 0), (17, 1), (101, 0), (250, 1)]:
        bp = b.copy(); bp["v"][i, d] += h
        bm = b.copy(); bm["v"][i, d] -= h
        fd = np.sum(per_body_loss(bp) - per_body_loss(bm)) / len(b) / (2 * h)
        assert abs(fd - g["g_v0"][i, d]) <= 1e-6 * abs(g["g_v0"][i, d]), (i, d, fd)
    # x0 gradient as well
    i, d = 42, 0
    bp = b.copy(); bp["p"][i, d] += h
    bm = b.copy(); bm["p"][i, d] -= h
    fd = np.sum(per_body_loss(bp) - per_body_loss(bm)) / len(b) / (2 * h)
    # the targets are constants: only x_T moves with x0
    assert abs(fd - g["g_x0"][i, d]) <= 1e-6 * abs(g["g_x0"][i, d])


def test_tree_jt_is_exact_at_theta_zero(oracle):
    b = plummer(1500, seed=4)
    nodes, _ = oracle.build_tree_dfs(b)
    mu = np.random.default_rng(1).normal(size=(len(b), 3))
    y = oracle.tree_jt(b, nodes, mu, theta=0.0)
    ref = oracle.adjoint_direct(b, 1.0, 1, dL_dx=mu)["g_x0"] - mu
    e = np.linalg.norm(y - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert e.max() <= 1e-12


def test_tree_jt_approximates_direct_sum(oracle):
    b = plummer(3000, seed=5)
    nodes, _ = oracle.build_tree_dfs(b)
    mu = np.random.default_rng(2).normal(size=(len(b), 3))
    ref = oracle.adjoint_direct(b, 1.0, 1, dL_dx=mu)["g_x0"] - mu
    y = oracle.tree_jt(b, nodes, mu, theta=0.3)
    e = np.linalg.norm(y - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert np.sqrt(np.mean(e ** 2)) < 1e-2  # monopole truncation of the tidal tensors


def test_grouped_tree_jt_is_exact_at_theta_zero(oracle):
    b = plummer(1500, seed=4)
    nodes, _ = oracle.build_tree_dfs(b)
    mu = np.random.default_rng(1).normal(size=(len(b), 3))
    y = oracle.tree_jt_group(b, nodes, mu, theta=0.0)
    ref = oracle.adjoint_direct(b, 1.0, 1, dL_dx=mu)["g_x0"] - mu
    e = np.linalg.norm(y - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert e.max() <= 1e-12


def test_grouped_tree_jt_approximates_direct_sum(oracle):
    b = plummer(3000, seed=5)
    nodes, _ = oracle.build_tree_dfs(b)
    mu = np.random.default_rng(2).normal(size=(len(b), 3))
    ref = oracle.adjoint_direct(b, 1.0, 1, dL_dx=mu)["g_x0"] - mu
    y = oracle.tree_jt_group(b, nodes, mu, theta=0.3)
    e = np.linalg.norm(y - ref, axis=1) / np.linalg.norm(ref, axis=1)
    y1 = oracle.tree_jt(b, nodes, mu, theta=0.3)
    e1 = np.linalg.norm(y1 - ref, axis=1) / np.linalg.norm(ref, axis=1)
    # the grouped set refines the reference walk's: no larger truncation error overall
    assert np.sqrt(np.mean(e ** 2)) <= np.sqrt(np.mean(e1 ** 2))
