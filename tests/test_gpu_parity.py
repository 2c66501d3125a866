"""GPU parity: libkdnbody.so (through its C ABI) against the golden fixtures made by the
reference's own C port and against the oracle.

Bars: node membership, split_dim, split_val and size bit-exact; node mass and centre of
mass within the reference's own sequential-sum bound (moment_rtol); FP64 accelerations
within 1e-12 relative per body (two runs of the reference algorithm with different pivot
seeds already differ by up to ~1e-13: the summation order inside a leaf follows the
pivots); mixed-precision accelerations within 1e-4 relative of an FP64 direct sum."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import (assert_accel_close, check_split_invariant, leaf_map, leaf_sets, rel_err,
                      replay_positions)

pytestmark = pytest.mark.gpu

ACC_RTOL = 1e-12
MIXED_RTOL = 1e-4


def moment_rtol(n):
    """The reference sums a node's masses and mass-weighted positions sequentially over its
    bodies (array_kd_tree.rs:536-547), so its own rounding error on a node of n bodies is up
    to about n * 2^-52 relative; the device sums in tree order.  Node moments are compared
    at that bound (never looser than 1e-12)."""
    return max(1e-12, 2.0 * n * 2.0 ** -52)


def gpu_tree(kd, bodies, leaf=7, layout="dfs", theta=0.3, precision="fp64"):
    s = kd.KDTreeSim(len(bodies), leaf_size=leaf, layout=layout, theta=theta,
                     precision=precision)
    s.set_bodies(bodies)
    last = s.build_tree()
    return s, s.nodes(), last


# ------------------------------------------------------------------ reference test cases

def test_single_node(kd):
    b = kd.two_bodies()
    for layout in ("dfs", "par4"):
        s, nodes, last = gpu_tree(kd, b, leaf=8, layout=layout)
        assert last == 0
        assert nodes[0]["num_parts"] == 2
        assert sorted(nodes[0]["particles"][:2]) == [0, 1]
        acc = s.calc_accel()
        # 1/r^2 pull of each body on the other
        assert np.allclose(acc[0], [1e-20, 0, 0], rtol=1e-15)
        assert np.allclose(acc[1], [-1.0, 0, 0], rtol=1e-15)
        s.close()


def test_two_leaves(kd):
    b = kd.circular_orbits(11, seed=3)
    for layout, leaf in [("dfs", 7), ("par4", 8)]:
        s, nodes, _ = gpu_tree(kd, b, leaf=leaf, layout=layout)
        check_split_invariant(nodes, b)
        assert nodes[0]["num_parts"] == 0
        assert nodes[1]["num_parts"] + nodes[2]["num_parts"] == 12
        s.close()


# ------------------------------------------------------------------ golden (reference C port)

def test_membership_and_accel_vs_golden_every_step(kd, oracle, golden):
    n = int(golden["n"])
    s = kd.KDTreeSim(n, leaf_size=7, layout="dfs", theta=0.3)
    for k, b in enumerate(replay_positions(golden)):
        s.set_bodies(b)
        last = s.build_tree()
        nodes = s.nodes()
        assert last == int(golden["last_node"][k])
        assert np.array_equal(leaf_map(nodes, n), golden["leaf_of"][k]), f"step {k}"
        internal = golden["split_dim"][k] >= 0
        assert np.array_equal(nodes["split_dim"][internal].astype(np.int64),
                              golden["split_dim"][k][internal])
        assert np.array_equal(nodes["split_val"][internal], golden["split_val"][k][internal])
        assert np.allclose(nodes["m"][internal], golden["m"][k][internal], rtol=1e-12, atol=0)
        assert np.allclose(nodes["cm"][internal], golden["cm"][k][internal], rtol=1e-12,
                           atol=1e-15)
        acc = s.calc_accel()
        _, absum = oracle.calc_accel_abs(b, oracle.build_tree_dfs(b, leaf=7)[0], 0.3)
        assert_accel_close(acc, golden["acc"][k], absum, ACC_RTOL)
    s.close()


def test_simple_sim_vs_golden(kd, golden):
    b = golden["init"].copy().view(kd.PARTICLE_DTYPE)
    kd.simple_sim(b, float(golden["dt"]), int(golden["steps"]), leaf_size=7)
    assert np.abs(b["p"] - golden["final"]["p"]).max() < 1e-13
    assert np.abs(b["v"] - golden["final"]["v"]).max() < 1e-11
    assert np.array_equal(b["m"], golden["final"]["m"])
    assert np.array_equal(b["r"], golden["final"]["r"])


# ------------------------------------------------------------------ oracle, larger sizes

@pytest.mark.parametrize("n,leaf,layout,gen", [
    (5001, 7, "dfs", "circ"), (20_000, 8, "par4", "ring"), (100_000, 7, "dfs", "ring"),
    (100_000, 8, "par4", "plummer"), (65_537, 7, "par4", "ring"), (1023, 7, "dfs", "plummer"),
    (1025, 8, "dfs", "ring"), (33_000, 7, "dfs", "plummer"), (2000, 7, "dfs", "plummer"),
    (2560, 8, "par4", "ring"), (1281, 7, "dfs", "circ"),
])
def test_tree_and_accel_vs_oracle(kd, oracle, n, leaf, layout, gen):
    b = {"circ": lambda: kd.circular_orbits(n - 1, seed=n),
         "ring": lambda: kd.ring(n, seed=n),
         "plummer": lambda: kd.plummer(n, seed=n)}[gen]()
    s, nodes, _ = gpu_tree(kd, b, leaf=leaf, layout=layout)
    onodes = (oracle.build_tree_dfs(b, leaf=leaf)[0] if layout == "dfs"
              else oracle.build_tree_par4(b, leaf=leaf))
    assert len(nodes) == len(onodes)
    assert leaf_sets(nodes) == leaf_sets(onodes)
    internal = onodes["num_parts"] == 0
    for f in ("split_dim", "split_val", "size", "left", "right"):
        assert np.array_equal(nodes[f][internal], onodes[f][internal]), f
    tol = moment_rtol(n)
    assert np.allclose(nodes["m"][internal], onodes["m"][internal], rtol=tol, atol=0)
    assert np.allclose(nodes["cm"][internal], onodes["cm"][internal], rtol=tol,
                       atol=tol * np.abs(b["p"]).max())
    acc = s.calc_accel()
    oacc, absum = oracle.calc_accel_abs(b, onodes, 0.3)
    assert_accel_close(acc, oacc, absum, ACC_RTOL)
    s.close()


def test_c2_size_one_million(kd, oracle):
    """1,000,000-body ring, leaf 7, theta 0.3: membership bit-exact against the oracle and
    accelerations of 4,096 sampled bodies within 1e-12."""
    n = 1_000_000
    b = kd.ring(n, seed=2024)
    s, nodes, _ = gpu_tree(kd, b, leaf=7, layout="dfs")
    onodes, _ = oracle.build_tree_dfs(b, leaf=7)
    assert np.array_equal(leaf_map(nodes, n), leaf_map(onodes, n))
    internal = onodes["num_parts"] == 0
    assert np.array_equal(nodes["split_val"][internal], onodes["split_val"][internal])
    acc = s.calc_accel()
    oacc, absum = oracle.calc_accel_abs(b, onodes, 0.3)
    assert_accel_close(acc, oacc, absum, ACC_RTOL)
    s.close()


def test_steps_keep_matching_the_oracle(kd, oracle):
    """Five steps of the step loop on both sides from the same bodies (leaf 8, PAR4)."""
    n = 30_000
    b0 = kd.ring(n, seed=77)
    g = b0.copy()
    kd.simple_sim(g, 1e-3, 5, leaf_size=8)
    o = b0.copy()
    oracle.simple_sim(o, 1e-3, 5, leaf=8, layout="par4")
    assert np.abs(g["p"] - o["p"]).max() < 1e-13
    assert np.abs(g["v"] - o["v"]).max() < 1e-11


# ------------------------------------------------------------------ edge cases

@pytest.mark.parametrize("n", [1, 2, 6, 7, 8, 9, 15, 16, 17])
def test_tiny_sizes(kd, oracle, n):
    b = kd.plummer(max(n, 2), seed=n)[:n].copy()
    for leaf, layout in [(7, "dfs"), (8, "par4")]:
        s, nodes, last = gpu_tree(kd, b, leaf=leaf, layout=layout)
        onodes = (oracle.build_tree_dfs(b, leaf=leaf)[0] if layout == "dfs"
                  else oracle.build_tree_par4(b, leaf=leaf))
        assert leaf_sets(nodes) == leaf_sets(onodes)
        acc = s.calc_accel()
        oacc, absum = oracle.calc_accel_abs(b, onodes, 0.3)
        d = np.linalg.norm(acc - oacc, axis=1)
        assert (d <= 1e-12 * absum).all()
        s.close()


def test_ties_give_a_valid_median_split(kd):
    """Many equal coordinates (a lattice): the reference's own choice among tied bodies
    depends on its random pivots, so the check is the split post-condition with ties:
    left <= split_val <= right, len/2 bodies left, every body exactly once."""
    g = np.arange(40, dtype=np.float64)
    x, y, z = np.meshgrid(g, g, g[:10], indexing="ij")
    n = x.size
    b = np.zeros(n, dtype=kd.PARTICLE_DTYPE)
    b["p"] = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
    b["m"] = 1.0
    s, nodes, _ = gpu_tree(kd, b, leaf=7)
    members = np.concatenate([nd["particles"][: nd["num_parts"]] for nd in nodes
                              if nd["num_parts"] > 0])
    assert np.array_equal(np.sort(members), np.arange(n))
    p = b["p"]

    def collect(i):
        nd = nodes[i]
        if nd["num_parts"] > 0:
            return list(nd["particles"][: nd["num_parts"]])
        return collect(int(nd["left"])) + collect(int(nd["right"]))

    for i, nd in enumerate(nodes[:200]):
        if nd["num_parts"] == 0:
            d, sv = int(nd["split_dim"]), nd["split_val"]
            L = np.array(collect(int(nd["left"])), dtype=np.int64)
            R = np.array(collect(int(nd["right"])), dtype=np.int64)
            assert len(L) == (len(L) + len(R)) // 2
            assert (p[L, d] <= sv).all() and (p[R, d] >= sv).all()
    s.close()


def test_invalid_bodies_are_rejected(kd):
    b = kd.ring(1000, seed=1)
    s = kd.KDTreeSim(1000)
    bad = b.copy()
    bad["p"][10, 1] = np.nan
    with pytest.raises(kd.KDError) as e:
        s.set_bodies(bad)
    assert "KD_ENUMERIC" in str(e.value)
    bad = b.copy()
    bad["m"][3] = -1.0
    with pytest.raises(kd.KDError):
        s.set_bodies(bad)
    with pytest.raises(kd.KDError):
        s.set_bodies(b[:999])
    with pytest.raises(kd.KDError):
        s.build_tree()  # no valid bodies yet
    s.set_bodies(b)
    s.build_tree()
    s.close()


# ------------------------------------------------------------------ mixed precision

def test_mixed_precision_vs_direct_sum(kd, oracle):
    n = 200_000
    b = kd.ring(n, seed=31)
    s = kd.KDTreeSim(n, leaf_size=7, precision="mixed")
    s.set_bodies(b)
    s.build_tree()
    acc = s.calc_accel()
    rng = np.random.default_rng(4)
    sinks = np.concatenate([[0], rng.choice(np.arange(1, n), 4095, replace=False)])
    ref = oracle.direct_accel(b, sinks)
    err = rel_err(acc[sinks], ref)
    assert err.max() <= MIXED_RTOL, err.max()
    s.set_precision("fp64")
    acc64 = s.calc_accel()
    # against the FP64 tree: equal to theta truncation, except body 0, whose mixed value is
    # its direct sum and whose tree value carries the tree's truncation of a cancelling sum
    assert rel_err(acc[sinks[1:]], acc64[sinks[1:]]).max() <= MIXED_RTOL
    s.close()


def test_mixed_precision_plummer(kd, oracle):
    """Equal-mass sphere (no heavy body): the FP32 terms carry everything.  Compared with
    the oracle's FP64 grouped walk (the same interaction set), so the check isolates the
    precision error from the theta error; the rare node whose FP32 group test falls the
    other way than the FP64 one shows in the maximum only."""
    n = 100_000
    b = kd.plummer(n, seed=41)
    s = kd.KDTreeSim(n, leaf_size=7, precision="mixed", theta=0.5)
    s.set_bodies(b)
    s.build_tree()
    acc = s.calc_accel()
    s.close()
    nodes, _ = oracle.build_tree_dfs(b, leaf=7)
    ref, _ = oracle.calc_accel_group(b, nodes, 0.5)
    err = rel_err(acc, ref)
    assert np.sqrt(np.mean(err ** 2)) <= 1e-5
    assert np.median(err) <= 1e-6
    assert err.max() <= 1e-3


@pytest.mark.parametrize("gen,n,theta", [("ring", 200_000, 0.3), ("plummer", 50_000, 0.5),
                                         ("plummer", 3_000, 0.0), ("ring", 5, 0.3),
                                         ("ring", 33, 0.3)])
def test_grouped_walk_matches_oracle(kd, oracle, gen, n, theta):
    """The mixed path's grouped walk against its FP64 restatement: accelerations and the
    interaction counts (the group test in FP32 may decide a borderline node differently)."""
    b = kd.ring(n, seed=52) if gen == "ring" else kd.plummer(n, seed=52)
    with kd.KDTreeSim(n, leaf_size=7, precision="mixed", theta=theta) as s:
        s.set_bodies(b)
        s.build_tree()
        s.set_counting(True)
        acc = s.calc_accel()
        cnt = s.counts()
    nodes, _ = oracle.build_tree_dfs(b, leaf=7)
    ref, rc = oracle.calc_accel_group(b, nodes, theta)
    # the ring's central body is a heavy body: its mixed acceleration is its FP64 direct sum
    # (tests/test_gpu_direct.py), not the grouped walk's value
    err = rel_err(acc, ref)[1:] if gen == "ring" else rel_err(acc, ref)
    assert np.sqrt(np.mean(err ** 2)) <= 1e-5, np.sqrt(np.mean(err ** 2))
    assert err.max() <= 1e-3, err.max()
    inter, rinter = cnt["p2p"] + cnt["m2p"], rc["p2p"] + rc["m2p"]
    assert abs(inter - rinter) <= 1e-3 * rinter, (cnt, rc)
    assert abs(cnt["opened"] - rc["tests"]) <= 1e-3 * rc["tests"] + 2, (cnt, rc)
    if theta == 0.0:
        assert cnt["m2p"] == 0 and cnt["p2p"] == n * (n - 1)


# ------------------------------------------------------------------ energy diagnostic

@pytest.mark.parametrize("gen,theta,tol", [("ring", 0.3, 1e-9), ("plummer", 0.3, 1e-3),
                                           ("plummer", 0.0, 1e-6)])
def test_energy_matches_direct_sum(kd, oracle, gen, theta, tol):
    n = 3000
    b = kd.ring(n, seed=9) if gen == "ring" else kd.plummer(n, seed=9)
    with kd.KDTreeSim(n, theta=theta) as s:
        s.set_bodies(b)
        ke, pe = s.energy()
    rke, rpe = oracle.energy(b)
    assert ke == pytest.approx(rke, rel=1e-12)
    assert pe == pytest.approx(rpe, rel=tol)


# ------------------------------------------------------------------ 1M-body FP64 run

def assert_same_slots(nodes, onodes):
    """Node arrays equal slot by slot: leaf membership (as sets: the order inside a leaf
    follows the reference's pivots), split_dim, split_val, size and child slots of every
    internal node; unused PAR4 slots on both sides."""
    assert len(nodes) == len(onodes)
    assert np.array_equal(nodes["num_parts"], onodes["num_parts"])
    k = nodes["num_parts"].astype(np.int64)
    used = np.arange(nodes["particles"].shape[1])[None, :] < k[:, None]
    big = np.iinfo(np.uint64).max
    a = np.sort(np.where(used, nodes["particles"], big), axis=1)
    o = np.sort(np.where(used, onodes["particles"], big), axis=1)
    assert np.array_equal(a, o), "leaf membership differs"
    internal = (onodes["num_parts"] == 0) & ((onodes["left"] != 0) | (onodes["right"] != 0))
    assert np.array_equal(internal, (nodes["num_parts"] == 0) &
                          ((nodes["left"] != 0) | (nodes["right"] != 0)))
    for f in ("split_dim", "split_val", "size", "left", "right"):
        assert np.array_equal(nodes[f][internal], onodes[f][internal]), f


def test_fp64_1M_ring_100_steps_every_step(kd, oracle):
    """The 1,000,000-body ring on the FP64 GPU path for 100 steps (theta 0.3, leaf 7,
    dt 1e-3, PAR4 numbering).  At EVERY step the oracle rebuilds the tree from the GPU's own
    state: node slots bit-exact (membership, split_dim, split_val, size, children), and the
    accelerations of 512 seeded sinks per step within 1e-12 of the oracle walk -- the
    reference's big_solar_with_steps (array_kd_tree.rs:816-832) at the BASELINE's size."""
    n, steps = 1_000_000, 100
    b = kd.ring(n, seed=13)
    rng = np.random.default_rng(14)
    with kd.KDTreeSim(n, leaf_size=7, layout="par4", precision="fp64", theta=0.3) as s:
        s.set_bodies(b)
        for step in range(steps):
            state = s.get_bodies()
            s.build_tree()
            nodes = s.nodes()
            acc = s.calc_accel()
            onodes = oracle.build_tree_par4(state, leaf=7)
            assert_same_slots(nodes, onodes)
            sinks = np.sort(rng.choice(n, 512, replace=False)).astype(np.uint64)
            oacc, absum = oracle.calc_accel_sinks(state, onodes, sinks, 0.3)
            got = acc[sinks.astype(np.int64)]
            d = np.linalg.norm(got - oacc, axis=1)
            assert (d <= 1e-12 * absum).all(), (step, (d / absum).max())
            a = np.linalg.norm(oacc, axis=1)
            well = absum <= 100.0 * a
            assert (d[well] <= 1e-12 * a[well]).all(), (step, (d[well] / a[well]).max())
            s.simple_sim(1e-3, 1)
        final = s.get_bodies()
    assert np.isfinite(final["p"]).all() and np.isfinite(final["v"]).all()


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_graph_steps_match_direct_launches(kd, precision):
    """kd_simple_sim replays one captured step (a CUDA graph); with timing on it launches
    every kernel directly.  Both give bit-identical states, also across a change of dt (the
    graph is captured again)."""
    n = 20_000
    b = kd.plummer(n, seed=3)
    with kd.KDTreeSim(n, leaf_size=7, precision=precision, theta=0.5) as s:
        s.set_bodies(b)
        s.simple_sim(1e-3, 3)
        s.simple_sim(2e-3, 2)
        graph = s.get_bodies().copy()
        s.set_bodies(b)
        s.set_timing(True)
        s.simple_sim(1e-3, 3)
        s.simple_sim(2e-3, 2)
        s.set_timing(False)
        direct = s.get_bodies().copy()
    assert np.array_equal(graph["p"], direct["p"]) and np.array_equal(graph["v"], direct["v"])
