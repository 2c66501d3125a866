"""CPU tests of the oracle: pinned against the reference's own C port (compiled from the
reference sources into oracle/_ref), the golden fixtures that port produced, and the known
answers and structural cases of the reference's own tests."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import (assert_accel_close, check_split_invariant, leaf_map, leaf_sets, rel_err,
                      replay_positions)
from multilanguagekdtree_gb300.array_particle import circular_orbits, plummer, ring, two_bodies


# ------------------------------------------------------------------ quickstat (quickstat.rs)

@pytest.mark.parametrize("seed", [1, 2, 3, 17, 12345])
def test_quickstat_small_known_answer(oracle, seed):
    # quickstat.rs:191-197: the only known-answer test of the reference
    idx = oracle.quickstat_index([2.3, 9.8, 3.1, 1.6, 6.7, 7.8, 8.6], 3, seed=seed)
    assert idx[3] == 4


def test_quickstat_random_postconditions(oracle):
    # quickstat.rs:199-219: i < goal => v < v[goal]; i >= goal => v >= v[goal]
    rng = np.random.default_rng(5)
    n = 100_000
    vals = rng.random(n)
    idx = np.arange(n, dtype=np.uint64)
    for t in range(25):
        goal = int(rng.integers(0, n))
        idx = oracle.quickstat_index(vals, goal, idx=idx, seed=t)
        v = vals[idx.astype(np.int64)]
        assert (v[:goal] < v[goal]).all()
        assert (v[goal:] >= v[goal]).all()
        assert np.array_equal(np.sort(idx), np.arange(n))


# ------------------------------------------------------------------ node counts

def test_nodes_needed_formulas(oracle):
    # Parallel/RustVersion/src/array_kd_tree.rs:45-53
    assert oracle.nodes_needed_par(2, 8) == 1
    assert oracle.nodes_needed_par(8, 8) == 1
    assert oracle.nodes_needed_par(9, 8) == 3
    assert oracle.nodes_needed_par(12, 8) == 7
    assert oracle.nodes_needed_par(1_000_000, 8) == 524_287
    # Sequential/RustVersion/src/array_kd_tree.rs:37-39
    assert oracle.nodes_needed_seq(2, 7) == 2
    assert oracle.nodes_needed_seq(12, 7) == 10


def test_c_port_node_count_differs(refc):
    # the C port allocates 2*(n/(MAX_PARTS-1)+1) (Parallel/CVersion/src/kdtree.c:15-19), the
    # count its two_leaves test expects (test.c: 6 for 12 bodies); the Rust formula gives 10
    assert refc.allocate_node_vec_len(12) == 6
    assert refc.allocate_node_vec_len(2) == 2


# ------------------------------------------------------------------ reference test cases

@pytest.mark.parametrize("layout", ["dfs", "par4"])
def test_single_node(oracle, layout):
    b = two_bodies()
    nodes = oracle.build_tree_dfs(b)[0] if layout == "dfs" else oracle.build_tree_par4(b, leaf=8)
    assert nodes[0]["num_parts"] == 2


@pytest.mark.parametrize("layout,leaf", [("dfs", 7), ("par4", 7), ("dfs", 8), ("par4", 8)])
def test_two_leaves(oracle, layout, leaf):
    b = circular_orbits(11, seed=3)  # 12 bodies
    nodes = (oracle.build_tree_dfs(b, leaf=leaf)[0] if layout == "dfs"
             else oracle.build_tree_par4(b, leaf=leaf))
    check_split_invariant(nodes, b)
    assert nodes[0]["num_parts"] == 0
    assert nodes[1]["num_parts"] + nodes[2]["num_parts"] == 12


@pytest.mark.parametrize("layout,leaf", [("dfs", 7), ("par4", 8)])
def test_big_solar(oracle, layout, leaf):
    b = circular_orbits(5000, seed=4)
    nodes = (oracle.build_tree_dfs(b, leaf=leaf)[0] if layout == "dfs"
             else oracle.build_tree_par4(b, leaf=leaf))
    check_split_invariant(nodes, b)


def test_big_solar_with_steps(oracle):
    b = circular_orbits(5000, seed=5)
    oracle.simple_sim(b, 1e-3, 10, leaf=8, layout="par4")
    nodes = oracle.build_tree_par4(b, leaf=8)
    check_split_invariant(nodes, b)


# ------------------------------------------------------------------ pin against the C port

@pytest.mark.parametrize("case", ["ring1000", "circ5000", "plummer3000"])
def test_oracle_matches_reference_c(oracle, refc, case):
    b = {"ring1000": lambda: ring(1000, seed=7),
         "circ5000": lambda: circular_orbits(5000, seed=8),
         "plummer3000": lambda: plummer(3000, seed=9)}[case]()
    ref_nodes, ref_last, _ = refc.build_tree(b, seed=3)
    nodes, last = oracle.build_tree_dfs(b, leaf=7, seed=11)
    assert last == ref_last
    assert leaf_sets(nodes) == leaf_sets(ref_nodes)
    internal = ref_nodes["num_parts"] == 0
    assert np.array_equal(nodes["split_dim"][internal], ref_nodes["split_dim"][internal])
    assert np.array_equal(nodes["split_val"][internal], ref_nodes["split_val"][internal])
    assert np.array_equal(nodes["size"][internal], ref_nodes["size"][internal])
    assert np.allclose(nodes["m"][internal], ref_nodes["m"][internal], rtol=1e-13, atol=0)
    assert np.allclose(nodes["cm"][internal], ref_nodes["cm"][internal], rtol=1e-13, atol=1e-15)
    acc, absum = oracle.calc_accel_abs(b, nodes, 0.3)
    acc_ref = refc.calc_accel(b, ref_nodes)
    assert_accel_close(acc, acc_ref, absum, 1e-12)


def test_oracle_vs_golden_every_step(oracle, golden):
    n = int(golden["n"])
    for k, b in enumerate(replay_positions(golden)):
        nodes, last = oracle.build_tree_dfs(b, leaf=7, seed=100 + k)
        assert last == int(golden["last_node"][k])
        assert np.array_equal(leaf_map(nodes, n), golden["leaf_of"][k])
        internal = golden["split_dim"][k] >= 0
        assert np.array_equal(nodes["split_dim"][internal].astype(np.int64),
                              golden["split_dim"][k][internal])
        assert np.array_equal(nodes["split_val"][internal], golden["split_val"][k][internal])
        assert np.allclose(nodes["m"][internal], golden["m"][k][internal], rtol=1e-13, atol=0)
        acc, absum = oracle.calc_accel_abs(b, nodes, 0.3)
        assert_accel_close(acc, golden["acc"][k], absum, 1e-12)


def test_oracle_simple_sim_vs_golden(oracle, golden):
    b = golden["init"].copy()
    oracle.simple_sim(b, float(golden["dt"]), int(golden["steps"]), leaf=7, layout="dfs")
    assert np.abs(b["p"] - golden["final"]["p"]).max() < 1e-13
    assert np.abs(b["v"] - golden["final"]["v"]).max() < 1e-11


def test_golden_replay_matches_reference_step_loop(golden):
    # the fixture's replayed positions agree with the C port's own simple_sim
    assert np.abs(golden["final"]["p"] - golden["ref_simple_sim_final"]["p"]).max() < 1e-13


# ------------------------------------------------------------------ oracle self-consistency

def test_par4_and_dfs_hold_the_same_leaves(oracle):
    b = ring(20_000, seed=12)
    dfs, _ = oracle.build_tree_dfs(b, leaf=8)
    par = oracle.build_tree_par4(b, leaf=8)
    assert sorted(leaf_sets(dfs).values()) == sorted(leaf_sets(par).values())
    a1 = oracle.calc_accel(b, dfs)
    a2 = oracle.calc_accel(b, par)
    assert rel_err(a1, a2).max() <= 1e-13


def test_theta_zero_is_direct_sum(oracle):
    b = plummer(2000, seed=13)
    nodes, _ = oracle.build_tree_dfs(b)
    acc = oracle.calc_accel(b, nodes, 0.0)
    sinks = np.arange(len(b))
    direct = oracle.direct_accel(b, sinks)
    assert rel_err(acc, direct).max() <= 1e-12


# ------------------------------------------------------------------ grouped walk (mixed path)

def test_grouped_walk_theta_zero_is_direct_sum(oracle):
    b = plummer(2000, seed=21)
    nodes, _ = oracle.build_tree_dfs(b, leaf=7)
    acc, cnt = oracle.calc_accel_group(b, nodes, 0.0)
    ref = oracle.direct_accel(b, np.arange(len(b)))
    assert rel_err(acc, ref).max() <= 1e-12
    assert cnt["m2p"] == 0 and cnt["p2p"] == len(b) * (len(b) - 1)


@pytest.mark.parametrize("gen,theta", [("ring", 0.3), ("plummer", 0.5)])
def test_grouped_walk_refines_reference_walk(oracle, gen, theta):
    """Every node the group test accepts passes the per-body test of every sink in the
    group, so the grouped set holds at least as many terms per body and no larger overall
    truncation error than the reference walk."""
    n = 20_000
    b = ring(n, seed=22) if gen == "ring" else plummer(n, seed=22)
    nodes, _ = oracle.build_tree_dfs(b, leaf=7)
    ag, cg = oracle.calc_accel_group(b, nodes, theta)
    ab = oracle.calc_accel(b, nodes, theta)
    sinks = np.arange(1, n, 7)
    ref = oracle.direct_accel(b, sinks)
    eg, eb = rel_err(ag[sinks], ref), rel_err(ab[sinks], ref)
    assert np.sqrt(np.mean(eg ** 2)) <= np.sqrt(np.mean(eb ** 2))
    pb = oracle.walk_counts(b, nodes, np.arange(n), theta)
    assert cg["p2p"] + cg["m2p"] >= pb["p2p"] + pb["m2p"]
