"""The device-side guards: a walk whose traversal stack runs out and a median select that
runs out of refinement passes stop, set the device error word and the call returns
KD_EDEVICE -- no trap, no wait.  The limits are lowered through kd_set_device_limits so that
each guard fires on a small ring; the next call on the same context, with the limits back at
their defaults, must succeed and agree with the oracle.

The reference has no such path (its walk and quickselect panic on a bad index); the checks
are the failure-detection plan of the GPU port.  Every case here was read for memory safety
before it ran: the stack checks come before any push, a failed select narrows its candidates
into the block sort's fixed buffers, and the partition writes only inside its segment."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import assert_accel_close, leaf_sets

pytestmark = pytest.mark.gpu


def expect_device_error(kd, fn, text):
    with pytest.raises(kd.KDError) as e:
        fn()
    assert "KD_EDEVICE" in str(e.value) and text in str(e.value), str(e.value)


def test_grouped_walk_stack_guard(kd, oracle):
    n = 20_000
    b = kd.ring(n, seed=71)
    with kd.KDTreeSim(n, precision="mixed") as s:
        s.set_bodies(b)
        s.build_tree()
        good = s.calc_accel().copy()
        s.set_device_limits(stack_entries=4)
        expect_device_error(kd, s.calc_accel, "traversal stack overflow")
        s.set_device_limits()
        again = s.calc_accel()
    assert np.array_equal(again, good)


def test_fp64_walk_stack_guard_then_oracle_parity(kd, oracle):
    n = 20_000
    b = kd.ring(n, seed=72)
    with kd.KDTreeSim(n, precision="fp64") as s:
        s.set_bodies(b)
        s.build_tree()
        s.set_device_limits(stack_entries=3)
        expect_device_error(kd, s.calc_accel, "traversal stack overflow")
        s.set_device_limits()
        acc = s.calc_accel()
    nodes, _ = oracle.build_tree_dfs(b, leaf=7)
    oacc, absum = oracle.calc_accel_abs(b, nodes, 0.3)
    assert_accel_close(acc, oacc, absum)


def test_select_guard_then_exact_tree(kd, oracle):
    """n = 20,000: the last two levels above the subtree finish (2,500- and 1,250-body
    segments) select their medians in shared memory, which takes at least one radix pass;
    with none left the selects report the failure.  The master state is untouched, so the
    next build, with the default limits, is the exact tree again."""
    n = 20_000
    b = kd.ring(n, seed=73)
    with kd.KDTreeSim(n, precision="fp64") as s:
        s.set_bodies(b)
        s.set_device_limits(select_passes=0)
        expect_device_error(kd, s.build_tree, "median select failed to converge")
        with pytest.raises(kd.KDError):  # the failed build left no tree to walk
            s.calc_accel()
        s.set_device_limits()
        s.build_tree()
        nodes = s.nodes()
        acc = s.calc_accel()
    onodes, _ = oracle.build_tree_dfs(b, leaf=7)
    assert leaf_sets(nodes) == leaf_sets(onodes)
    internal = onodes["num_parts"] == 0
    assert np.array_equal(nodes["split_val"][internal], onodes["split_val"][internal])
    oacc, absum = oracle.calc_accel_abs(b, onodes, 0.3)
    assert_accel_close(acc, oacc, absum)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_failed_steps_leave_the_bodies_in_place(kd, oracle, precision):
    """A step loop whose walk overflows returns KD_EDEVICE with the bodies where the failed
    step started (its kick-drift is skipped); after the limits are restored the same context
    steps on normally."""
    n = 20_000
    b = kd.ring(n, seed=74)
    with kd.KDTreeSim(n, precision=precision) as s:
        s.set_bodies(b)
        s.set_device_limits(stack_entries=3)
        expect_device_error(kd, lambda: s.simple_sim(1e-3, 3), "traversal stack overflow")
        after = s.get_bodies()
        assert np.array_equal(after["p"], b["p"]) and np.array_equal(after["v"], b["v"])
        s.set_device_limits()
        s.simple_sim(1e-3, 2)
        out = s.get_bodies()
    if precision == "fp64":
        o = b.copy()
        oracle.simple_sim(o, 1e-3, 2, leaf=7, layout="dfs")
        assert np.abs(out["p"] - o["p"]).max() < 1e-13
    else:
        assert np.isfinite(out["p"]).all() and not np.array_equal(out["p"], b["p"])


def test_limits_are_validated(kd):
    with kd.KDTreeSim(100) as s:
        with pytest.raises(kd.KDError):
            s.set_device_limits(stack_entries=1)
        with pytest.raises(kd.KDError):
            s.set_device_limits(select_passes=17)
