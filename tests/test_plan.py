"""CPU tests of the host plan behind the grouped walk: the sink groups the library packs
(kd_group_plan) are the oracle's groups (make_groups / group_split of kdoracle.c) for the
same n, so both walk the same grouped interaction set."""
import numpy as np
import pytest

from multilanguagekdtree_gb300.array_kd_tree import group_plan
from multilanguagekdtree_gb300.array_particle import ring


@pytest.mark.parametrize("leaf", [7, 8])
@pytest.mark.parametrize("n", [1, 5, 8, 9, 64, 65, 1000, 12345, 100_003])
def test_group_plan_matches_oracle(oracle, n, leaf):
    nodes, _ = oracle.build_tree_dfs(ring(n, seed=3), leaf=leaf)
    gs_o, sp_o = oracle.groups(nodes, n)
    gs, sp = group_plan(n, leaf)
    assert np.array_equal(gs.astype(np.uint64), gs_o)
    assert np.array_equal(sp.astype(np.uint64), sp_o)


@pytest.mark.parametrize("n", [1000, 100_003])
def test_groups_are_whole_leaves_of_at_most_64_bodies(n):
    gs, sp = group_plan(n, 7)
    sizes = np.diff(gs.astype(np.int64))
    assert gs[0] == 0 and gs[-1] == n
    assert sizes.min() >= 1 and sizes.max() <= 64
    # each split lies inside its group, or at its end for a one-leaf group
    assert np.all(sp >= gs[:-1]) and np.all(sp <= gs[1:])
    # greedy packing: a group and its successor together exceed 64 bodies
    assert np.all(sizes[:-1] + sizes[1:] > 64)


@pytest.mark.parametrize("n,leaf", [(0, 7), (100, 1), (100, 9)])
def test_group_plan_rejects_bad_arguments(n, leaf):
    with pytest.raises(ValueError):
        group_plan(n, leaf)


def test_group_plan_reports_the_count_when_the_buffer_is_short():
    import ctypes as C

    from multilanguagekdtree_gb300 import _lib
    lib = _lib.load()
    ng = C.c_size_t(0)
    rc = lib.kd_group_plan(1000, 7, None, None, 0, C.byref(ng))
    assert rc != 0 and ng.value == len(group_plan(1000, 7)[1])
    # a stale message of an earlier call is replaced by this call's reason
    assert b"kd_group_plan" in lib.kd_last_error(None)
    rc = lib.kd_group_plan(0, 7, None, None, 0, C.byref(ng))
    assert rc != 0 and b"n < 2^31" in lib.kd_last_error(None)
