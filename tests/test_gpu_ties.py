"""Trees of inputs with many equal coordinates, which the oracle cannot arbitrate node by
node: the reference settles equal coordinates by its random pivots, the GPU build orders
them by body id (the exact median on (coordinate, id)).  Positions are put on a grid along
one or two dimensions (never all three, so no two bodies coincide), at sizes whose subtrees
are finished both by the multi-block levels and by the shared-memory finish.  Checked: the
split invariant with ties (left <= split_val <= right along the split dimension, equal
coordinates ordered by id across the split, the median in the right child), identical trees
from repeated builds, and the FP64 walk on the GPU's tree against the oracle's walk on the
same tree."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import assert_accel_close

pytestmark = pytest.mark.gpu


def subtree_members(nodes):
    """Body indices under every node (post order, no recursion)."""
    out = {}
    stack = [(0, False)]
    while stack:
        i, done = stack.pop()
        nd = nodes[i]
        k = int(nd["num_parts"])
        if k > 0:
            out[i] = nd["particles"][:k].astype(np.int64)
        elif done:
            out[i] = np.concatenate([out[int(nd["left"])], out[int(nd["right"])]])
        else:
            stack.append((i, True))
            stack.append((int(nd["left"]), False))
            stack.append((int(nd["right"]), False))
    return out


def check_tie_split_invariant(nodes, bodies):
    p = bodies["p"]
    mem = subtree_members(nodes)
    assert np.array_equal(np.sort(mem[0]), np.arange(len(bodies)))
    for i, nd in enumerate(nodes):
        if int(nd["num_parts"]) > 0 or i not in mem:
            continue
        d, sv = int(nd["split_dim"]), float(nd["split_val"])
        left, right = mem[int(nd["left"])], mem[int(nd["right"])]
        assert len(left) == (len(left) + len(right)) // 2
        assert (p[left, d] <= sv).all() and (p[right, d] >= sv).all(), i
        tl, tr = left[p[left, d] == sv], right[p[right, d] == sv]
        assert len(tr) > 0, i  # the median lies in the right child
        if len(tl):
            assert tl.max() < tr.min(), i


def gridded(kd, kind, n, seed):
    if kind == "ring":
        b = kd.ring(n, seed=seed)
        b["p"][:, 0] = np.round(b["p"][:, 0] * 64) / 64  # x on a 1/64 grid
        b["p"][:, 2] = 0.0                                # every z equal
    else:
        b = kd.plummer(n, seed=seed)
        b["p"][:, :2] = np.round(b["p"][:, :2] * 16) / 16  # x, y on a 1/16 grid
    return b


@pytest.mark.parametrize("kind,n,leaf,layout", [("ring", 20_000, 7, "dfs"),
                                                ("plummer", 30_001, 7, "dfs"),
                                                ("ring", 100_003, 8, "par4")])
def test_trees_with_equal_coordinates(kd, oracle, kind, n, leaf, layout):
    b = gridded(kd, kind, n, seed=17)
    assert len(np.unique(b["p"][:, 0])) < n // 4  # many ties along x
    with kd.KDTreeSim(n, leaf_size=leaf, layout=layout, precision="fp64") as s:
        s.set_bodies(b)
        s.build_tree()
        nodes = s.nodes()
        acc = s.calc_accel().copy()
        s.build_tree()
        again = s.nodes()
    for f in ("num_parts", "particles", "split_dim", "split_val", "size", "left", "right"):
        assert np.array_equal(nodes[f], again[f]), f
    check_tie_split_invariant(nodes, b)
    oacc, absum = oracle.calc_accel_abs(b, nodes, 0.3)
    assert_accel_close(acc, oacc, absum)
