"""kd_print_tree against a restatement of the reference's print_tree, byte for byte."""
from __future__ import annotations

import numpy as np
import pytest

from treedump import print_tree

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("layout,leaf", [("dfs", 7), ("par4", 8), ("par4", 7)])
def test_print_tree_matches_the_reference_format(kd, tmp_path, layout, leaf):
    b = kd.ring(700, seed=4)
    b["p"][5] = (-0.0, 1e-7, 0.30000000000000004)
    b["p"][6] = (1.0, -2.5e-5, 123456.125)
    with kd.KDTreeSim(len(b), leaf_size=leaf, layout=layout) as s:
        s.set_bodies(b)
        s.build_tree()
        nodes = s.nodes()
        path = s.print_tree(path=str(tmp_path / f"tree_{layout}.txt"))
    if layout == "par4":
        length = kd.nodes_needed(len(b), leaf, "par4")
    else:
        length = max(len(nodes), kd.nodes_needed(len(b), leaf, "dfs"))
    got = open(path).read()
    assert got == print_tree(nodes, b, length)
    assert got.splitlines()[0] == str(length)


def test_print_tree_default_name(kd, tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    b = kd.ring(50, seed=1)
    with kd.KDTreeSim(len(b)) as s:
        s.set_bodies(b)
        s.build_tree()
        assert s.print_tree(step=10) == "tree10.txt"
    assert (tmp_path / "tree10.txt").read_text().startswith(str(
        max(kd.nodes_needed(50, 7, "dfs"), 15)))
