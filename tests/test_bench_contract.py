"""The bench's JSON contract on the CPU: the reference arm (the oracle's step loop of the
reference algorithm) on a small ring, and the algorithmic-work helpers."""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_prints_one_json_line():
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                          "--n", "20000", "--steps", "2", "--warmup", "1"],
                         capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert out.returncode == 0, out.stderr
    lines = [l for l in out.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "body-steps/s"
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["config"]["n_bodies"] == 20000


def test_walk_flops_counts_interactions_and_group_tests():
    sys.path.insert(0, str(ROOT))
    import bench
    cnt = {"p2p": 10, "m2p": 5, "opened": 3, "visits": 99}
    assert bench.walk_flops(cnt) == 18 * 15 + 20 * 3


@pytest.mark.parametrize("ws,t,expect", [(1, 2.0, 500.0), (4, 2.0, 2000.0)])
def test_replica_value_is_whole_job(ws, t, expect):
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.replica_value(ws, 100, 10, t) == pytest.approx(expect)


@pytest.mark.parametrize("n,leaf,expect", [(10_000_000, 7, 21), (20_000_000, 7, 22), (7, 7, 0),
                                           (8, 7, 1)])
def test_tree_levels(n, leaf, expect):
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.tree_levels(n, leaf) == expect


@pytest.mark.parametrize("n,exceeds", [(10_000_000, True), (4_000_000, True), (20_000, False)])
def test_l2_note_states_how_the_inputs_stand_against_the_l2(n, exceeds):
    sys.path.insert(0, str(ROOT))
    import bench
    note = bench.l2_note(n)
    assert ("exceed the 129 MB L2" in note) == exceeds
    assert f"{64.0 * n / 1e6:.0f}" in note or f"{64.0 * n / 1e6:.1f}" in note
