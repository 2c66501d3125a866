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
                          "--n", "20000", "--steps", "4", "--warmup", "3"],
                         capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert out.returncode == 0, out.stderr
    lines = [l for l in out.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "body-steps/s"
    assert d["value"] > 0 and d["higher_is_better"] is True
    # the arm runs exactly the --steps / --warmup it was given (each a sampled step)
    assert d["steps"] == 4 and d["warmup"] == 3
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert "sampled" in d["cpu_baseline"]["sample"]
    assert d["e2e"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["config"]["n_bodies"] == 20000
    parts = d["step_parts_s"]
    assert d["ms_per_step"] == pytest.approx(1e3 * sum(parts.values()), rel=1e-9)


def test_sampled_rate_matches_a_full_step_when_every_sink_is_walked():
    """With the sample fraction at 1 the sampled step is the whole step: its extrapolated
    rate is the measured one."""
    sys.path.insert(0, str(ROOT))
    import bench
    from multilanguagekdtree_gb300.array_particle import ring
    b = ring(5000, seed=3)
    rate, threads, cpu_s, parts, ns = bench.sampled_cpu_rate(b, 2, 0, 7, 0.3, 1e-3, 1.0, 1)
    assert ns == 5000 and threads >= 1
    assert rate == pytest.approx(5000 * 2 / cpu_s, rel=1e-9)


def test_walk_flops_counts():
    sys.path.insert(0, str(ROOT))
    import bench
    cnt = {"p2p": 10, "m2p": 5, "opened": 3, "visits": 99}
    assert bench.grouped_walk_flops(cnt) == 18 * 15 + 20 * 3
    r = bench.walk_roofline(1000, 2.0, 100.0, 4e5, 50.0, "peak note")
    assert r["achieved"] == pytest.approx(100.0 * 1000 / 2.0 / 1e12)
    assert r["frac"] == pytest.approx(r["achieved"] / 50.0)
    assert r["grouped_set"]["flops_per_body"] == pytest.approx(400.0)


def test_reference_walk_flops_follow_the_oracle_counts(oracle):
    """18 per pair, 10 per opening test, 9 per accepted node of the reference walk."""
    sys.path.insert(0, str(ROOT))
    import numpy as np

    import bench
    from multilanguagekdtree_gb300.array_particle import ring
    b = ring(20_000, seed=4)
    sinks = np.arange(0, 20_000, 7)
    alg, per = bench.reference_walk_flops(b, 7, 0.3, sinks)
    nodes = oracle.build_tree_par4(b, leaf=7)
    c = oracle.walk_counts(b, nodes, sinks, 0.3)
    k = len(sinks)
    assert alg == pytest.approx((18 * c["p2p"] + 10 * c["opened"] + 9 * c["m2p"]) / k)
    assert per["visits"] == pytest.approx(c["visits"] / k)


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
