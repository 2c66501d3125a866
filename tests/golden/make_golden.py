"""Generate the golden fixtures of the 1,000-body ring case from the REFERENCE ITSELF.

Runs the reference's own C port of the path (MarkCLewis/MultiLanguageKDTree
Parallel/CVersion/src/kdtree.c + particle.c, compiled from the reference checkout into
oracle/_ref/libkdref.so by oracle/build.py; MAX_PARTS = 7, THETA = 0.3, DFS numbering) on a
seeded ring of 1,000 bodies for 10 steps of dt = 1e-3, and records per step:

* ``leaf_of[step, body]``: DFS index of the leaf holding each body (node membership);
* ``split_dim``, ``split_val`` of every internal node (DFS numbering; -1 / 0 for leaves);
* ``m``, ``cm`` of every internal node;
* the acceleration of every body (the C port's calc_accel, kdtree.c:230-233);

plus the initial and final bodies.  Between steps the kick-drift of kdtree.c:296-305 is
applied in numpy with the same IEEE operation order (v + dt*a, then p + dt*v), so the
positions fed to step k are the reference's own.

Run here, where the reference is mounted:  python tests/golden/make_golden.py
The output ring1000.npz is committed; tests read it on any machine.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from multilanguagekdtree_gb300.array_particle import ring  # noqa: E402  (input generator)
from oracle import RefC  # noqa: E402

N, STEPS, DT, SEED = 1000, 10, 1e-3, 1234


def leaf_map(nodes, n):
    leaf_of = np.full(n, -1, dtype=np.int32)
    for i, nd in enumerate(nodes):
        k = int(nd["num_parts"])
        if k > 0:
            leaf_of[nd["particles"][:k].astype(np.int64)] = i
    assert (leaf_of >= 0).all()
    return leaf_of


def main():
    ref = RefC()
    bodies = ring(N, seed=SEED)
    init = bodies.copy()
    b = bodies.copy()
    acc_all, leaf_all, sd_all, sv_all, m_all, cm_all = [], [], [], [], [], []
    last_nodes = []
    for step in range(STEPS):
        nodes, last, _ = ref.build_tree(b, seed=step + 1)
        acc = ref.calc_accel(b, nodes)
        acc_all.append(acc)
        leaf_all.append(leaf_map(nodes, N))
        internal = nodes["num_parts"] == 0
        sd_all.append(np.where(internal, nodes["split_dim"].astype(np.int64), -1))
        sv_all.append(np.where(internal, nodes["split_val"], 0.0))
        m_all.append(np.where(internal, nodes["m"], 0.0))
        cm_all.append(np.where(internal[:, None], nodes["cm"], 0.0))
        last_nodes.append(last)
        # kick-drift, kdtree.c:296-305
        b["v"] = b["v"] + DT * acc
        b["p"] = b["p"] + DT * b["v"]
    # the reference's own step loop from the same start, as a cross-check of the replay
    b2 = init.copy()
    ref.simple_sim(b2, DT, STEPS, seed=99)
    dev = np.abs(b2["p"] - b["p"]).max()
    assert dev < 1e-13, dev
    out = Path(__file__).resolve().parent / "ring1000.npz"
    np.savez_compressed(
        out, n=N, steps=STEPS, dt=DT, seed=SEED, leaf_size=7, theta=0.3,
        init=init.view(np.uint8), final=b.view(np.uint8),
        acc=np.stack(acc_all), leaf_of=np.stack(leaf_all), split_dim=np.stack(sd_all),
        split_val=np.stack(sv_all), m=np.stack(m_all), cm=np.stack(cm_all),
        last_node=np.array(last_nodes), ref_simple_sim_final=b2.view(np.uint8))
    print(f"wrote {out} ({out.stat().st_size} bytes); simple_sim replay deviation {dev:.3e}")


if __name__ == "__main__":
    main()
