"""Device generators (kd_generate): shape and statistics of each workload, determinism."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def gen(kd, n, kind, seed):
    with kd.KDTreeSim(n) as s:
        s.generate(kind, seed)
        return s.get_bodies()


def test_ring(kd):
    n = 1_000_000
    b = gen(kd, n, "ring", 7)
    assert b["m"][0] == 1.0 and (b["p"][0] == 0).all() and (b["v"][0] == 0).all()
    assert (b["m"][1:] == 1e-14).all()
    p, v = b["p"][1:], b["v"][1:]
    r = np.hypot(p[:, 0], p[:, 1])
    assert r.min() >= 0.8 and r.max() <= 1.2
    assert abs(r.mean() - 1.0) < 2e-3
    assert abs(p[:, 2].std() / 1e-4 - 1.0) < 0.02 and abs(p[:, 2].mean()) < 1e-6
    speed = np.hypot(v[:, 0], v[:, 1])
    assert np.allclose(speed, np.sqrt(1.0 / r), rtol=1e-14)
    assert np.abs((p[:, 0] * v[:, 0] + p[:, 1] * v[:, 1]) / (r * speed)).max() < 1e-14
    phi = np.arctan2(p[:, 1], p[:, 0])
    assert abs(np.cos(phi).mean()) < 5e-3 and abs(np.sin(phi).mean()) < 5e-3
    b2 = gen(kd, n, "ring", 7)
    assert np.array_equal(b.view(np.uint8), b2.view(np.uint8))
    assert not np.array_equal(b["p"], gen(kd, n, "ring", 8)["p"])


def test_circular_orbits(kd):
    k = 100_000
    b = gen(kd, k + 1, "circular", 3)
    d = np.hypot(b["p"][1:, 0], b["p"][1:, 1])
    ref = 0.1 + (np.arange(k, dtype=np.float64) * 5.0 / float(k))  # array_particle.rs:29
    assert np.allclose(d, ref, rtol=1e-15)
    assert (b["p"][:, 2] == 0).all() and (b["m"][1:] == 1e-14).all() and b["m"][0] == 1.0


def test_plummer(kd):
    n = 1_000_000
    b = gen(kd, n, "plummer", 5)
    assert np.allclose(b["m"], 1.0 / n)
    p, v = b["p"], b["v"]
    assert np.abs(p.mean(axis=0)).max() < 1e-12 and np.abs(v.mean(axis=0)).max() < 1e-12
    r = np.linalg.norm(p, axis=1)
    assert r.max() < 20.1
    # half-mass radius of a Plummer sphere of scale radius 1: (2^(2/3) - 1)^(-1/2) = 1.305
    assert abs(np.median(r) / 1.3048 - 1.0) < 0.02
    # kinetic energy 3 pi / 64 (virial equilibrium, G = M = a = 1)
    ke = 0.5 * np.sum(b["m"] * np.sum(v * v, axis=1))
    assert abs(ke / (3 * np.pi / 64) - 1.0) < 0.02


def test_generated_bodies_step(kd):
    with kd.KDTreeSim(200_000, precision="mixed") as s:
        s.generate("ring", 1)
        s.simple_sim(1e-3, 2)
        b = s.get_bodies()
    assert np.isfinite(b["p"]).all()
