"""The FP64 direct sum (kd_direct_accel) -- the yardstick of every mixed-precision accuracy
figure -- against the oracle's direct sum, and the heavy bodies of the mixed path, whose own
accelerations are FP64 direct sums over all bodies.

Bar: the same terms summed in another order differ by rounding proportional to the sum of
the terms' magnitudes, so every sink is held to |da| <= 1e-12 * sum|terms|, and the
well-conditioned ones to |da| <= 1e-12 |a| (conftest.assert_accel_close).  The ring's
central body is the ill-conditioned case: ~N pulls of 1e-14 that cancel a thousand-fold."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import assert_accel_close, rel_err

pytestmark = pytest.mark.gpu

ACC_RTOL = 1e-12
MIXED_RTOL = 1e-4


def sample_sinks(n, k, seed):
    """k seeded sinks, body 0 always among them."""
    rng = np.random.default_rng(seed)
    s = rng.choice(np.arange(1, n), k - 1, replace=False)
    return np.sort(np.concatenate([[0], s])).astype(np.uint64)


@pytest.mark.parametrize("gen,n", [("ring", 200_000), ("plummer", 50_000)])
def test_direct_accel_matches_oracle(kd, oracle, gen, n):
    b = kd.ring(n, seed=61) if gen == "ring" else kd.plummer(n, seed=61)
    sinks = sample_sinks(n, 4096, 62)
    with kd.KDTreeSim(n) as s:
        s.set_bodies(b)
        got = s.direct_accel(sinks)
    ref, absum = oracle.direct_accel_abs(b, sinks)
    d = np.linalg.norm(got - ref, axis=1)
    assert (d <= ACC_RTOL * absum).all(), (d / absum).max()
    if gen == "plummer":  # no cancellation: every sink is well conditioned
        assert rel_err(got, ref).max() <= ACC_RTOL
    else:
        assert_accel_close(got, ref, absum, ACC_RTOL)


def binary_ring(kd, n, seed):
    """The ring with a second heavy body: body 1 of mass 0.01 on a circular orbit at r = 3
    (outside the ring), so the mixed path has two heavy bodies that pull on each other."""
    b = kd.ring(n, seed=seed)
    b["p"][1] = [3.0, 0.0, 0.0]
    b["v"][1] = [0.0, np.sqrt(1.01 / 3.0), 0.0]
    b["m"][1] = 0.01
    return b


@pytest.mark.parametrize("two", [False, True])
def test_heavy_bodies_are_direct_sums(kd, oracle, two):
    """The heavy bodies' accelerations on the mixed path equal the FP64 direct sum (not the
    theta-truncated tree value, which is off by its whole size for the ring's centre)."""
    n = 200_000
    b = binary_ring(kd, n, 63) if two else kd.ring(n, seed=63)
    heavy = np.array([0, 1] if two else [0], dtype=np.uint64)
    with kd.KDTreeSim(n, precision="mixed") as s:
        s.set_bodies(b)
        s.build_tree()
        acc = s.calc_accel()
    ref, absum = oracle.direct_accel_abs(b, heavy)
    d = np.linalg.norm(acc[heavy.astype(np.int64)] - ref, axis=1)
    assert (d <= ACC_RTOL * absum).all(), d / absum


def test_mixed_error_includes_the_central_body(kd, oracle):
    """Relative error of the mixed walk against the FP64 direct sum on 4,096 sinks, body 0
    included, within the 1e-4 contract."""
    n = 200_000
    b = kd.ring(n, seed=64)
    sinks = sample_sinks(n, 4096, 65)
    with kd.KDTreeSim(n, precision="mixed") as s:
        s.set_bodies(b)
        s.build_tree()
        acc = s.calc_accel()
    ref = oracle.direct_accel(b, sinks)
    err = rel_err(acc[sinks.astype(np.int64)], ref)
    assert err.max() <= MIXED_RTOL, err.max()
    assert err[0] <= 1e-9, err[0]  # body 0: an FP64 direct sum itself


def test_mixed_step_moves_heavy_bodies_by_their_direct_sums(kd, oracle):
    """One mixed step of the two-heavy-body ring: the heavy bodies' new velocities follow
    v + dt a with a their FP64 direct sums (kick-drift in the reference's order)."""
    n, dt = 50_000, 1e-3
    b = binary_ring(kd, n, 66)
    heavy = np.array([0, 1], dtype=np.uint64)
    ref, absum = oracle.direct_accel_abs(b, heavy)
    with kd.KDTreeSim(n, precision="mixed") as s:
        s.set_bodies(b)
        s.simple_sim(dt, 1)
        out = s.get_bodies()
    for k, i in enumerate(heavy.astype(np.int64)):
        v = b["v"][i] + dt * ref[k]
        tol = dt * ACC_RTOL * absum[k] + 2e-16 * np.abs(v).max()
        assert np.abs(out["v"][i] - v).max() <= tol, (i, out["v"][i], v)
