"""GPU quickstat_index against the reference's own quickstat tests
(Parallel/RustVersion/src/quickstat.rs:191-253) and an exact selection."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def check_post(vals, idx, goal, n_total=None):
    v = vals[idx.astype(np.int64)]
    assert (v[:goal] < v[goal]).all()
    assert (v[goal:] >= v[goal]).all()


def test_small_known_answer(kd):
    # quickstat.rs:191-197
    idx = kd.quickstat_index([2.3, 9.8, 3.1, 1.6, 6.7, 7.8, 8.6], 3)
    assert idx[3] == 4


@pytest.mark.parametrize("n", [1000, 100_000, 3_000_000])
def test_random_postconditions(kd, n):
    # quickstat.rs:199-219
    rng = np.random.default_rng(n)
    vals = rng.random(n)
    for goal in [0, n - 1, n // 2] + list(rng.integers(0, n, 5)):
        idx = kd.quickstat_index(vals, int(goal))
        check_post(vals, idx, int(goal))
        assert np.array_equal(np.sort(idx), np.arange(n, dtype=np.uint64))
        assert vals[idx[goal]] == np.partition(vals, goal)[goal]


def test_random_slice(kd):
    # quickstat.rs:221-253: select inside a sub-slice of the index vector
    rng = np.random.default_rng(3)
    n = 100_000
    vals = rng.random(n)
    for _ in range(10):
        start = int(rng.integers(0, n // 4))
        end = start + 1 + int(rng.integers(0, 3 * n // 4))
        goal = int(rng.integers(start, end))
        sub = kd.quickstat_index(vals, goal - start, indices=np.arange(start, end))
        check_post(vals, sub, goal - start)
        assert np.array_equal(np.sort(sub), np.arange(start, end, dtype=np.uint64))


def test_rejects_bad_input(kd):
    with pytest.raises(kd.KDError):
        kd.quickstat_index([1.0, 2.0], 2)
    with pytest.raises(kd.KDError):
        kd.quickstat_index([1.0, float("nan"), 2.0], 1)
    with pytest.raises(kd.KDError):
        kd.quickstat_index([1.0, 2.0], 0, indices=[0, 5])
