"""GPU tests of the host transfers of kd_set_bodies / kd_get_bodies: page-locked buffers are
read and written in place by the converting kernels, pageable (and misaligned pinned)
buffers go through the staging copy; both paths must give the same bytes."""
import numpy as np
import pytest

import multilanguagekdtree_gb300 as kd

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def pinned_records(n, offset=0):
    """n particle records in page-locked memory, starting `offset` bytes into the buffer."""
    t = torch.empty(n * 64 + offset, dtype=torch.uint8, pin_memory=True)
    return t, t.numpy()[offset:offset + n * 64].view(kd.PARTICLE_DTYPE)


@pytest.mark.parametrize("offset", [0, 8])
@pytest.mark.parametrize("n", [1, 257, 3001])
def test_pinned_and_pageable_transfers_agree(n, offset):
    b = kd.ring(n, seed=5)
    keep_in, pin_in = pinned_records(n, offset)
    pin_in[...] = b
    keep_out, pin_out = pinned_records(n, offset)
    pin_out[...] = np.zeros(1, dtype=kd.PARTICLE_DTYPE)
    with kd.KDTreeSim(n, precision="mixed") as s1, kd.KDTreeSim(n, precision="mixed") as s2:
        s1.set_bodies(b)
        s2.set_bodies(pin_in)
        # the round trip alone is exact
        assert s2.get_bodies(out=pin_out).tobytes() == b.tobytes()
        s1.simple_sim(1e-3, 3)
        s2.simple_sim(1e-3, 3)
        ref = s1.get_bodies()
        s2.get_bodies(out=pin_out)
        assert pin_out.tobytes() == ref.tobytes()
    del keep_in, keep_out


def test_pinned_transfer_rejects_non_finite_input():
    n = 513
    b = kd.ring(n, seed=2)
    keep, pin = pinned_records(n)
    pin[...] = b
    pin["p"][100, 1] = np.nan
    with kd.KDTreeSim(n, precision="mixed") as s:
        with pytest.raises(kd.KDError):
            s.set_bodies(pin)
    del keep
