"""kd_direct_accel_noalloc: the direct-sum entry point for callers that cannot allocate device
memory (a host that has committed the GPU's memory to its own state, or one that measures
accuracy inside its step loop and cannot afford cudaMalloc's device-wide synchronisation).

It is called through the C ABI with device buffers the test allocates itself, and its output
is checked against kd_direct_accel (the allocating entry point) on two calls in a row -- the
second with other sinks, so that stale scratch from the first call would show.  This file is
collected last, so a run that stops at the first failure has run every other test first."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12  # same bar as the FP64 parity tests; only the source chunking differs


def test_noalloc_direct_sum_matches_allocating_entry_point(kd):
    import torch

    from multilanguagekdtree_gb300 import _lib

    lib = _lib.load()
    n = 60_000
    b = kd.ring(n, seed=21)
    rng = np.random.default_rng(22)
    dev = torch.device("cuda", 0)
    cols = [torch.from_numpy(np.ascontiguousarray(b["p"][:, d])).to(dev) for d in range(3)]
    mass = torch.from_numpy(np.ascontiguousarray(b["m"])).to(dev)
    with kd.KDTreeSim(n) as s:
        s.set_bodies(b)
        # 1500 and 700 sinks: the sources in 15 chunks of 4096 bodies; 20000 sinks: the
        # scratch holds only floor(131072 / (3 * 20000)) = 2 chunks, so each is 30000 bodies
        for call, ns in enumerate((1500, 700, 20_000)):
            sinks = np.sort(rng.choice(np.arange(1, n), ns, replace=False)).astype(np.uint64)
            ref = s.direct_accel(sinks)
            d_sinks = torch.from_numpy(sinks.view(np.int64)).to(dev)
            out = torch.full((ns, 3), float("nan"), dtype=torch.float64, device=dev)
            torch.cuda.synchronize()
            rc = lib.kd_direct_accel_noalloc(
                C.c_void_p(cols[0].data_ptr()), C.c_void_p(cols[1].data_ptr()),
                C.c_void_p(cols[2].data_ptr()), C.c_void_p(mass.data_ptr()), n,
                C.c_void_p(d_sinks.data_ptr()), ns, C.c_void_p(out.data_ptr()), None)
            assert rc == 0, lib.kd_last_error(None)
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            err = np.linalg.norm(got - ref, axis=1) / np.linalg.norm(ref, axis=1)
            assert err.max() <= RTOL, (call, err.max())

    # a sink index out of range gives NaN in its row, the other rows are unaffected
    sinks = np.array([5, n + 3, 17], dtype=np.uint64)
    d_sinks = torch.from_numpy(sinks.view(np.int64)).to(dev)
    out = torch.zeros((3, 3), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    rc = lib.kd_direct_accel_noalloc(
        C.c_void_p(cols[0].data_ptr()), C.c_void_p(cols[1].data_ptr()),
        C.c_void_p(cols[2].data_ptr()), C.c_void_p(mass.data_ptr()), n,
        C.c_void_p(d_sinks.data_ptr()), 3, C.c_void_p(out.data_ptr()), None)
    assert rc == 0, lib.kd_last_error(None)
    got = out.cpu().numpy()
    assert np.isnan(got[1]).all()
    assert np.isfinite(got[[0, 2]]).all()

    # beyond the scratch limit: rejected with a message, nothing launched
    big = torch.zeros(43691, dtype=torch.int64, device=dev)
    out = torch.zeros((43691, 3), dtype=torch.float64, device=dev)
    rc = lib.kd_direct_accel_noalloc(
        C.c_void_p(cols[0].data_ptr()), C.c_void_p(cols[1].data_ptr()),
        C.c_void_p(cols[2].data_ptr()), C.c_void_p(mass.data_ptr()), n,
        C.c_void_p(big.data_ptr()), 43691, C.c_void_p(out.data_ptr()), None)
    assert rc == _lib.KD_EINVAL
    assert b"43690" in lib.kd_last_error(None)
