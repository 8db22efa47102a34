"""The allocation-free dot product (sfem_gb300_dot_noalloc).

It exists for callers that cannot call cudaMalloc at the point where they need
a reduction (an enclosing stream capture, an arena that owns all device memory,
a plugin host that forbids allocations): its scratch is a fixed array inside the
library.  The test calls it through the C ABI, twice in a row (the shared scratch
must be left ready for the next call), and compares with a float64 numpy dot of the
same inputs (within the rounding the vector type allows: per-thread partial sums in
the vector type, the reduction in double) and with the workspace-based sfem_gb300_dot.
This file is collected last on purpose."""

import ctypes

import numpy as np
import pytest

from sfem_gb300 import capi

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dt", ["f64", "f32"])
def test_dot_noalloc_matches_dot_twice(cuda, dt):
    import torch

    lib = capi.load()
    tdt, rt = (torch.float64, capi.FLOAT64) if dt == "f64" else (torch.float32, capi.FLOAT32)
    ws = torch.zeros(lib.sfem_gb300_reduce_workspace_size(), dtype=torch.uint8, device=cuda)
    for n, seed in ((3_000_001, 1), (777, 2)):
        g = torch.Generator(device=cuda).manual_seed(seed)
        x = torch.randn(n, dtype=tdt, device=cuda, generator=g)
        y = torch.randn(n, dtype=tdt, device=cuda, generator=g)
        res = torch.zeros(3, dtype=torch.float64, device=cuda)
        capi.check(lib.sfem_gb300_dot(rt, capi.i64(n), capi.vp(x), capi.vp(y), capi.vp(ws), capi.vp(res), None), "dot")
        for k in (1, 2):  # two calls in a row on the shared scratch
            capi.check(lib.sfem_gb300_dot_noalloc(rt, capi.i64(n), capi.vp(x), capi.vp(y),
                                                  capi.c_void(res.data_ptr() + 8 * k), None), "dot_noalloc")
        r = res.cpu().numpy()
        xh, yh = x.double().cpu().numpy(), y.double().cpu().numpy()
        exact = float(np.dot(xh, yh))
        mag = float(np.dot(np.abs(xh), np.abs(yh)))
        # float64 inputs: ~1e-16 per term; float32 inputs: each thread sums at most a few
        # dozen products in float (relative error ~ k * 6e-8) before the double reduction
        tol = 1e-13 if dt == "f64" else 2e-6
        assert abs(r[1] - exact) <= tol * mag, (n, r[1], exact, mag)
        assert abs(r[1] - r[0]) <= tol * mag, (n, r)
        assert r[1] == r[2], r  # the second call sees a clean scratch


def test_dot_noalloc_rejects_oversized(cuda):
    lib = capi.load()
    rc = lib.sfem_gb300_dot_noalloc(capi.FLOAT64, capi.i64(2**31), None, None, None, None)
    assert rc == 1
    assert "outside" in capi.last_error()
