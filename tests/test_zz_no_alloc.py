"""The allocation-free entry point (rnng_eps_graph_l2_static) against the regular one.

Callers that cannot allocate device memory when they need the graph (for example
work issued while a CUDA graph is being captured, or inside a framework that owns the
device allocator) use rnng_eps_graph_l2_static: they pass their own device buffers
and the library uses a fixed scratch array instead of allocating.  Its result must be
the regular entry point's result, bit for bit, and stay so on a second call that
reuses the scratch array (which keeps the previous call's contents).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sorted(u, v, w):
    o = np.lexsort((v, u))
    return u[o], v[o], w[o]


def _static_call(lib, xd, ids, n, d, r, u, v, w, cap):
    cnt = ctypes.c_int64(-1)
    rc = lib.rnng_eps_graph_l2_static(xd.data_ptr(), None if ids is None else ids.data_ptr(), n, d,
                                      ctypes.c_float(r), u.data_ptr(), v.data_ptr(), w.data_ptr(), cap,
                                      ctypes.byref(cnt), None)
    return rc, cnt.value


def test_static_matches_regular_entry_point_twice():
    import torch

    import rnng_gb300
    from rnng_gb300 import synth

    lib = rnng_gb300.load()
    x = synth.l2_mixture(n=6000, d=24, k=16, seed=31)
    r = np.float32(4.5)
    with rnng_gb300.Context(0) as ctx:
        want = ctx.eps_graph_l2(x, r, mode="bf16")
    assert want[0].size > 500
    n, d = x.shape
    xd = torch.from_numpy(x).cuda()
    cap = want[0].size + 4096
    u = torch.empty(cap, dtype=torch.int64, device="cuda")
    v = torch.empty(cap, dtype=torch.int64, device="cuda")
    w = torch.empty(cap, dtype=torch.float32, device="cuda")
    for _ in range(2):
        u.fill_(-1)
        rc, m = _static_call(lib, xd, None, n, d, r, u, v, w, cap)
        assert rc == 0 and m == want[0].size
        got = _sorted(u[:m].cpu().numpy(), v[:m].cpu().numpy(), w[:m].cpu().numpy())
        assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])
        assert np.array_equal(got[2].view(np.uint32), want[2].view(np.uint32))


def test_static_ids_limits_and_overflow():
    import torch

    import rnng_gb300
    from rnng_gb300 import synth

    lib = rnng_gb300.load()
    x = synth.l2_mixture(n=1000, d=8, k=4, seed=32)
    r = np.float32(2.0)
    ids = (np.arange(1000, dtype=np.int64) * 7 + 3)[::-1].copy()
    with rnng_gb300.Context(0) as ctx:
        want = ctx.eps_graph_l2(x, r, mode="fp32", ids=ids)
    xd = torch.from_numpy(x).cuda()
    idd = torch.from_numpy(ids).cuda()
    cap = want[0].size
    u = torch.empty(cap, dtype=torch.int64, device="cuda")
    v = torch.empty(cap, dtype=torch.int64, device="cuda")
    w = torch.empty(cap, dtype=torch.float32, device="cuda")
    rc, m = _static_call(lib, xd, idd, 1000, 8, r, u, v, w, cap)
    assert rc == 0 and m == cap
    got = _sorted(u.cpu().numpy(), v.cpu().numpy(), w.cpu().numpy())
    assert all(np.array_equal(a, b) for a, b in zip(got, want))
    # too small an output: the total is still reported, with RNNG_ERR_OVERFLOW
    rc, m = _static_call(lib, xd, idd, 1000, 8, r, u, v, w, cap // 2)
    assert rc == 4 and m == cap
    # beyond the fixed scratch's point limit: rejected before any GPU work
    rc, m = _static_call(lib, xd, None, 70000, 8, r, u, v, w, cap)
    assert rc == 1 and m == 0
