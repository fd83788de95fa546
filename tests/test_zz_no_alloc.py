"""The allocation-free entry point (rnng_eps_graph_l2_static) against the regular one
and the oracle.

Callers that may not allocate device memory when they need the graph (a plugin in a
process whose device memory belongs to a framework's pool, a real-time loop that must
not allocate after start-up) use rnng_eps_graph_l2_static: they pass their own device
buffers and the library uses a fixed scratch array instead of allocating.  Its result
must be the regular entry point's result, bit for bit, and stay so on a second call
that reuses the scratch array (which keeps the previous call's contents).
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

    import oracle
    import rnng_gb300
    from rnng_gb300 import synth

    lib = rnng_gb300.load()
    x = synth.l2_mixture(n=6000, d=24, k=16, seed=31)
    r = np.float32(4.5)
    with rnng_gb300.Context(0) as ctx:
        want = ctx.eps_graph_l2(x, r, mode="bf16")
    ref = oracle.eps_graph_l2(x, r)
    assert np.array_equal(want[0], ref[0]) and np.array_equal(want[1], ref[1])
    assert np.array_equal(want[2].view(np.uint32), ref[2].view(np.uint32))
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


def test_static_scratch_overflow_with_large_capacity():
    """More edges than the scratch array stages (2^20) while the caller's capacity is
    larger: RNNG_ERR_OVERFLOW, the true total in *count, and each of the 2^20 written
    edges a distinct valid pair with the regular entry point's weight bits."""
    import torch

    import rnng_gb300

    lib = rnng_gb300.load()
    rng = np.random.default_rng(33)
    n, d = 2000, 6
    x = rng.normal(size=(n, d)).astype(np.float32)
    r = np.float32(1e6)  # every pair
    with rnng_gb300.Context(0) as ctx:
        wu, wv, ww = ctx.eps_graph_l2(x, r, mode="fp32")
    total = n * (n - 1) // 2
    assert wu.size == total
    wmat = np.zeros((n, n), np.uint32)
    wmat[wu, wv] = ww.view(np.uint32)
    xd = torch.from_numpy(x).cuda()
    cap = total + 10
    u = torch.full((cap,), -1, dtype=torch.int64, device="cuda")
    v = torch.full((cap,), -1, dtype=torch.int64, device="cuda")
    w = torch.zeros(cap, dtype=torch.float32, device="cuda")
    for _ in range(2):
        rc, m = _static_call(lib, xd, None, n, d, r, u, v, w, cap)
        assert rc == 4 and m == total
        staged = 1 << 20
        gu, gv, gw = u.cpu().numpy(), v.cpu().numpy(), w.cpu().numpy()
        assert np.all(gu[staged:] == -1)  # nothing beyond the staged edges is written
        gu, gv, gw = gu[:staged], gv[:staged], gw[:staged]
        assert np.all((gu >= 0) & (gu < gv) & (gv < n))
        assert np.unique(gu * n + gv).size == staged
        assert np.array_equal(wmat[gu, gv], gw.view(np.uint32))


def test_static_wide_points_and_infinite_radius():
    """d > 256 (the regular entry point's FP32-direct tiles as the baseline), and radius
    +inf: complete over finite rows, refused (RNNG_ERR_UNSUPPORTED) when a row holds an
    infinity and no NaN, as the regular entry point does."""
    import torch

    import rnng_gb300
    from rnng_gb300 import synth

    lib = rnng_gb300.load()
    x = synth.l2_mixture(n=1500, d=300, k=6, seed=34)
    r = np.float32(np.sqrt(2.0 * 300) * 1.05)
    with rnng_gb300.Context(0) as ctx:
        want = ctx.eps_graph_l2(x, r, mode="fp32")
        assert want[0].size > 1000
        xd = torch.from_numpy(x).cuda()
        cap = max(want[0].size, 200 * 199 // 2) + 100
        u = torch.empty(cap, dtype=torch.int64, device="cuda")
        v = torch.empty(cap, dtype=torch.int64, device="cuda")
        w = torch.empty(cap, dtype=torch.float32, device="cuda")
        rc, m = _static_call(lib, xd, None, 1500, 300, r, u, v, w, cap)
        assert rc == 0 and m == want[0].size
        got = _sorted(u[:m].cpu().numpy(), v[:m].cpu().numpy(), w[:m].cpu().numpy())
        assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])
        assert np.array_equal(got[2].view(np.uint32), want[2].view(np.uint32))
        # radius +inf: NaN rows have no edge, the rest is complete
        y = x[:200].copy()
        y[[3, 50], 7] = np.nan
        y[60, :] = np.inf
        y[60, 0] = np.nan
        inf = np.float32(np.inf)
        want = ctx.eps_graph_l2(y, inf, mode="fp32")
        assert want[0].size == 197 * 196 // 2
        yd = torch.from_numpy(y).cuda()
        rc, m = _static_call(lib, yd, None, 200, 300, inf, u, v, w, cap)
        assert rc == 0 and m == want[0].size
        got = _sorted(u[:m].cpu().numpy(), v[:m].cpu().numpy(), w[:m].cpu().numpy())
        assert np.array_equal(got[0], want[0]) and np.array_equal(got[2].view(np.uint32), want[2].view(np.uint32))
        # an infinite coordinate without a NaN in its row: refused by both entry points
        y[60, 0] = 1.0
        with pytest.raises(rnng_gb300.RnngError) as e:
            ctx.eps_graph_l2(y, inf, mode="fp32")
        assert e.value.code == 6
        yd = torch.from_numpy(y).cuda()
        rc, m = _static_call(lib, yd, None, 200, 300, inf, u, v, w, cap)
        assert rc == 6 and m == 0
        # ... and the next call with a finite radius works again
        rc, m = _static_call(lib, yd, None, 200, 300, r, u, v, w, cap)
        assert rc == 0 and m == ctx.eps_graph_l2(y, r, mode="fp32")[0].size
