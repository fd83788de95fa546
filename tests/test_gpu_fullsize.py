"""The benchmark workloads at their full sizes against the CPU oracle.

The oracle's brute force over all pairs of 1M or 5M points takes hours, so each
check here takes blocks of rows spread over the point set and compares every edge
incident to them with the oracle's edges of those rows against all later points
(the oracle's row range).  Together with bit-equality of the BF16 and FP32-direct
forms over the whole edge list this pins the headline edge set at its own size.
Bar: bit-exact (u, v and weight bits)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def same(a, b):
    (u1, v1, w1), (u2, v2, w2) = a, b
    return (np.array_equal(u1, u2) and np.array_equal(v1, v2)
            and np.array_equal(np.asarray(w1, np.float32).view(np.uint32), np.asarray(w2, np.float32).view(np.uint32)))


def rows_against_oracle(orc, x, r, got, starts, block=40):
    u, v, w = got
    checked = 0
    for r0 in starts:
        r1 = min(r0 + block, x.shape[0])
        want = orc.eps_graph_l2(x, r, rows=(r0, r1))
        sel = (u >= r0) & (u < r1)
        assert same((u[sel], v[sel], w[sel]), want), (r0, int(sel.sum()), want[0].size)
        checked += want[0].size
    return checked


def fp64_error(x, u, v, w, chunk=1 << 19):
    """max |w - L2 in float64| over the edges (the reference's FP32 rounding, not an error of the path)."""
    err = 0.0
    for s in range(0, u.size, chunk):
        a = x[u[s:s + chunk]].astype(np.float64)
        a -= x[v[s:s + chunk]]
        d64 = np.sqrt(np.einsum("ij,ij->i", a, a))
        err = max(err, float(np.max(np.abs(w[s:s + chunk].astype(np.float64) - d64))))
    return err


def test_k2_full_size_1m_descriptors(ctx, orc):
    """1,000,000 x 128 integer descriptors at the headline radius: the BF16 form equals the
    FP32-direct form edge for edge, and both equal the oracle on sampled row blocks."""
    from rnng_gb300 import synth
    x = synth.descriptor()
    r = synth.EPS_K2
    bf = ctx.eps_graph_l2(x, r, mode="bf16")
    assert bf[0].size > 9_000_000
    fp = ctx.eps_graph_l2(x, r, mode="fp32")
    assert same(bf, fp)
    del fp
    checked = rows_against_oracle(orc, x, r, bf, (0, 250_013, 500_000, 777_777, 999_960))
    assert checked > 50
    assert fp64_error(x, *bf) < 1e-5 * float(r)


def test_k5_full_size_5m_zipf(ctx, orc):
    """5,000,000 x 32 Zipf mixture: the same checks at the uneven-cell configuration."""
    from rnng_gb300 import synth
    x = synth.zipf_mixture()
    r = synth.EPS_K5
    bf = ctx.eps_graph_l2(x, r, mode="bf16")
    assert bf[0].size > 40_000_000
    fp = ctx.eps_graph_l2(x, r, mode="fp32")
    assert same(bf, fp)
    del fp
    checked = rows_against_oracle(orc, x, r, bf, (0, 1_234_567, 2_500_000, 4_999_960))
    assert checked > 50
    assert fp64_error(x, *bf) < 1e-5 * max(1.0, float(r))


def test_k4_full_size_500k_torus_graph(ctx, orc):
    """500,000 torus points in R^16: the Rips path's epsilon graph (both forms) against the
    oracle on sampled row blocks, and the full filtration's edges equal that graph."""
    from rnng_gb300 import synth
    x = synth.torus16()
    r = synth.EPS_K4
    bf = ctx.eps_graph_l2(x, r, mode="bf16")
    assert bf[0].size > 5_000_000
    assert same(bf, ctx.eps_graph_l2(x, r, mode="fp32"))
    checked = rows_against_oracle(orc, x, r, bf, (0, 100_000, 250_000, 499_960), block=60)
    assert checked > 200
    ids, vals = ctx.rips_l2(x, r, maxdim=1, mode="bf16")
    # maxdim 1: the vertices (value 0), then the edges, ids a + C(b, 2) | 1 << 60 over u < v
    u, v, w = bf
    eid = (v * (v - 1) // 2 + u) | (1 << 60)
    o = np.lexsort((eid, w))
    want_ids = np.concatenate([np.arange(x.shape[0], dtype=np.int64), eid[o]])
    want_vals = np.concatenate([np.zeros(x.shape[0], np.float32), w[o]])
    assert np.array_equal(ids, want_ids) and np.array_equal(vals.view(np.uint32), want_vals.view(np.uint32))
