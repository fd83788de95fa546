"""GPU Vietoris-Rips filtration against the golden fixture made by RNNG's rips path
(per-cell build_filtration + merge) and against the oracle (bit-exact ids and values)."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def same(a, b):
    return np.array_equal(a[0], b[0]) and np.array_equal(np.asarray(a[1]).view(np.uint32),
                                                          np.asarray(b[1]).view(np.uint32))


@pytest.mark.parametrize("mode", ["fp32", "bf16"])
def test_golden_k4(ctx, mode):
    g = golden("k4_rips")
    got = ctx.rips_l2(g["x"], g["radius"], maxdim=int(g["maxdim"]), mode=mode)
    assert same(got, (g["ids"], g["values"]))


@pytest.mark.parametrize("maxdim", [0, 1, 2])
def test_random_against_oracle(ctx, orc, maxdim):
    rng = np.random.default_rng(maxdim + 50)
    x = rng.normal(size=(900, 5)).astype(np.float32)
    r = np.float32(1.1)
    u, v, w = orc.eps_graph_l2(x, r)
    want = orc.rips(x.shape[0], u, v, w, maxdim)
    assert same(ctx.rips_l2(x, r, maxdim=maxdim), want)


def test_ids_and_edge_cases(ctx, orc):
    rng = np.random.default_rng(60)
    x = rng.normal(size=(400, 3)).astype(np.float32)
    r = np.float32(0.9)
    ids = rng.permutation(400).astype(np.int64) * 11 + 5
    gi, gv = ctx.rips_l2(x, r, maxdim=2, ids=ids)
    # expected filtration over the labels: vertices, edges and triangles by brute force
    u, v, w = orc.eps_graph_l2(x, r)
    wmap = {}
    for a, b, c in zip(ids[u].tolist(), ids[v].tolist(), w.tolist()):
        wmap[(min(a, b), max(a, b))] = c
    adj = {}
    for (a, b) in wmap:
        adj.setdefault(a, set()).add(b)
    want = [(0.0, orc.simplex_id([i])) for i in ids.tolist()]
    want += [(c, orc.simplex_id([a, b])) for (a, b), c in wmap.items()]
    for a in adj:
        for b in adj[a]:
            for c in adj[a] & adj.get(b, set()):
                want.append((max(wmap[(a, b)], wmap[(a, c)], wmap[(b, c)]), orc.simplex_id([a, b, c])))
    want.sort()
    assert gi.tolist() == [t for _, t in want]
    assert np.array_equal(gv, np.array([val for val, _ in want], np.float32))
    # duplicates collapse to zero-length edges and triangles at value 0
    y = np.ones((10, 4), np.float32)
    yi, yv = ctx.rips_l2(y, 0.0, maxdim=2)
    assert yi.size == 10 + 45 + 120 and np.all(yv == 0)
    # empty input and a negative radius
    assert ctx.rips_l2(np.zeros((0, 3), np.float32), 1.0)[0].size == 0
    ni, nv = ctx.rips_l2(x, -1.0, maxdim=2)
    assert ni.size == 400 and np.all(nv == 0)


def test_torus_100k_against_oracle_cliques(ctx, orc):
    from rnng_gb300 import synth
    x = synth.torus16(n=100_000, seed=4)
    r = synth.choose_eps(x, 30.0, sample=20000)
    u, v, w = ctx.eps_graph_l2(x, r, mode="fp32")
    want = orc.rips(x.shape[0], u, v, w, 2)
    got = ctx.rips_l2(x, r, maxdim=2, mode="bf16")
    assert same(got, want) and got[0].size > 1_000_000
