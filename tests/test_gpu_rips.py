"""GPU Vietoris-Rips filtration against the golden fixture made by RNNG's rips path
(per-cell build_filtration + merge) and against the oracle (bit-exact ids and values)."""
import numpy as np
import pytest

from conftest import colex_max_id, golden

pytestmark = pytest.mark.gpu


def same(a, b):
    return np.array_equal(a[0], b[0]) and np.array_equal(np.asarray(a[1]).view(np.uint32),
                                                          np.asarray(b[1]).view(np.uint32))


@pytest.mark.parametrize("mode", ["fp32", "bf16"])
def test_golden_k4(ctx, mode):
    g = golden("k4_rips")
    got = ctx.rips_l2(g["x"], g["radius"], maxdim=int(g["maxdim"]), mode=mode)
    assert same(got, (g["ids"], g["values"]))


@pytest.mark.parametrize("mode", ["fp32", "bf16"])
def test_golden_nan_rows(ctx, mode):
    """Points with NaN coordinates are vertices without edges, as in RNNG's rips path."""
    g = golden("nan_rips")
    got = ctx.rips_l2(g["x"], g["radius"], maxdim=int(g["maxdim"]), mode=mode)
    assert same(got, (g["ids"], g["values"]))


@pytest.mark.parametrize("mode", ["fp32", "bf16"])
def test_golden_k4_maxdim3(ctx, mode):
    """The rips driver's default dimension (tetrahedra) against RNNG's own output."""
    g = golden("k4_rips3")
    got = ctx.rips_l2(g["x"], g["radius"], maxdim=3, mode=mode)
    assert same(got, (g["ids"], g["values"]))


def test_golden_edit_rips_through_edges(ctx):
    """Edit-distance complex: the GPU edit epsilon graph fed to rnng_rips_edges equals
    RNNG's rips path with EditDistance."""
    g = golden("k3_rips_edit")
    u, v, w = ctx.eps_graph_edit((g["atoms"], g["offsets"]), g["radius"])
    got = ctx.rips_edges(int(g["n"]), u, v, w, maxdim=int(g["maxdim"]))
    assert same(got, (g["ids"], g["values"]))


@pytest.mark.parametrize("maxdim", [2, 3, 4, 6])
def test_higher_dimensions_against_oracle(ctx, orc, maxdim):
    rng = np.random.default_rng(maxdim + 70)
    x = rng.normal(size=(700, 3)).astype(np.float32)
    r = np.float32(0.8)
    u, v, w = orc.eps_graph_l2(x, r)
    want = orc.rips(x.shape[0], u, v, w, maxdim)
    got = ctx.rips_l2(x, r, maxdim=maxdim, mode="fp32")
    assert same(got, want)
    # RNNG's Binom wraps its 64-bit falling product (700 * 699 * ... beyond 6 factors), so
    # ids of 7-vertex simplices here carry wrapped bits, identically on both sides;
    # below that the dimension field decodes
    decodable = maxdim <= 4
    if decodable:
        dims = want[0].view(np.uint64) >> np.uint64(60)
        assert int(dims.max()) == maxdim
    # the same complex from the edge list, rows permuted and edges in both orientations
    perm = rng.permutation(x.shape[0])
    inv = np.argsort(perm)
    flip = rng.random(u.size) < 0.5
    uu, vv = np.where(flip, inv[v], inv[u]), np.where(flip, inv[u], inv[v])
    got2 = ctx.rips_edges(x.shape[0], uu, vv, w, maxdim=maxdim, ids=perm.astype(np.int64))
    assert same(got2, want)
    # per-simplex flags: the OR of its vertices' flags (RNNG's interior)
    vflag = (rng.random(x.shape[0]) < 0.3).astype(np.uint8)
    gi, gv, gf = ctx.rips_edges(x.shape[0], uu, vv, w, maxdim=maxdim, ids=perm.astype(np.int64),
                                vertex_flags=vflag)
    assert same((gi, gv), want)
    if not decodable:
        return
    flag_of_id = np.zeros(x.shape[0], np.uint8)
    flag_of_id[perm] = vflag
    want_f = [max(flag_of_id[vtx] for vtx in _verts(int(i))) for i in gi]
    assert gf.tolist() == want_f


def _verts(sid: int) -> list[int]:
    """Vertices of a simplex id (sum of C(v_i, i+1) over sorted v, dim << 60)."""
    from math import comb
    dim, rest = sid >> 60, sid & ((1 << 60) - 1)
    out = []
    for i in range(dim, -1, -1):
        lo, hi = i, 1 << 21  # largest v with C(v, i+1) <= rest
        while lo < hi:
            mid = (lo + hi + 1) // 2
            if comb(mid, i + 1) <= rest:
                lo = mid
            else:
                hi = mid - 1
        out.append(lo)
        rest -= comb(lo, i + 1)
    assert rest == 0
    return out[::-1]


def test_rips_edges_rejects_bad_graphs(ctx):
    import rnng_gb300
    with pytest.raises(rnng_gb300.RnngError):
        ctx.rips_edges(3, [0, 1], [1, 0], [1.0, 1.0])  # the same pair twice
    with pytest.raises(rnng_gb300.RnngError):
        ctx.rips_edges(3, [0], [0], [1.0])  # self-loop
    with pytest.raises(rnng_gb300.RnngError):
        ctx.rips_edges(3, [0], [3], [1.0])  # row out of range
    with pytest.raises(rnng_gb300.RnngError):
        ctx.rips_edges(3, [0], [1], [-1.0])  # negative value
    with pytest.raises(rnng_gb300.RnngError):
        ctx.rips_l2(np.zeros((4, 2), np.float32), 1.0, maxdim=16)
    ids, vals = ctx.rips_edges(4, [], [], [], maxdim=3)
    assert ids.tolist() == [0, 1, 2, 3] and np.all(vals == 0)


@pytest.mark.parametrize("maxdim", [0, 1, 2])
def test_random_against_oracle(ctx, orc, maxdim):
    rng = np.random.default_rng(maxdim + 50)
    x = rng.normal(size=(900, 5)).astype(np.float32)
    r = np.float32(1.1)
    u, v, w = orc.eps_graph_l2(x, r)
    want = orc.rips(x.shape[0], u, v, w, maxdim)
    assert same(ctx.rips_l2(x, r, maxdim=maxdim), want)


def brute_filtration(orc, x, r, labels):
    """Vertices, edges and triangles over rows, ids from the rows' labels, sorted by
    (value, id); equal (value, id) records are identical, so the sequence is unique."""
    u, v, w = orc.eps_graph_l2(x, r)
    wmap = {(a, b): c for a, b, c in zip(u.tolist(), v.tolist(), w.tolist())}
    adj = {}
    for (a, b) in wmap:
        adj.setdefault(a, set()).add(b)
    lab = labels.tolist()
    want = [(0.0, orc.simplex_id([i])) for i in lab]
    want += [(c, orc.simplex_id([lab[a], lab[b]])) for (a, b), c in wmap.items()]
    for a in adj:
        for b in adj[a]:
            for c in adj[a] & adj.get(b, set()):
                want.append((max(wmap[(a, b)], wmap[(a, c)], wmap[(b, c)]), orc.simplex_id([lab[a], lab[b], lab[c]])))
    want.sort()
    return [t for _, t in want], np.array([val for val, _ in want], np.float32)


@pytest.mark.parametrize("labels", ["spread", "at_bound", "above_bound", "beyond_wrap", "negative", "repeated"])
def test_ids_against_brute_force(ctx, orc, labels):
    """Ids that allow generation in id order (spread, at_bound) and ids that need the
    general sort (above the exact-binomial bound, wrapping binomials, negative or
    repeated ids) give the same filtration as a brute-force enumeration."""
    rng = np.random.default_rng(60)
    x = rng.normal(size=(400, 3)).astype(np.float32)
    r = np.float32(0.9)
    p = rng.permutation(400).astype(np.int64)
    bound = colex_max_id(2)
    ids = {"spread": p * 11 + 5, "at_bound": p + (bound - 399), "above_bound": p + (bound - 398),
           "beyond_wrap": p + 3_000_000, "negative": p - 200,
           "repeated": rng.integers(0, 150, size=400).astype(np.int64)}[labels]
    gi, gv = ctx.rips_l2(x, r, maxdim=2, ids=ids)
    wi, wv = brute_filtration(orc, x, r, ids)
    assert gi.tolist() == wi
    assert np.array_equal(gv.view(np.uint32), wv.view(np.uint32))
    # the same through the edge-list entry point, with flags
    u, v, w = orc.eps_graph_l2(x, r)
    fi, fv, ff = ctx.rips_edges(400, u, v, w, maxdim=2, ids=ids, vertex_flags=np.ones(400, np.uint8))
    assert fi.tolist() == wi and np.array_equal(fv.view(np.uint32), wv.view(np.uint32)) and np.all(ff == 1)


def test_edge_cases(ctx):
    rng = np.random.default_rng(61)
    x = rng.normal(size=(400, 3)).astype(np.float32)
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
    u, v, w = orc.eps_graph_l2(x, r)  # the oracle's own edges, all pairs
    want = orc.rips(x.shape[0], u, v, w, 2)
    got = ctx.rips_l2(x, r, maxdim=2, mode="bf16")
    assert same(got, want) and got[0].size > 1_000_000
