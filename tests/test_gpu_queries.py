"""Batch radius queries, exact Voronoi assignment and Graph finalisation on the GPU,
against the oracle (bit-exact)."""
import numpy as np
import pytest

from conftest import golden, golden_points

pytestmark = pytest.mark.gpu


def test_radius_query_matches_oracle(ctx, orc):
    rng = np.random.default_rng(40)
    x = rng.normal(size=(3000, 17)).astype(np.float32)
    q = (rng.normal(size=(700, 17)) * 1.1).astype(np.float32)
    r = np.float32(3.2)
    want = orc.cross_l2(x, q, r)  # (query row, point row)
    got = ctx.radius_query_l2(x, q, r)
    assert all(np.array_equal(a, b) for a, b in zip(got[:2], want[:2]))
    assert np.array_equal(got[2].view(np.uint32), want[2].view(np.uint32))
    ids = np.arange(3000, dtype=np.int64) * 5 + 1
    qids = np.arange(700, dtype=np.int64) + 100000
    gu, gv, gw = ctx.radius_query_l2(x, q, r, ids=ids, qids=qids)
    o = np.lexsort((ids[want[1]], qids[want[0]]))
    assert np.array_equal(gu, qids[want[0]][o]) and np.array_equal(gv, ids[want[1]][o])
    # the indexed set queried with itself includes every self match at distance 0
    su, sv, sw = ctx.radius_query_l2(x[:500], x[:500], r)
    assert np.sum(su == sv) == 500 and np.all(sw[su == sv] == 0)
    # empty batch
    assert ctx.radius_query_l2(x, q[:0], r)[0].size == 0


@pytest.mark.parametrize("m", [1, 7, 33, 100])
def test_voronoi_matches_reference_rule(ctx, orc, m):
    g = golden("k1_landmark")
    x = golden_points(g)
    c = x[(np.arange(m) * len(x)) // m]
    cell, dist = ctx.voronoi_l2(x, c)
    wc, wd = orc.voronoi(x, c)
    assert np.array_equal(cell, wc) and np.array_equal(dist.view(np.uint32), wd.view(np.uint32))


def test_nonfinite_points_and_centres(ctx, orc):
    """NaN and infinite coordinates: a query or point with one matches nothing, a
    point whose distances are all NaN keeps cell 0 at FLT_MAX (the reference's initial
    best), and a NaN centre is never nearest - as in RNNG's loops."""
    rng = np.random.default_rng(41)
    x = rng.normal(size=(2000, 9)).astype(np.float32)
    q = rng.normal(size=(500, 9)).astype(np.float32)
    x[rng.choice(2000, 50, replace=False), rng.integers(0, 9, 50)] = np.nan
    x[rng.choice(2000, 20, replace=False), rng.integers(0, 9, 20)] = -np.inf
    q[rng.choice(500, 30, replace=False), rng.integers(0, 9, 30)] = np.inf
    want = orc.cross_l2(x, q, np.float32(2.5))
    got = ctx.radius_query_l2(x, q, np.float32(2.5))
    assert all(np.array_equal(a, b) for a, b in zip(got[:2], want[:2])) and want[0].size > 1000
    assert np.array_equal(got[2].view(np.uint32), want[2].view(np.uint32))
    c = x[::97].copy()
    c[3] = np.nan
    c[5, 2] = np.inf
    cell, dist = ctx.voronoi_l2(x, c)
    wc, wd = orc.voronoi(x, c)
    assert np.array_equal(cell, wc) and np.array_equal(dist.view(np.uint32), wd.view(np.uint32))
    assert not np.any(cell == 3)


def test_voronoi_ties_go_to_the_last_centre(ctx):
    x = np.zeros((5, 3), np.float32)
    c = np.zeros((4, 3), np.float32)  # four identical centres: every point ties
    cell, dist = ctx.voronoi_l2(x, c)
    assert np.all(cell == 3) and np.all(dist == 0)


def test_graph_finalize_matches_reference_semantics(ctx, orc):
    g = golden("k1_systolic")
    x = golden_points(g)
    u, v, w = ctx.eps_graph_l2(x, g["radius"], mode="bf16")
    fu, fv, fw = ctx.graph_finalize(u, v, w, x.shape[0])
    assert fu.size == int(g["reported_edges"])
    # every vertex has its self-loop, and both orientations are present, sorted
    ru = np.concatenate([np.arange(x.shape[0]), u, v])
    rv = np.concatenate([np.arange(x.shape[0]), v, u])
    rw = np.concatenate([np.zeros(x.shape[0], np.float32), w, w])
    o = np.lexsort((rv, ru))
    assert np.array_equal(fu, ru[o]) and np.array_equal(fv, rv[o])
    assert np.array_equal(fw.view(np.uint32), rw[o].view(np.uint32))


@pytest.mark.parametrize("m", [1, 7, 30])
def test_voronoi_edit_matches_oracle(ctx, orc, m):
    from rnng_gb300 import synth
    seqs = synth.dna_families(n_seeds=40, mutants=12, seed=m)
    atoms, offsets = synth.pack_seqs(seqs)
    rng = np.random.default_rng(m)
    lm = np.sort(rng.choice(len(seqs), size=m, replace=False))
    cseqs = [seqs[i] for i in lm]
    catoms, coffsets = synth.pack_seqs(cseqs)
    cell, dist = ctx.voronoi_edit((atoms, offsets), (catoms, coffsets))
    wc, wd = orc.voronoi_edit(atoms, offsets, catoms, coffsets)
    assert np.array_equal(cell, wc) and np.array_equal(dist, wd)


def test_voronoi_edit_long_and_empty_strings(ctx, orc):
    """Centres of 0 to 700 characters (1..11 words), ties between equal centres."""
    rng = np.random.default_rng(5)
    alphabet = np.frombuffer(b"ACGTN", np.uint8)
    seqs = [bytes(rng.choice(alphabet, size=int(rng.integers(0, 700)))) for _ in range(300)] + [b""]
    centres = [b"", seqs[3], seqs[3], bytes(rng.choice(alphabet, size=700)), seqs[10][:64], seqs[11][:65]]
    import rnng_gb300
    atoms, offsets = rnng_gb300._csr(seqs)
    catoms, coffsets = rnng_gb300._csr(centres)
    cell, dist = ctx.voronoi_edit((atoms, offsets), (catoms, coffsets))
    wc, wd = orc.voronoi_edit(atoms, offsets, catoms, coffsets)
    assert np.array_equal(cell, wc) and np.array_equal(dist, wd)
    assert cell[3] == 2  # equal centres: the last wins
