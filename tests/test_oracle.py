"""The CPU oracle pinned against RNNG's own outputs (golden fixtures made by running
RNNG's headers, tests/golden/make_golden.py) and against hand-checked known answers."""
import itertools
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden, golden_points, graph_text


def _have_rnng_sources() -> bool:
    import oracle
    return oracle.ref_source_dir() is not None


EDGE_FIXTURES = ["k1_systolic", "k1_landmark", "k2_landmark", "k5_landmark", "nan_systolic", "nan_landmark"]


@pytest.mark.parametrize("name", EDGE_FIXTURES)
def test_oracle_l2_matches_reference(orc, name):
    g = golden(name)
    x = golden_points(g)
    u, v, w = orc.eps_graph_l2(x, g["radius"])
    assert np.array_equal(u, g["u"]) and np.array_equal(v, g["v"])
    assert np.array_equal(w.view(np.uint32), g["w"].view(np.uint32))
    # the driver's printed count is its self-loops plus both orientations of every edge;
    # a row with a NaN coordinate is at distance NaN from itself and has no self-loop
    assert int(g["reported_edges"]) == int(np.isfinite(x).all(axis=1).sum()) + 2 * u.size


def test_oracle_edit_matches_reference(orc):
    g = golden("k3_edit")
    u, v, w = orc.eps_graph_edit(g["atoms"], g["offsets"], g["radius"])
    assert np.array_equal(u, g["u"]) and np.array_equal(v, g["v"])
    assert np.array_equal(w, g["w"])
    assert int(g["reported_edges"]) == int(g["n"]) + 2 * u.size


@pytest.mark.parametrize("name", ["k4_rips", "k4_rips3", "k3_rips_edit", "nan_rips"])
def test_oracle_rips_matches_reference(orc, name):
    g = golden(name)
    if "atoms" in g:
        u, v, w = orc.eps_graph_edit(g["atoms"], g["offsets"], g["radius"])
    else:
        u, v, w = orc.eps_graph_l2(g["x"], g["radius"])
    ids, vals = orc.rips(int(g["n"]), u, v, w, int(g["maxdim"]))
    assert np.array_equal(ids, g["ids"])
    assert np.array_equal(vals.view(np.uint32), g["values"].view(np.uint32))
    dims = np.asarray(g["ids"]).view(np.uint64) >> np.uint64(60)
    assert int(dims.max()) == int(g["maxdim"])  # the top dimension is populated


def test_reference_isolates_nan_rows():
    """What RNNG's own paths did with NaN coordinates: the systolic and landmark drivers
    give the same edges, no edge touches a row with a NaN, and the rips filtration keeps
    those rows as vertices (value 0) with no higher simplex on them."""
    a, b = golden("nan_systolic"), golden("nan_landmark")
    for k in ("u", "v", "w"):
        assert np.array_equal(a[k], b[k])
    bad = np.nonzero(~np.isfinite(a["x"]).all(axis=1))[0]
    assert bad.size == 45
    assert not np.isin(a["u"], bad).any() and not np.isin(a["v"], bad).any()
    r = golden("nan_rips")
    bad_r = np.nonzero(~np.isfinite(r["x"]).all(axis=1))[0]
    ids = np.asarray(r["ids"]).view(np.uint64)
    dims = ids >> np.uint64(60)
    verts = ids[dims == 0].astype(np.int64)
    assert np.isin(bad_r, verts).all() and verts.size == int(r["n"])
    # an edge id is a + C(b, 2) with a < b: no edge may carry a NaN row as either end
    e = (ids[dims == 1] & np.uint64((1 << 60) - 1)).astype(np.int64)
    hi = np.floor((1 + np.sqrt(1 + 8 * e.astype(np.float64))) / 2).astype(np.int64)
    hi -= (hi * (hi - 1) // 2 > e)
    lo = e - hi * (hi - 1) // 2
    assert np.all(lo < hi) and not np.isin(hi, bad_r).any() and not np.isin(lo, bad_r).any()


CELL_FIXTURES = ["k1_cells", "k1_cells_rips", "k3_cells", "dup_cells"]


@pytest.mark.parametrize("name", CELL_FIXTURES)
def test_oracle_cells_match_reference(orc, name):
    """Voronoi assignment, coalescing, ghosts and interior flags restated in Python
    (oracle.landmark_cells) equal RNNG's, including its empty-cell indexing."""
    g = golden(name)
    metric = "edit" if "atoms" in g else "l2"
    data = (g["atoms"], g["offsets"]) if metric == "edit" else g["x"]
    r = orc.landmark_cells(metric, data, g["landmarks"], g["radius"], bool(g["rips"]))
    for k in r:
        assert np.array_equal(r[k], g[k]), k
    if name == "dup_cells":
        assert (g["npts"] == 0).sum() > 0 and g["ghosts"].size > 0


def test_oracle_voronoi_edit_matches_reference(orc):
    g = golden("k3_cells")
    lm = g["landmarks"]
    atoms, offsets = g["atoms"], g["offsets"]
    catoms = np.concatenate([atoms[offsets[i]:offsets[i + 1]] for i in lm])
    coffsets = np.concatenate([[0], np.cumsum([offsets[i + 1] - offsets[i] for i in lm])]).astype(np.int64)
    cell, dist = orc.voronoi_edit(atoms, offsets, catoms, coffsets)
    want_cell = np.repeat(g["cell_id"], g["npts"])
    order = np.argsort(g["ids"])
    assert np.array_equal(cell, want_cell[order])
    assert np.array_equal(dist, g["dist"][order])


def _lev(s, t):
    prev = list(range(len(t) + 1))
    for i, a in enumerate(s, 1):
        cur = [i]
        for j, b in enumerate(t, 1):
            cur.append(min(prev[j] + 1, cur[j - 1] + 1, prev[j - 1] + (a != b)))
        prev = cur
    return prev[-1]


def test_edit_known_answers(orc):
    cases = [(b"kitten", b"sitting", 3), (b"", b"abc", 3), (b"abc", b"", 3), (b"", b"", 0), (b"abc", b"abc", 0),
             (b"flaw", b"lawn", 2), (b"ACGT", b"TGCA", 4), (b"AAAA", b"AAA", 1)]
    for s, t, want in cases:
        assert orc.edit(s, t) == want
    rng = np.random.default_rng(0)
    for _ in range(200):
        s = bytes(rng.choice(list(b"ACGT"), size=rng.integers(0, 40)))
        t = bytes(rng.choice(list(b"ACGT"), size=rng.integers(0, 40)))
        assert orc.edit(s, t) == _lev(s, t) == orc.edit(t, s)


def test_l2seq_is_sequential_float32(orc):
    rng = np.random.default_rng(1)
    for d in (1, 3, 8, 31, 128, 200):
        p = rng.normal(size=d).astype(np.float32) * 7
        q = rng.normal(size=d).astype(np.float32) * 7
        acc = np.float32(0)
        for k in range(d):
            delta = np.float32(p[k] - q[k])
            acc = np.float32(acc + np.float32(delta * delta))
        assert orc.l2seq(p, q) == np.sqrt(acc, dtype=np.float32)
        assert orc.l2seq(p, q) == orc.l2seq(q, p)


def test_binom_and_simplex_ids(orc):
    assert orc.binom(5, 2) == 10 and orc.binom(0, 1) == 0 and orc.binom(1, 2) == 0 and orc.binom(7, 0) == 1
    assert orc.binom(500000, 3) == 500000 * 499999 * 499998 // 6
    assert orc.simplex_id([3]) == 3
    assert orc.simplex_id([4, 1]) == (1 + 6) | (1 << 60)
    assert orc.simplex_id([0, 2, 5]) == (0 + 1 + 10) | (2 << 60)


def test_rips_against_brute_force(orc):
    rng = np.random.default_rng(2)
    n = 40
    x = rng.normal(size=(n, 3)).astype(np.float32)
    r = np.float32(1.2)
    u, v, w = orc.eps_graph_l2(x, r)
    wmap = {(a, b): c for a, b, c in zip(u.tolist(), v.tolist(), w.tolist())}
    want = [(0.0, orc.simplex_id([i])) for i in range(n)]
    want += [(c, orc.simplex_id([a, b])) for (a, b), c in wmap.items()]
    for a, b, c in itertools.combinations(range(n), 3):
        if (a, b) in wmap and (a, c) in wmap and (b, c) in wmap:
            want.append((max(wmap[(a, b)], wmap[(a, c)], wmap[(b, c)]), orc.simplex_id([a, b, c])))
    want.sort()
    ids, vals = orc.rips(n, u, v, w, 2)
    assert [int(i) for i in ids] == [i for _, i in want]
    assert np.array_equal(vals, np.array([val for val, _ in want], np.float32))


@pytest.mark.skipif(not _have_rnng_sources(), reason="needs the RNNG sources ($RNNG_SRC) to build its drivers")
def test_unchanged_reference_drivers_agree(orc, tmp_path):
    """RNNG's own drivers, built unchanged against the MPI shim, report the fixture's counts."""
    orc.build(ref=True)
    g = golden("k1_systolic")
    from rnng_gb300 import synth
    p = str(tmp_path / "k1.fvecs")
    synth.write_fvecs(p, g["x"])
    for drv, extra in (("systolic", []), ("landmark", ["-m", "30", "-F", "-s", "7"])):
        out = str(tmp_path / f"{drv}.mtx")
        r = subprocess.run([os.path.join(ROOT, "oracle", "_ref", drv), "-i", p, "-r", "1.5", "-o", out] + extra,
                           capture_output=True, text=True, check=True)
        assert f"edges={int(g['reported_edges'])}" in r.stderr
        lines = open(out).read().split("\n")
        assert lines[0].split()[-1] == str(int(g["reported_edges"]))


@pytest.mark.parametrize("name,centres", [("k1_systolic", 30), ("k2_landmark", 12), ("k5_landmark", 25),
                                          ("nan_landmark", 9)])
def test_landmark_pipeline_port_matches_brute_force(orc, name, centres):
    """RNNG's landmark pipeline restated on the CPU (oracle/landmark.c: Voronoi cells,
    cover trees, ghosts, batched radius queries) finds exactly the brute-force edges,
    on one thread and on all threads."""
    g = golden(name)
    x = golden_points(g)
    want = orc.eps_graph_l2(x, g["radius"])
    full = orc.num_threads()
    for threads in (1, full):
        orc.set_threads(threads)
        (u, v, w), info = orc.landmark_l2(x, g["radius"], num_centers=centres)
        assert np.array_equal(u, want[0]) and np.array_equal(v, want[1])
        assert np.array_equal(w.view(np.uint32), want[2].view(np.uint32))
        assert info["num_cells"] == centres and info["threads"] == threads
    orc.set_threads(full)


@pytest.mark.parametrize("centres", [1, 7, 40])
def test_landmark_pipeline_port_edit_distance(orc, centres):
    """The same pipeline under RNNG's edit distance (its driver's `-D edit` path) finds
    the edges RNNG's own driver found on the DNA fixture, on one thread and on all."""
    g = golden("k3_edit")
    full = orc.num_threads()
    for threads in (1, full):
        orc.set_threads(threads)
        (u, v, w), info = orc.landmark_edit(g["atoms"], g["offsets"], g["radius"], num_centers=centres)
        order = np.lexsort((v, u))
        u, v, w = u[order], v[order], w[order]
        assert np.array_equal(u, g["u"]) and np.array_equal(v, g["v"])
        assert np.array_equal(w.view(np.uint32), g["w"].view(np.uint32))
        assert info["num_cells"] == centres and info["threads"] == threads
    orc.set_threads(full)


def test_landmark_pipeline_port_duplicates_and_tiny(orc):
    rng = np.random.default_rng(5)
    x = np.repeat(rng.normal(size=(40, 5)).astype(np.float32), 7, axis=0)
    for r, m in ((0.0, 10), (0.8, 40), (5.0, 3), (0.8, 25)):
        want = orc.eps_graph_l2(x, np.float32(r))
        (u, v, w), info = orc.landmark_l2(x, np.float32(r), num_centers=m)
        if info["empty_cells"] == 0:
            assert np.array_equal(u, want[0]) and np.array_equal(v, want[1])
        else:  # RNNG's ghost step indexes cells by non-empty position: edges can go missing
            assert np.isin(u * x.shape[0] + v, want[0] * x.shape[0] + want[1]).all()
    for n in (0, 1, 2):
        (u, v, w), _ = orc.landmark_l2(np.zeros((n, 3), np.float32), 1.0, num_centers=1)
        assert u.size == (1 if n == 2 else 0)


@pytest.mark.skipif(not _have_rnng_sources(), reason="needs the RNNG sources ($RNNG_SRC) to build its drivers")
@pytest.mark.parametrize("name,m", [("k1_landmark", 30), ("nan_landmark", 20)])
def test_graph_text_matches_reference_driver(orc, tmp_path, name, m):
    """The expected graph file the drop-in test compares with is the file RNNG's own
    pipeline writes (Graph + redistribute_edges + write_file, the harness's graph mode)."""
    orc.build(ref=True)
    from rnng_gb300 import synth
    g = golden(name)
    x = golden_points(g)
    p = str(tmp_path / "in.fvecs")
    synth.write_fvecs(p, x)
    out = str(tmp_path / "out.mtx")
    subprocess.run([os.path.join(ROOT, "oracle", "_ref", "ref_harness"), "graph", "l2", p, repr(float(g["radius"])),
                    str(m), "7", out], check=True, capture_output=True)
    assert open(out).read() == graph_text(g, x.shape[0])
