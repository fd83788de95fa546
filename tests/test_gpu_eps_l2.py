"""GPU L2 epsilon graph (both tile modes) against the CPU oracle and the golden
fixtures made by RNNG's own code.  Bar: bit-exact edge sets and weights."""
import numpy as np
import pytest

from conftest import golden, golden_points

pytestmark = pytest.mark.gpu
MODES = ["fp32", "bf16"]


def same(a, b):
    (u1, v1, w1), (u2, v2, w2) = a, b
    return (np.array_equal(u1, u2) and np.array_equal(v1, v2)
            and np.array_equal(np.asarray(w1, np.float32).view(np.uint32), np.asarray(w2, np.float32).view(np.uint32)))


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("name", ["k1_systolic", "k2_landmark", "k5_landmark", "nan_systolic"])
def test_golden_fixture(ctx, mode, name):
    g = golden(name)
    got = ctx.eps_graph_l2(golden_points(g), g["radius"], mode=mode)
    assert same(got, (g["u"], g["v"], g["w"]))


CASES = [
    # (n, d, scale, radius, seed)
    (2, 3, 1.0, 10.0, 0),
    (127, 5, 1.0, 1.0, 1),
    (129, 16, 1.0, 3.0, 2),
    (300, 64, 1.0, 9.0, 3),
    (1000, 33, 0.5, 3.0, 4),
    (2000, 128, 1.0, 14.5, 5),
    (777, 200, 1.0, 18.0, 6),
    (3000, 8, 3.0, 1.2, 7),
]


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("case", CASES)
def test_random_against_oracle(ctx, orc, mode, case):
    n, d, scale, r, seed = case
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-10, 10, size=(8, d))
    x = (centres[rng.integers(0, 8, n)] + scale * rng.normal(size=(n, d))).astype(np.float32)
    want = orc.eps_graph_l2(x, np.float32(r))
    got = ctx.eps_graph_l2(x, np.float32(r), mode=mode)
    assert same(got, want), (len(got[0]), len(want[0]))


@pytest.mark.parametrize("nt", [1, 2, 3])
@pytest.mark.parametrize("case", CASES)
def test_item_forms_against_oracle(ctx, orc, case, nt):
    """Every item form of the Gram kernel - one row tile with one or two column tiles, or a
    pair of row tiles with one column tile (odd and even tile counts) - gives RNNG's edges,
    with small queue chunks so that even these sizes take many chunks."""
    n, d, scale, r, seed = case
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-10, 10, size=(8, d))
    x = (centres[rng.integers(0, 8, n)] + scale * rng.normal(size=(n, d))).astype(np.float32)
    want = orc.eps_graph_l2(x, np.float32(r))
    ctx.set_gram_tuning(nt, 5, 0)
    try:
        got = ctx.eps_graph_l2(x, np.float32(r), mode="bf16")
        st = ctx.stats()
    finally:
        ctx.set_gram_tuning(0, 0, 0)
    assert same(got, want), (len(got[0]), len(want[0]))
    if st["gram_nt"] and d <= 128:
        assert st["gram_nt"] == nt


@pytest.mark.parametrize("mode", MODES)
def test_edge_cases(ctx, orc, mode):
    # empty and single point
    for n in (0, 1):
        u, v, w = ctx.eps_graph_l2(np.zeros((n, 4), np.float32), 1.0, mode=mode)
        assert u.size == 0
    # duplicates: every pair is an edge at distance 0, also with radius 0
    x = np.ones((300, 12), np.float32)
    for r in (0.0, 0.5):
        u, v, w = ctx.eps_graph_l2(x, r, mode=mode)
        assert u.size == 300 * 299 // 2 and np.all(w == 0)
    # negative radius admits nothing
    u, v, w = ctx.eps_graph_l2(x, -1.0, mode=mode)
    assert u.size == 0
    # radius exactly at a realised distance is included (<=)
    rng = np.random.default_rng(9)
    y = rng.normal(size=(500, 7)).astype(np.float32)
    ou, ov, ow = orc.eps_graph_l2(y, np.float32(1.0))
    r = ow[len(ow) // 2]
    assert same(ctx.eps_graph_l2(y, r, mode=mode), orc.eps_graph_l2(y, r))
    # explicit ids: edges are reported in id space with u < v
    ids = (np.arange(500, dtype=np.int64)[::-1] * 3 + 11).copy()
    gu, gv, gw = ctx.eps_graph_l2(y, r, mode=mode, ids=ids)
    wu, wv = ids[ou[ow <= r]], ids[ov[ow <= r]]
    a, b = np.minimum(wu, wv), np.maximum(wu, wv)
    order = np.lexsort((b, a))
    assert np.array_equal(gu, a[order]) and np.array_equal(gv, b[order])


@pytest.mark.parametrize("mode", MODES)
def test_integer_descriptors_30k(ctx, orc, mode):
    from rnng_gb300 import synth
    x = synth.descriptor(n=30000, d=128, k=30, seed=12)
    r = synth.EPS_K2
    assert same(ctx.eps_graph_l2(x, r, mode=mode), orc.eps_graph_l2(x, r))


def test_small_dimensions_take_fp32_tiles(ctx, orc):
    """BF16 mode evaluates tiles of fewer than 16 dimensions on the CUDA cores (no Gram
    kernel time), from 16 on with the tensor-core Gram form; both give RNNG's edges."""
    from rnng_gb300 import synth
    for d, gram in ((8, False), (15, False), (16, True)):
        x = synth.l2_mixture(n=3000, d=d, seed=d)
        r = np.float32(1.1 * np.sqrt(d))
        got = ctx.eps_graph_l2(x, r, mode="bf16")
        assert (ctx.stats()["ms_gram"] > 0) == gram
        assert same(got, orc.eps_graph_l2(x, r)) and got[0].size > 0


def test_modes_agree_and_fp64_error(ctx, orc):
    """Both modes give the oracle's edges on a Zipf mixture (the folded BF16 kernel), and
    RNNG's FP32 weights stay within 1e-5 radius of the exact distance."""
    from rnng_gb300 import synth
    x = synth.zipf_mixture(n=40000, d=32, k=256, seed=21)
    r = np.float32(4.5)
    a = ctx.eps_graph_l2(x, r, mode="fp32")
    b = ctx.eps_graph_l2(x, r, mode="bf16")
    assert same(a, orc.eps_graph_l2(x, r)) and same(a, b) and a[0].size > 0
    u, v, w = a
    d64 = np.sqrt(((x[u].astype(np.float64) - x[v].astype(np.float64)) ** 2).sum(1))
    assert np.max(np.abs(w - d64)) < 1e-5 * max(1.0, float(r))


@pytest.mark.parametrize("mode", MODES)
def test_both_pruning_paths_exact(ctx, orc, mode):
    """Tile pairs are pruned on the tensor cores when the BF16 ball test is tight (compact
    integer descriptors) and by the FP32 ball test when its error terms would widen it
    (tight clusters whose spread is large against eps); both keep every edge."""
    from rnng_gb300 import synth
    rng = np.random.default_rng(32)
    far = rng.normal(size=(40, 16))
    far = 1000.0 * far / np.linalg.norm(far, axis=1, keepdims=True)  # tight clusters on a sphere of radius 1000
    spread = (far[rng.integers(0, 40, 8000)] + 0.1 * rng.normal(size=(8000, 16))).astype(np.float32)
    cases = [(synth.descriptor(n=20000, d=128, k=20, seed=31), synth.EPS_K2, 1),
             (spread, np.float32(0.45), 0)]
    for x, r, tensor in cases:
        got = ctx.eps_graph_l2(x, r, mode=mode)
        st = ctx.stats()
        assert st["prune_tensor"] == tensor, st["prune_widen"]
        assert same(got, orc.eps_graph_l2(x, r)) and got[0].size > 0


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("d", [8, 24, 100, 300])
def test_nonfinite_rows(ctx, orc, mode, d):
    """Rows with a NaN or infinite coordinate get no edges and leave every other edge in
    place (RNNG's dist <= radius is false for them); NaN, +inf and -inf, single
    coordinates and whole rows, in every tile position."""
    import rnng_gb300
    if mode == "bf16" and d > 256:
        pytest.skip("BF16 mode supports d <= 256")
    rng = np.random.default_rng(d)
    n = 3000
    centres = rng.uniform(-6, 6, size=(10, d))
    x = (centres[rng.integers(0, 10, n)] + rng.normal(size=(n, d))).astype(np.float32)
    r = np.float32(np.sqrt(2.0 * d) * 0.9)
    bad = rng.choice(n, size=90, replace=False)
    vals = np.array([np.nan, np.inf, -np.inf], np.float32)
    x[bad[:60], rng.integers(0, d, size=60)] = vals[np.arange(60) % 3]
    x[bad[60:75]] = np.nan
    x[bad[75:], :] = np.inf
    want = orc.eps_graph_l2(x, r)
    assert want[0].size > 1000
    got = ctx.eps_graph_l2(x, r, mode=mode)
    assert same(got, want)
    assert not np.isin(got[0], bad).any() and not np.isin(got[1], bad).any()
    # through the Rips entry point: non-finite rows stay vertices without edges
    ids, vals_ = ctx.rips_l2(x[:800], r, maxdim=1, mode=mode)
    u, v, w = orc.eps_graph_l2(x[:800], r)
    wi, wv = orc.rips(800, u, v, w, 1)
    assert np.array_equal(ids, wi) and np.array_equal(vals_.view(np.uint32), wv.view(np.uint32))
    # all rows but one, and all rows, non-finite
    y = np.full((500, d), np.nan, np.float32)
    assert ctx.eps_graph_l2(y, r, mode=mode)[0].size == 0
    y[7] = 0.0
    assert ctx.eps_graph_l2(y, r, mode=mode)[0].size == 0
    y[300] = 0.0
    u, v, w = ctx.eps_graph_l2(y, r, mode=mode)
    assert u.tolist() == [7] and v.tolist() == [300] and w.tolist() == [0.0]
    # an infinite radius would admit pairs at distance +inf: refused, not guessed
    with pytest.raises(rnng_gb300.RnngError) as e:
        ctx.eps_graph_l2(x, np.float32(np.inf), mode=mode)
    assert e.value.code == 6
    # ... unless every non-finite row holds a NaN (at distance NaN from everything): then
    # the graph is complete over the finite rows
    y = x[:260].copy()
    y[~np.isfinite(y).all(axis=1), 0] = np.nan
    y[5, 1] = np.nan
    want = orc.eps_graph_l2(y, np.float32(np.inf))
    assert same(ctx.eps_graph_l2(y, np.float32(np.inf), mode=mode), want)
    k = int(np.isfinite(y).all(axis=1).sum())
    assert want[0].size == k * (k - 1) // 2
    # the context stays usable and finite inputs take the unscreened path again
    z = x[np.isfinite(x).all(axis=1)]
    assert same(ctx.eps_graph_l2(z, r, mode=mode), orc.eps_graph_l2(z, r))


@pytest.mark.parametrize("mode", MODES)
def test_unbounded_radius(ctx, orc, mode):
    """radius +inf, FLT_MAX and 1e30 admit every pair, also for integer points that BF16
    holds exactly (every tile's error radius 0, where an infinite threshold times 0
    would be NaN)."""
    rng = np.random.default_rng(77)
    xi = rng.integers(0, 16, size=(300, 16)).astype(np.float32)
    xf = rng.normal(size=(300, 16)).astype(np.float32)
    for x in (xi, xf):
        for r in (np.float32(np.inf), np.float32(np.finfo(np.float32).max), np.float32(1e30)):
            want = orc.eps_graph_l2(x, r)
            assert want[0].size == 300 * 299 // 2
            assert same(ctx.eps_graph_l2(x, r, mode=mode), want)
    ids, vals = ctx.rips_l2(xi[:60], np.float32(np.inf), maxdim=2, mode=mode)
    u, v, w = orc.eps_graph_l2(xi[:60], np.float32(np.inf))
    wi, wv = orc.rips(60, u, v, w, 2)
    assert wi.size == 60 + 60 * 59 // 2 + 60 * 59 * 58 // 6
    assert np.array_equal(ids, wi) and np.array_equal(vals.view(np.uint32), wv.view(np.uint32))


SCALES = [-75, -70, -60, -40, 40, 58, 61]


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("e", SCALES)
def test_power_of_two_scales(ctx, orc, mode, e):
    """The same point set scaled by 2^e (exact in float32): RNNG's L2 of the scaled
    points, subnormal squares at the small end included, decides the edges."""
    rng = np.random.default_rng(88)
    centres = rng.uniform(-4, 4, size=(6, 16))
    base = (centres[rng.integers(0, 6, 2500)] + rng.normal(size=(2500, 16))).astype(np.float32)
    s = np.float32(2.0 ** e)
    x = (base * s).astype(np.float32)
    r = np.float32(np.float32(3.6) * s)
    want = orc.eps_graph_l2(x, r)
    assert want[0].size > 3000
    assert same(ctx.eps_graph_l2(x, r, mode=mode), want)


def test_gram_tuning_table_and_override(ctx, orc):
    """The Gram kernel's work-queue chunk, column tiles per item and B slots come from the
    committed tuning table (rnng_gb300/gram_tuning.json) and can be forced per context;
    every setting gives RNNG's edges."""
    import json
    import os

    from rnng_gb300 import synth
    table = json.load(open(os.path.join(os.path.dirname(synth.__file__), "gram_tuning.json")))["rows"]
    row = min((r for r in table if r["kind"] == "bf16" and r["dp"] == 64), key=lambda r: r["min_pairs"])
    x = synth.zipf_mixture(n=20000, d=32, k=64, seed=41)
    r = np.float32(4.5)
    want = orc.eps_graph_l2(x, r)
    got = ctx.eps_graph_l2(x, r, mode="bf16")
    st = ctx.stats()
    assert st["tile_pairs"] < max(t["min_pairs"] for t in table if t["dp"] == 64) or len(table) == 1
    assert (st["gram_nt"], st["gram_chunk"]) == (row["nt"], row["chunk"])
    assert same(got, want)
    for nt, chunk, slots in ((2, 1, 2), (1, 2, 3), (2, 7, 0), (1, 5, 2), (3, 1, 2), (3, 9, 0)):
        ctx.set_gram_tuning(nt, chunk, slots)
        got = ctx.eps_graph_l2(x, r, mode="bf16")
        st = ctx.stats()
        assert st["gram_nt"] == nt and st["gram_chunk"] == (chunk + (chunk & 1 if nt == 1 else 0))
        assert same(got, want)
    ctx.set_gram_tuning(0, 0, 0)
    ctx.eps_graph_l2(x, r, mode="bf16")
    assert (ctx.stats()["gram_nt"], ctx.stats()["gram_chunk"]) == (row["nt"], row["chunk"])


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("d", [32, 128])
def test_device_points_off_16_byte_boundary(ctx, orc, mode, d):
    """Device points that start 4 bytes past a 16-byte boundary (a view into a larger
    buffer) give the oracle's edges: the library copies them to an aligned buffer before
    its 16-byte loads (host-side result, INPUT_DEVICE only)."""
    torch = pytest.importorskip("torch")
    import rnng_gb300
    rng = np.random.default_rng(40 + d)
    n = 1500
    centres = rng.uniform(-10, 10, size=(8, d))
    x = (centres[rng.integers(0, 8, n)] + rng.normal(size=(n, d))).astype(np.float32)
    r = np.float32(1.6 * np.sqrt(d))
    want = orc.eps_graph_l2(x, r)
    buf = torch.zeros(n * d + 1, dtype=torch.float32, device="cuda")
    buf[1:] = torch.from_numpy(x.reshape(-1)).cuda()
    xd = buf[1:]
    assert xd.data_ptr() % 16 == 4
    e = ctx.eps_graph_l2_raw(xd.data_ptr(), None, n, d, r, rnng_gb300.MODES[mode],
                             rnng_gb300.INPUT_DEVICE | rnng_gb300.SORT_OUTPUT)
    assert same(ctx._edges_out(e), want)


@pytest.mark.parametrize("d", [33, 128])
@pytest.mark.parametrize("case", ["plain", "ids", "nonfinite"])
def test_unsorted_host_results_written_by_the_recheck(ctx, orc, d, case):
    """Host results without sorting come straight from the recheck (it writes each edge as
    input ids u < v and its weight into the pinned staging block): the same edges and
    weight bits as the oracle's, with caller ids and with rows left out for NaNs."""
    rng = np.random.default_rng(70 + d)
    n = 6000
    centres = rng.uniform(-10, 10, size=(12, d))
    x = (centres[rng.integers(0, 12, n)] + rng.normal(size=(n, d))).astype(np.float32)
    r = np.float32(1.5 * np.sqrt(d))
    ids = None
    if case == "nonfinite":
        x[rng.choice(n, 25, replace=False), rng.integers(0, d, 25)] = np.nan
    want = orc.eps_graph_l2(x, r)
    if case == "ids":
        ids = (rng.permutation(n).astype(np.int64) * 7 + 11)
        u, v = ids[want[0]], ids[want[1]]
        want = (np.minimum(u, v), np.maximum(u, v), want[2])
        o = np.lexsort((want[1], want[0]))
        want = tuple(a[o] for a in want)
    u, v, w = ctx.eps_graph_l2(x, r, mode="bf16", ids=ids, sort=False)
    assert (u < v).all()
    o = np.lexsort((v, u))
    assert same((u[o], v[o], w[o]), want)
