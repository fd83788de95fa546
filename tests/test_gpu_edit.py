"""GPU edit-distance epsilon graph against the oracle and the golden fixture made by
RNNG's own landmark path with EditDistance (bit-exact: integer distances)."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


def test_golden_k3(ctx):
    g = golden("k3_edit")
    got = ctx.eps_graph_edit((g["atoms"], g["offsets"]), g["radius"])
    assert same(got, (g["u"], g["v"], g["w"]))


@pytest.mark.parametrize("radius", [0.0, 1.0, 3.5, 8.0, 16.0, 20.0])
def test_dna_families_against_oracle(ctx, orc, radius):
    from rnng_gb300 import synth
    seqs = synth.dna_families(n_seeds=60, mutants=30, rate=0.05, seed=7)
    atoms, offsets = synth.pack_seqs(seqs)
    want = orc.eps_graph_edit(atoms, offsets, np.float32(radius))
    got = ctx.eps_graph_edit((atoms, offsets), np.float32(radius))
    assert same(got, want) and (radius < 1 or got[0].size > 0)


def test_edge_cases(ctx, orc):
    rng = np.random.default_rng(5)
    seqs = [b"", b"", b"A", b"AB", b"BA", b"ABC" * 40, b"ABC" * 40, b"x" * 300, b"x" * 299 + b"y"]
    seqs += [bytes(rng.integers(0, 256, size=rng.integers(0, 50)).astype(np.uint8)) for _ in range(400)]
    atoms, offsets = np.frombuffer(b"".join(seqs), np.uint8), np.zeros(len(seqs) + 1, np.int64)
    np.cumsum([len(s) for s in seqs], out=offsets[1:])
    for r in (0.0, 2.0, 5.0, 12.0):
        want = orc.eps_graph_edit(atoms, offsets, np.float32(r))
        assert same(ctx.eps_graph_edit((atoms, offsets), np.float32(r)), want)
    # ids, a negative radius, and too few strings
    ids = np.arange(len(seqs), dtype=np.int64) * 3 + 7
    u, v, w = ctx.eps_graph_edit((atoms, offsets), 2.0, ids=ids)
    wu, wv, ww = orc.eps_graph_edit(atoms, offsets, np.float32(2.0))
    o = np.lexsort((ids[wv], ids[wu]))
    assert np.array_equal(u, ids[wu][o]) and np.array_equal(v, ids[wv][o])
    assert ctx.eps_graph_edit((atoms, offsets), -1.0)[0].size == 0
    assert ctx.eps_graph_edit([b"ACGT"], 3.0)[0].size == 0
    assert ctx.eps_graph_edit([], 3.0)[0].size == 0


def test_k3_shape_against_oracle(ctx, orc):
    from rnng_gb300 import synth
    seqs = synth.dna_families(n_seeds=125, mutants=40, seed=3)  # 5,000 strings of the K3 kind
    atoms, offsets = synth.pack_seqs(seqs)
    r = synth.EPS_K3
    assert same(ctx.eps_graph_edit((atoms, offsets), r), orc.eps_graph_edit(atoms, offsets, r))


def test_k3_full_size_rows_sample(ctx, orc):
    """The full 200,000-string workload: edges incident to a sample of rows match a
    brute-force oracle over all later strings."""
    from rnng_gb300 import synth
    seqs = synth.dna_families()
    atoms, offsets = synth.pack_seqs(seqs)
    r = synth.EPS_K3
    u, v, w = ctx.eps_graph_edit((atoms, offsets), r)
    assert u.size > 100000
    for r0 in (0, 77777, 199800):
        r1 = r0 + 40
        wu, wv, ww = orc.eps_graph_edit(atoms, offsets, r, rows=(r0, r1))
        sel = (u >= r0) & (u < r1)
        assert same((u[sel], v[sel], w[sel]), (wu, wv, ww))


@pytest.mark.parametrize("nsym", [3, 6])
def test_alphabets_against_oracle(ctx, orc, nsym):
    """Families over 3 symbols (exact 4-gram filter, bins unused) and 6 symbols (hashed
    3-gram filter, bit-vector verification) against the oracle."""
    rng = np.random.default_rng(40 + nsym)
    letters = np.frombuffer(b"QRSTUVWX"[:nsym], np.uint8)
    seqs = []
    for _ in range(50):
        base = letters[rng.integers(0, nsym, size=int(rng.integers(60, 110)))]
        for _ in range(20):
            s = base.copy()
            for _ in range(int(rng.integers(0, 6))):
                p = int(rng.integers(0, s.size))
                op = int(rng.integers(0, 3))
                if op == 0:
                    s[p] = letters[rng.integers(0, nsym)]
                elif op == 1:
                    s = np.insert(s, p, letters[rng.integers(0, nsym)])
                elif s.size > 1:
                    s = np.delete(s, p)
            seqs.append(s.tobytes())
    atoms = np.frombuffer(b"".join(seqs), np.uint8)
    offsets = np.zeros(len(seqs) + 1, np.int64)
    np.cumsum([len(s) for s in seqs], out=offsets[1:])
    for r in (2.0, 6.0):
        want = orc.eps_graph_edit(atoms, offsets, np.float32(r))
        got = ctx.eps_graph_edit((atoms, offsets), np.float32(r))
        assert same(got, want) and got[0].size > 0


def test_short_strings_exact_filter(ctx, orc):
    """Strings shorter than the filter's 4-grams over a DNA alphabet (no q-grams: the
    filter passes them all, verification decides)."""
    seqs = [b"", b"A", b"AC", b"ACG", b"ACGT", b"ACGTA", b"TTT", b"GA", b"", b"CCCC", b"ACGTACGT"] * 13
    atoms = np.frombuffer(b"".join(seqs), np.uint8)
    offsets = np.zeros(len(seqs) + 1, np.int64)
    np.cumsum([len(s) for s in seqs], out=offsets[1:])
    for r in (0.0, 1.0, 3.0):
        assert same(ctx.eps_graph_edit((atoms, offsets), np.float32(r)), orc.eps_graph_edit(atoms, offsets, np.float32(r)))
