"""CPU checks of the arithmetic the GPU paths rely on (no GPU):

- the edit-distance filters: the L1 distance of capped q-gram profiles never exceeds
  2 q x (edit distance), for the exact 4-gram profile (counts capped at 2) and the
  hashed 3-gram profile (capped at 8), and their thermometer rows turn it into
  n_a + n_b - 2 x_a.x_b;
- the Rips id order: below the exact-binomial bound, the colex order of vertex tuples
  is the order of RNNG's simplex ids, dimension by dimension;
- the statistics struct of the C ABI and its Python mirror have the same layout."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, colex_max_id


def _mutate(rng, s, letters, nedits):
    s = list(s)
    for _ in range(nedits):
        op = int(rng.integers(0, 3))
        p = int(rng.integers(0, len(s) + 1))
        if op == 0 and p < len(s):
            s[p] = letters[int(rng.integers(0, len(letters)))]
        elif op == 1:
            s.insert(p, letters[int(rng.integers(0, len(letters)))])
        elif s and p < len(s):
            del s[p]
    return bytes(s)


def _profile_exact4(s, code):
    c = np.zeros(256, np.int64)
    for i in range(len(s) - 3):
        c[code[s[i]] * 64 + code[s[i + 1]] * 16 + code[s[i + 2]] * 4 + code[s[i + 3]]] += 1
    return np.minimum(c, 2)


def _bin3(a, b, c):
    # the library's hashed 3-gram bin (32-bit products, top 6 bits)
    h = ((a * 0x9E3779B1) & 0xFFFFFFFF) ^ ((b * 0x85EBCA77) & 0xFFFFFFFF) ^ ((c * 0xC2B2AE3D) & 0xFFFFFFFF)
    return h >> 26


def _profile_hashed3(s):
    c = np.zeros(64, np.int64)
    for i in range(len(s) - 2):
        c[_bin3(s[i], s[i + 1], s[i + 2])] += 1
    return np.minimum(c, 8)


def _thermometer(p, levels):
    return (p[:, None] > np.arange(levels)[None, :]).astype(np.int64).ravel()


@pytest.mark.parametrize("alphabet", [b"ACGT", b"ACGTUV"])
def test_qgram_filter_bounds(orc, alphabet):
    rng = np.random.default_rng(len(alphabet))
    letters = list(alphabet)
    code = {b: i for i, b in enumerate(letters)}
    for _ in range(300):
        a = bytes(letters[int(k)] for k in rng.integers(0, len(letters), size=int(rng.integers(0, 60))))
        b = _mutate(rng, a, letters, int(rng.integers(0, 10)))
        ed = int(orc.edit(a, b))
        for q, prof, levels in ((3, _profile_hashed3, 8), ) + (((4, lambda s: _profile_exact4(s, code), 2),)
                                                               if len(letters) <= 4 else ()):
            pa, pb = prof(a), prof(b)
            l1 = int(np.abs(pa - pb).sum())
            assert l1 <= 2 * q * ed, (a, b, ed, l1)
            ta, tb = _thermometer(pa, levels), _thermometer(pb, levels)
            assert ta.sum() + tb.sum() - 2 * int(ta @ tb) == l1


def test_colex_order_is_id_order(orc):
    rng = np.random.default_rng(3)
    bound = colex_max_id(2)
    for top in (50, 5000, bound):
        verts = np.unique(rng.integers(max(0, top - 60), top + 1, size=40)).tolist()
        tuples = [(v,) for v in verts]
        tuples += [(a, b) for i, a in enumerate(verts) for b in verts[i + 1:]]
        tuples += [(a, b, c) for i, a in enumerate(verts) for j, b in enumerate(verts[i + 1:], i + 1)
                   for c in verts[j + 1:]]
        colex = sorted(tuples, key=lambda t: (len(t), t[::-1]))
        ids = [orc.simplex_id(list(t)) for t in colex]
        assert all(x < y for x, y in zip(ids, ids[1:])), top


def test_stats_struct_layout(tmp_path):
    """rnng_stats in include/rnng_gpu.h and rnng_gb300.Stats agree field by field."""
    import rnng_gb300
    fields = [f for f, _ in rnng_gb300.Stats._fields_]
    src = tmp_path / "layout.c"
    src.write_text('#include <stddef.h>\n#include <stdio.h>\n#include "rnng_gpu.h"\nint main(void) {\n'
                   + "".join(f'    printf("%zu\\n", offsetof(rnng_stats, {f}));\n' for f in fields)
                   + '    printf("%zu\\n", sizeof(rnng_stats));\n    return 0;\n}\n')
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    want = [getattr(rnng_gb300.Stats, f).offset for f in fields] + [ctypes.sizeof(rnng_gb300.Stats)]
    assert got == want
