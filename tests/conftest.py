import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (Blackwell, sm_103a build)")


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def ctx():
    import rnng_gb300
    rnng_gb300.build.build()
    c = rnng_gb300.Context(0)
    yield c
    c.close()


def golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def golden_points(g):
    if "x" in g:
        return g["x"]
    return g["x_u8"].astype(np.float32)


def colex_max_id(maxdim: int = 2) -> int:
    """Largest vertex id for which every simplex id up to maxdim is an exact binomial sum
    below the dimension bits (RNNG's Binom: a 64-bit falling product, signed division);
    up to it the library generates simplices in id order."""
    from math import comb, perm

    def exact(m):
        return all(perm(m, k) < 2 ** 63 and comb(m + 1, k) <= 2 ** 60 for k in range(1, maxdim + 2))
    lo, hi = 0, 1 << 40
    while lo < hi:
        mid = (lo + hi + 1) // 2
        lo, hi = (mid, hi) if exact(mid) else (lo, mid - 1)
    return lo


def graph_text(g, n):
    """The text RNNG's landmark driver writes for a fixture's graph (Graph::write_file after
    redistribute_edges at one rank, include/graph.hpp:20-116): both orientations of every
    edge plus the self-loop of every row with finite coordinates, sorted by (u, v, w), as
    "u v w" with six significant digits."""
    u, v, w = g["u"], g["v"], g["w"]
    x = golden_points(g)
    fin = np.isfinite(x).all(axis=1)
    selfs = np.nonzero(fin)[0]
    uu = np.concatenate([u, v, selfs])
    vv = np.concatenate([v, u, selfs])
    ww = np.concatenate([w, w, np.zeros(selfs.size, np.float32)])
    o = np.lexsort((ww.view(np.uint32), vv, uu))
    lines = ["%% %d %d %d" % (n, n, uu.size)] + ["%d %d %g" % (a, b, float(c)) for a, b, c in zip(uu[o], vv[o], ww[o])]
    return "\n".join(lines) + "\n"
