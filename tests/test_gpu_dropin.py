"""The drop-in headers (include/*.h) against RNNG's own outputs.

oracle/ref_harness.cpp makes the drivers' API calls (PointContainer, selection_sample,
VoronoiDiagram, coalesce_cells, the ghost steps, CoverTree searches, VoronoiComplex)
and dumps their results.  Compiled against RNNG's headers it made the golden fixtures;
here the same source is compiled against the drop-in headers and linked to
librnng_gpu.so, and every dump must equal the fixture bit for bit."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden, golden_points, graph_text

pytestmark = pytest.mark.gpu

HARNESS = os.path.join(ROOT, "oracle", "_build", "dropin_harness")


@pytest.fixture(scope="module")
def harness(ctx):
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "dropin"], check=True)
    return HARNESS


def run(harness, *args):
    r = subprocess.run([harness] + [str(a) for a in args], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, f"harness exited with {r.returncode}: {r.stderr[-2000:]}"


def write_input(tmp_path, g):
    from rnng_gb300 import synth
    if "atoms" in g:
        atoms, offsets = g["atoms"], g["offsets"]
        seqs = [atoms[offsets[i]:offsets[i + 1]].tobytes() for i in range(offsets.size - 1)]
        path = str(tmp_path / "in.seqs")
        synth.write_seqs(path, seqs)
        return "edit", path
    path = str(tmp_path / "in.fvecs")
    synth.write_fvecs(path, golden_points(g))
    return "l2", path


def assert_edges(orc, dump, g):
    u, v, w = orc.read_edge_dump(dump)
    eu, ev, ew, full = orc.reference_graph_semantics(u, v, w)
    assert np.array_equal(eu, g["u"]) and np.array_equal(ev, g["v"])
    assert np.array_equal(ew.view(np.uint32), g["w"].view(np.uint32))
    assert full == int(g["reported_edges"])


@pytest.mark.parametrize("name", ["k1_systolic", "nan_systolic"])
def test_systolic(harness, orc, tmp_path, name):
    g = golden(name)
    _, path = write_input(tmp_path, g)
    out = str(tmp_path / "out.bin")
    run(harness, "systolic", path, repr(float(g["radius"])), out)
    assert_edges(orc, out, g)


@pytest.mark.parametrize("name,m", [("k1_landmark", 30), ("k2_landmark", 12), ("k3_edit", 30), ("k5_landmark", 40),
                                    ("nan_landmark", 20)])
def test_landmark(harness, orc, tmp_path, name, m):
    g = golden(name)
    metric, path = write_input(tmp_path, g)
    out = str(tmp_path / "out.bin")
    run(harness, "landmark", metric, path, repr(float(g["radius"])), m, 7, out)
    assert_edges(orc, out, g)


@pytest.mark.parametrize("name", ["k1_cells", "k1_cells_rips", "k3_cells", "dup_cells"])
def test_cells_and_ghosts(harness, orc, tmp_path, name):
    g = golden(name)
    metric, path = write_input(tmp_path, g)
    out = str(tmp_path / "out.bin")
    run(harness, "cells", metric, path, repr(float(g["radius"])), int(g["m"]), int(g["seed"]), int(g["rips"]), out)
    got = orc.read_cells_dump(out)
    for k in got:
        assert np.array_equal(got[k], g[k]), k


@pytest.mark.parametrize("name,m", [("k4_rips", 24), ("k4_rips3", 12), ("k3_rips_edit", 10), ("nan_rips", 10)])
def test_rips(harness, orc, tmp_path, name, m):
    g = golden(name)
    metric, path = write_input(tmp_path, g)
    out = str(tmp_path / "out.bin")
    run(harness, "rips", metric, path, repr(float(g["radius"])), int(g["maxdim"]), m, 7, out)
    ids, vals = orc.merge_filtration(*orc.read_simplex_dump(out))
    assert np.array_equal(ids, g["ids"])
    assert np.array_equal(vals.view(np.uint32), g["values"].view(np.uint32))


@pytest.mark.parametrize("name,m", [("k1_landmark", 30), ("k2_landmark", 12), ("nan_landmark", 20)])
def test_landmark_graph_file(harness, tmp_path, name, m):
    """The landmark driver's whole path through the drop-in headers: the graph's
    redistribute_edges at one rank runs on the GPU (rnng_graph_finalize with
    RNNG_FINALIZE_AS_GIVEN) and the written file equals RNNG's own, byte for byte."""
    g = golden(name)
    metric, path = write_input(tmp_path, g)
    out = str(tmp_path / "out.mtx")
    run(harness, "graph", metric, path, repr(float(g["radius"])), m, 7, out)
    assert open(out).read() == graph_text(g, golden_points(g).shape[0])


def test_graph_finalize_as_given(ctx, orc):
    """rnng_graph_finalize with RNNG_FINALIZE_AS_GIVEN on edges as a driver collects them
    (both orientations, repeats, self-loops, any order) equals RNNG's redistribution."""
    import ctypes

    import rnng_gb300
    rng = np.random.default_rng(5)
    n = 3000
    u = rng.integers(0, n, 40000).astype(np.int64)
    v = rng.integers(0, n, 40000).astype(np.int64)
    w = rng.integers(0, 50, 40000).astype(np.float32) * np.float32(0.25)
    w[u == v] = 0.0
    # repeats and both orientations, as the per-cell queries record them
    u = np.concatenate([u, v, u[:500]])
    v2 = np.concatenate([v, u[:40000], v[:500]])
    w = np.concatenate([w, w, w[:500]])
    uu = np.concatenate([u, v2])
    vv = np.concatenate([v2, u])
    ww = np.concatenate([w, w]).view(np.uint32)
    o = np.lexsort((ww, vv, uu))
    uu, vv, ww = uu[o], vv[o], ww[o]
    keep = np.ones(uu.size, bool)
    keep[1:] = (uu[1:] != uu[:-1]) | (vv[1:] != vv[:-1]) | (ww[1:] != ww[:-1])
    ein = rnng_gb300.Edges(u.size, u.ctypes.data, v2.ctypes.data, w.ctypes.data, 0, 0)
    e = rnng_gb300.Edges()
    assert ctx.lib.rnng_graph_finalize(ctx.h, ctypes.byref(ein), n, 8, ctypes.byref(e)) == 0
    gu = rnng_gb300._host_copy(e.u, e.count, np.int64)
    gv = rnng_gb300._host_copy(e.v, e.count, np.int64)
    gw = rnng_gb300._host_copy(e.w, e.count, np.float32)
    assert np.array_equal(gu, uu[keep]) and np.array_equal(gv, vv[keep])
    assert np.array_equal(gw.view(np.uint32), ww[keep])
