"""Generates the golden fixtures in tests/golden/ by running RNNG's own CPU path.

RNNG ships no tests and no golden vectors, so the fixtures are made here: seeded
synthetic inputs (rnng_gb300.synth) are fed to RNNG's headers, compiled from the RNNG
source tree with the single-rank MPI shim (oracle/Makefile, target ``ref``), through
the binary-dump harness oracle/ref_harness.cpp, which makes the same API calls as
RNNG's drivers.  The expected outputs are stored with full float bits.

    make -C oracle ref            # needs the RNNG sources (RNNG_SRC=/path/to/RNNG)
    python tests/golden/make_golden.py [fixture names]   # default: all of them

Fixtures (npz, inputs + expected):
  k1_systolic   L2 mixture, 3000 x 8, radius 1.5, systolic path (cover tree + ring)
  k1_landmark   same input through the landmark path (Voronoi + ghosts + cell trees)
  k2_landmark   integer descriptors 0..255, 1200 x 128 (stored as uint8)
  k3_edit       DNA families, 300 strings, radius 8, landmark path with edit distance
  k4_rips       torus in R^16, 1200 points, maxdim 2, rips path
  k4_rips3      torus in R^16, 600 points, maxdim 3 (the rips driver's default)
  k3_rips_edit  DNA families, 96 strings, radius 8, maxdim 2, rips path with edit distance
  k5_landmark   Zipf Gaussian mixture, 2500 x 32
  k1_cells      the k1 input's Voronoi cells (30 landmarks) after coalescing, with the
                landmark driver's ghosts; k1_cells_rips with the rips driver's ghosts
                and interior flags
  k3_cells      the k3 strings' cells (30 landmarks) with the rips driver's ghosts
  dup_cells     400 points on 60 distinct positions in R^4, 40 landmarks: identical
                landmarks leave cells empty
  nan_systolic  L2 mixture, 2000 x 8, radius 3, with 45 rows holding NaN coordinates
                (40 with one, 5 all NaN), systolic path: such rows get no edges;
                nan_landmark the same input through the landmark path (20 landmarks)
  nan_rips      torus in R^16, 400 points, 12 of them with a NaN coordinate, maxdim 2,
                rips path: they stay vertices without edges
  (RNNG's cover tree does not survive infinite coordinates, so no fixture has them.)
Edge fixtures hold the unordered edge set (u < v) with weights, and the driver's
reported edge count (n + 2|E|); the Rips fixtures hold the merged filtration; the cell
fixtures hold per cell its id, point ids, distances to the centre, interior flags and
ghost ids, in RNNG's order.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from rnng_gb300 import synth  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")


ONLY = set(sys.argv[1:])


def wanted(name):
    return not ONLY or name in ONLY


def with_nan_rows(x, ones, whole, seed):
    """A copy of x with `ones` rows holding one NaN coordinate and `whole` rows all NaN."""
    rng = np.random.default_rng(seed)
    x = x.copy()
    rows = rng.choice(x.shape[0], size=ones + whole, replace=False)
    x[rows[:ones], rng.integers(0, x.shape[1], size=ones)] = np.nan
    x[rows[ones:]] = np.nan
    return x


def run(args):
    subprocess.run([HARNESS] + [str(a) for a in args], check=True)


def edges_fixture(name, tmp, mode, path_in, radius, extra, n, save_inputs):
    if not wanted(name):
        return
    out = os.path.join(tmp, name + ".bin")
    if mode == "systolic":
        run(["systolic", path_in, repr(float(radius)), out])
    else:
        run(["landmark", mode, path_in, repr(float(radius)), extra[0], extra[1], out])
    u, v, w = oracle.read_edge_dump(out)
    eu, ev, ew, full = oracle.reference_graph_semantics(u, v, w)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), radius=np.float32(radius), u=eu, v=ev, w=ew,
                        reported_edges=np.int64(full), n=np.int64(n), **save_inputs)
    print(f"{name}: n={n} |E|={eu.size} reported={full}")


def cells_fixture(name, tmp, metric, path_in, radius, m, seed, rips, save_inputs):
    if not wanted(name):
        return
    out = os.path.join(tmp, name + ".bin")
    run(["cells", metric, path_in, repr(float(radius)), m, seed, 1 if rips else 0, out])
    cells = oracle.read_cells_dump(out)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), radius=np.float32(radius), m=np.int64(m),
                        seed=np.int64(seed), rips=np.int64(1 if rips else 0), **cells, **save_inputs)
    empty = int((cells["npts"] == 0).sum())
    print(f"{name}: cells={cells['npts'].size} empty={empty} ghosts={cells['ghosts'].size}")


def rips_fixture(name, tmp, metric, path_in, radius, maxdim, m, seed, n, save_inputs):
    if not wanted(name):
        return
    out = os.path.join(tmp, name + ".bin")
    run(["rips", metric, path_in, repr(float(radius)), maxdim, m, seed, out])
    ids, vals = oracle.read_simplex_dump(out)
    mids, mvals = oracle.merge_filtration(ids, vals)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), radius=np.float32(radius), ids=mids, values=mvals,
                        maxdim=np.int64(maxdim), n=np.int64(n), **save_inputs)
    print(f"{name}: n={n} simplices={mids.size}")


def main():
    if not os.path.exists(HARNESS):
        raise SystemExit("build the reference harness first: make -C oracle ref")
    with tempfile.TemporaryDirectory() as tmp:
        # K1: systolic and landmark paths on the same input
        x1 = synth.l2_mixture(n=3000, d=8, k=16, seed=1)
        p1 = os.path.join(tmp, "k1.fvecs")
        synth.write_fvecs(p1, x1)
        edges_fixture("k1_systolic", tmp, "systolic", p1, np.float32(1.5), None, 3000, {"x": x1})
        edges_fixture("k1_landmark", tmp, "l2", p1, np.float32(1.5), ("30", "7"), 3000, {"x": x1})

        # K2-like: integer descriptors
        x2 = synth.descriptor(n=1200, d=128, k=12, seed=2)
        e2 = synth.choose_eps(x2, 20.0, sample=1200)
        p2 = os.path.join(tmp, "k2.fvecs")
        synth.write_fvecs(p2, x2)
        edges_fixture("k2_landmark", tmp, "l2", p2, e2, ("12", "7"), 1200, {"x_u8": x2.astype(np.uint8)})

        # K3-like: DNA families under edit distance
        seqs = synth.dna_families(n_seeds=30, mutants=10, seed=3)
        p3 = os.path.join(tmp, "k3.seqs")
        synth.write_seqs(p3, seqs)
        atoms, offsets = synth.pack_seqs(seqs)
        edges_fixture("k3_edit", tmp, "edit", p3, np.float32(8.0), ("30", "7"), len(seqs),
                      {"atoms": atoms, "offsets": offsets})

        # K5-like: Zipf Gaussian mixture in R^32
        x5 = synth.zipf_mixture(n=2500, d=32, k=48, seed=5)
        e5 = synth.choose_eps(x5, 20.0, sample=2500)
        p5 = os.path.join(tmp, "k5.fvecs")
        synth.write_fvecs(p5, x5)
        edges_fixture("k5_landmark", tmp, "l2", p5, e5, ("40", "7"), 2500, {"x": x5})

        # K4-like: Rips filtration up to triangles
        x4 = synth.torus16(n=1200, seed=4)
        e4 = synth.choose_eps(x4, 15.0, sample=1200)
        p4 = os.path.join(tmp, "k4.fvecs")
        synth.write_fvecs(p4, x4)
        rips_fixture("k4_rips", tmp, "l2", p4, e4, 2, 24, 7, 1200, {"x": x4})

        # K4-like at the rips driver's default dimension 3
        x43 = synth.torus16(n=600, seed=44)
        e43 = synth.choose_eps(x43, 12.0, sample=600)
        p43 = os.path.join(tmp, "k43.fvecs")
        synth.write_fvecs(p43, x43)
        rips_fixture("k4_rips3", tmp, "l2", p43, e43, 3, 12, 7, 600, {"x": x43})

        # Rips over edit distance
        seqs_r = synth.dna_families(n_seeds=12, mutants=8, seed=33)
        p3r = os.path.join(tmp, "k3r.seqs")
        synth.write_seqs(p3r, seqs_r)
        atoms_r, offsets_r = synth.pack_seqs(seqs_r)
        rips_fixture("k3_rips_edit", tmp, "edit", p3r, np.float32(8.0), 2, 10, 7, len(seqs_r),
                     {"atoms": atoms_r, "offsets": offsets_r})

        # Voronoi cells and ghosts
        cells_fixture("k1_cells", tmp, "l2", p1, np.float32(1.5), 30, 7, False, {"x": x1})
        cells_fixture("k1_cells_rips", tmp, "l2", p1, np.float32(1.5), 30, 7, True, {"x": x1})
        cells_fixture("k3_cells", tmp, "edit", p3, np.float32(8.0), 30, 7, True, {"atoms": atoms, "offsets": offsets})
        rng = np.random.default_rng(12)
        base = rng.normal(size=(60, 4)).astype(np.float32) * np.float32(2.0)
        xd = base[rng.integers(0, 60, size=400)]
        pd = os.path.join(tmp, "dup.fvecs")
        synth.write_fvecs(pd, xd)
        cells_fixture("dup_cells", tmp, "l2", pd, np.float32(3.0), 40, 11, True, {"x": xd})

        # rows with NaN coordinates
        xn = with_nan_rows(synth.l2_mixture(n=2000, d=8, k=16, seed=21), 40, 5, 21)
        pn = os.path.join(tmp, "nan.fvecs")
        synth.write_fvecs(pn, xn)
        edges_fixture("nan_systolic", tmp, "systolic", pn, np.float32(3.0), None, 2000, {"x": xn})
        edges_fixture("nan_landmark", tmp, "l2", pn, np.float32(3.0), ("20", "7"), 2000, {"x": xn})
        xt = synth.torus16(n=400, seed=22)
        er = synth.choose_eps(xt, 12.0, sample=400)
        xr = with_nan_rows(xt, 12, 0, 22)
        pr = os.path.join(tmp, "nanr.fvecs")
        synth.write_fvecs(pr, xr)
        rips_fixture("nan_rips", tmp, "l2", pr, er, 2, 10, 7, 400, {"x": xr})

if __name__ == "__main__":
    main()
