"""Generates the golden fixtures in tests/golden/ by running RNNG's own CPU path.

RNNG ships no tests and no golden vectors, so the fixtures are made here: seeded
synthetic inputs (rnng_gb300.synth) are fed to RNNG's headers, compiled from the RNNG
source tree with the single-rank MPI shim (oracle/Makefile, target ``ref``), through
the binary-dump harness oracle/ref_harness.cpp, which makes the same API calls as
RNNG's drivers.  The expected outputs are stored with full float bits.

    make -C oracle ref            # needs the RNNG sources (REF=/path/to/RNNG)
    python tests/golden/make_golden.py

Fixtures (npz, inputs + expected):
  k1_systolic   L2 mixture, 3000 x 8, radius 1.5, systolic path (cover tree + ring)
  k1_landmark   same input through the landmark path (Voronoi + ghosts + cell trees)
  k2_landmark   integer descriptors 0..255, 1200 x 128 (stored as uint8)
  k3_edit       DNA families, 300 strings, radius 8, landmark path with edit distance
  k4_rips       torus in R^16, 1200 points, maxdim 2, rips path
  k5_landmark   Zipf Gaussian mixture, 2500 x 32
Edge fixtures hold the unordered edge set (u < v) with weights, and the driver's
reported edge count (n + 2|E|); the Rips fixture holds the merged filtration.
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


def run(args):
    subprocess.run([HARNESS] + [str(a) for a in args], check=True)


def edges_fixture(name, tmp, mode, path_in, radius, extra, n, save_inputs):
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
        out = os.path.join(tmp, "k4.bin")
        run(["rips", p4, repr(float(e4)), 2, 24, 7, out])
        ids, vals = oracle.read_simplex_dump(out)
        mids, mvals = oracle.merge_filtration(ids, vals)
        np.savez_compressed(os.path.join(HERE, "k4_rips.npz"), radius=np.float32(e4), x=x4, ids=mids, values=mvals,
                            maxdim=np.int64(2), n=np.int64(1200))
        print(f"k4_rips: n=1200 simplices={mids.size}")


if __name__ == "__main__":
    main()
