"""Autotuner of the tensor-core Gram kernel.

Sweeps the kernel's three knobs on the benchmark configurations - the item form (nt: one
row tile with one 128-column tile, or with two for N = 256 MMAs, or 3: two row tiles
sharing one column tile), items per work-queue chunk, and B operand slots per CTA - and
writes the fastest setting per (operand kind, padded width,
tile-pair count) to rnng_gb300/gram_tuning.json.  The library reads that table when a
context is created (rnng_ctx_set_gram_tuning overrides it per context).

    python -m rnng_gb300.tune [--out PATH] [--repeat R] [--only k2,k5,...]

Each setting is timed as the Gram kernel's device time (rnng_stats.ms_gram, CUDA events
around its launch) of full epsilon-graph calls on device-resident inputs, median of R
calls after one warm-up call; the edge count is checked against the default setting's.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if os.path.dirname(HERE) not in sys.path:
    sys.path.insert(0, os.path.dirname(HERE))

CHUNKS = (8, 16, 32, 64, 128, 256)
SLOTS = (2, 3, 4, 0)  # 0: as many as fit in shared memory


def workloads(only):
    from rnng_gb300 import synth
    w = {
        "k2": ("bf16", "1M x 128 integer descriptors", lambda: (synth.descriptor(), synth.EPS_K2)),
        "k5": ("bf16", "5M x 32 Zipf mixture", lambda: (synth.zipf_mixture(), synth.EPS_K5)),
        "k4": ("bf16", "500k torus points in R^16", lambda: (synth.torus16(), synth.EPS_K4)),
        "k3": ("f8", "200k DNA strings, edit distance 8", lambda: (synth.pack_seqs(synth.dna_families()), synth.EPS_K3)),
    }
    return {k: v for k, v in w.items() if not only or k in only}


def main():
    import torch

    import rnng_gb300

    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "gram_tuning.json"))
    ap.add_argument("--repeat", type=int, default=3)
    ap.add_argument("--only", default="")
    args = ap.parse_args()
    only = [s for s in args.only.split(",") if s]
    ctx = rnng_gb300.Context(0)
    flags = rnng_gb300.INPUT_DEVICE | rnng_gb300.OUTPUT_DEVICE
    rows, report = [], []
    for name, (kind, desc, make) in workloads(only).items():
        data, radius = make()
        if kind == "bf16":
            x = torch.from_numpy(data).cuda()
            n, d = data.shape
            dp = -(-d // 64) * 64
            call = lambda: ctx.eps_graph_l2_raw(x.data_ptr(), None, n, d, radius, 1, flags).count
        else:
            atoms, offsets = data
            a, o = torch.from_numpy(atoms).cuda(), torch.from_numpy(offsets).cuda()
            n = offsets.size - 1
            dp = 512
            call = lambda: ctx.eps_graph_edit_raw(a.data_ptr(), o.data_ptr(), n, radius, flags).count

        def timed(nt, chunk, slots):
            ctx.set_gram_tuning(nt, chunk, slots)
            want = call()
            ms = []
            for _ in range(args.repeat):
                got = call()
                st = ctx.stats()
                assert got == want, (got, want)
                ms.append(st["ms_gram"])
            return statistics.median(ms), want, st

        base_ms, edges, st = timed(0, 0, 0)
        pairs = int(st["tile_pairs"])
        nts = (1, 2, 3) if kind == "bf16" and dp <= 128 else (1,)
        results = []
        t0 = time.time()
        for nt in nts:
            for chunk in CHUNKS:
                for slots in SLOTS:
                    ms, got, st = timed(nt, chunk, slots)
                    assert got == edges, (name, nt, chunk, slots, got, edges)
                    results.append({"nt": nt, "chunk": chunk, "slots": int(st["gram_slots"]), "ms": round(ms, 4)})
        # distinct effective settings only (slots 0 and an explicit maximum coincide)
        uniq = {}
        for r in results:
            key = (r["nt"], r["chunk"], r["slots"])
            if key not in uniq or r["ms"] < uniq[key]["ms"]:
                uniq[key] = r
        best = min(uniq.values(), key=lambda r: r["ms"])
        rows.append({"kind": kind, "dp": dp, "pairs": pairs, "nt": best["nt"], "chunk": best["chunk"],
                     "slots": best["slots"], "ms": best["ms"], "ms_untuned_default": round(base_ms, 4),
                     "workload": f"{name}: {desc}"})
        report.append({"workload": name, "sweep": sorted(uniq.values(), key=lambda r: r["ms"]),
                       "seconds": round(time.time() - t0, 1)})
        print(f"{name}: best {best} default {base_ms:.3f} ms ({pairs} tile pairs)", flush=True)
    ctx.set_gram_tuning(0, 0, 0)
    ctx.close()
    # rows of one (kind, dp): each applies from the midpoint (geometric) below its pair count
    rows.sort(key=lambda r: (r["kind"], r["dp"], r["pairs"]))
    prev = {}
    for r in rows:
        key = (r["kind"], r["dp"])
        r["min_pairs"] = 0 if key not in prev else int(np.sqrt(prev[key] * r["pairs"]))
        prev[key] = r["pairs"]
    table = {"about": "Gram kernel tuning: fastest (nt, chunk, slots) per operand kind, padded width dp and tile "
                      "pairs (a row applies from min_pairs on), measured by rnng_gb300/tune.py; ms = Gram kernel "
                      "device time per call",
             "rows": [{k: r[k] for k in ("kind", "dp", "min_pairs", "nt", "chunk", "slots", "ms", "ms_untuned_default",
                                         "pairs", "workload")} for r in rows]}
    with open(args.out, "w") as f:
        json.dump(table, f, indent=1)
    with open(os.path.splitext(args.out)[0] + "_sweep.json", "w") as f:
        json.dump(report, f, indent=1)
    print("wrote", args.out)


if __name__ == "__main__":
    main()
