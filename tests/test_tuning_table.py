"""The committed Gram tuning table (rnng_gb300/gram_tuning.json, read by the library at
context creation) is what its sweep (gram_tuning_sweep.json, written by the same run of
rnng_gb300/tune.py) found: every row is the fastest measured setting of its workload, rows
of one (kind, dp) apply from the geometric midpoint of neighbouring pair counts, and every
setting is one the kernel compiles (two or three column tiles only for BF16 operands of
at most two K-chunks)."""
import json
import math
import os

from conftest import ROOT

HERE = os.path.join(ROOT, "rnng_gb300")


def _load():
    with open(os.path.join(HERE, "gram_tuning.json")) as f:
        table = json.load(f)["rows"]
    with open(os.path.join(HERE, "gram_tuning_sweep.json")) as f:
        sweep = {s["workload"]: s["sweep"] for s in json.load(f)}
    return table, sweep


def test_rows_are_the_fastest_measured_settings():
    table, sweep = _load()
    assert table and len(table) == len(sweep)
    for r in table:
        name = r["workload"].split(":")[0]
        best = min(sweep[name], key=lambda s: s["ms"])
        assert (r["nt"], r["chunk"], r["slots"], r["ms"]) == (best["nt"], best["chunk"], best["slots"], best["ms"]), name
        assert r["ms"] <= r["ms_untuned_default"] * 1.01  # the tuned setting is not slower than the default


def test_rows_apply_from_midpoints_and_compile():
    table, _ = _load()
    groups = {}
    for r in table:
        assert r["kind"] in ("bf16", "f8") and r["dp"] % 64 == 0
        assert r["nt"] in (1, 2, 3) and r["chunk"] >= 1 and (r["slots"] == 0 or r["slots"] >= 2)
        if r["nt"] > 1:
            assert r["kind"] == "bf16" and r["dp"] <= 128
        groups.setdefault((r["kind"], r["dp"]), []).append(r)
    for rows in groups.values():
        rows.sort(key=lambda r: r["pairs"])
        assert rows[0]["min_pairs"] == 0
        for a, b in zip(rows, rows[1:]):
            assert b["min_pairs"] == int(math.sqrt(a["pairs"] * b["pairs"]))
