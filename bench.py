"""Benchmark: epsilon-graph edges/s on 1,000,000 x 128 float32 integer descriptors.

One step = one call of the epsilon-graph hot path (rnng_eps_graph_l2) over the whole
point set: partition, tile covers and pruning, BF16 tensor-core Gram tiles with the
exact FP32 recheck, compaction to the final (u, v, w) edge list.  The reported value
is edges/s of the BF16 form with the points already resident in HBM; the plain FP32
form (same partition and pruning, every pair evaluated with the sequential FP32 L2)
is timed beside it, and both produce the identical edge set.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

With --impl reference RNNG's own algorithm for the path (its landmark pipeline,
restated in C under oracle/) is timed on the host cores on a prefix sample of the same
workload (see cpu_landmark_leg below).  Under torchrun (N > 1)
every rank runs an independent replica on its own GPU (the path is not sharded).
Prints one JSON line on rank 0.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "eps-graph edges/s, 1M×128 f32: BF16-TC+recheck vs plain FP32 GPU, same edges"
UNIT = "edges/s"
N_POINTS, DIM = 1_000_000, 128


def workload(n=N_POINTS):
    from rnng_gb300 import synth
    return synth.descriptor(n=n, d=DIM), synth.EPS_K2


def config(extra=None, n=N_POINTS):
    from rnng_gb300 import synth
    name = "k2-descriptors-1Mx128-f32" if n == N_POINTS else f"k2-descriptors-{n}x128-f32 (profiling size)"
    c = {"workload": name, "points": n, "dim": DIM,
         "radius": float(synth.EPS_K2), "radius_hex": hex(int(np.float32(synth.EPS_K2).view(np.uint32))),
         "clusters": 1000, "values": "integers 0..255 stored as float32",
         "l2_flush": "not needed: inputs (512 MB) larger than L2 (129 MB)"}
    if extra:
        c.update(extra)
    return c


# ----------------------------------------------------------------------------- clocks

class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 25 ms with nvidia-smi's own
    timestamps.  start() launches the sampler before the warm-up (nvidia-smi takes a
    while to print its first sample), begin() / end() mark the timed region on the host's
    clock, and stop() keeps the samples inside it."""
    FIELDS = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []
        self.thread = None
        self.t0 = self.t1 = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "25"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def begin(self):
        import datetime
        self.t0 = datetime.datetime.now()

    def end(self):
        import datetime
        self.t1 = datetime.datetime.now()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        import datetime
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.1)  # the samples of the region's last moments
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons, total = [], [], set(), 0
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                ts = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f")
                clk, cmax = float(parts[1]), float(parts[2])
            except ValueError:
                continue
            total += 1
            if self.t0 and self.t1 and not (self.t0 <= ts <= self.t1):
                continue
            sm.append(clk)
            smax.append(cmax)
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "samples_all": total, "interval_ms": 25}


# ----------------------------------------------------------------------------- CPU leg

LANDMARK_PREFIX = 100_000  # points of the CPU reference sample
POINTS_PER_CELL = 1_000    # RNNG's landmark run of the descriptor workload: 1,000 landmarks for 1M points


def cpu_landmark_leg(x, radius, prefix: int = LANDMARK_PREFIX, centres: int | None = None,
                     threads: int | None = None) -> dict:
    """Times RNNG's own algorithm on the host cores: its landmark pipeline (Voronoi cells,
    cover trees, ghost points, batched radius queries; restated in oracle/landmark.c and
    checked there against RNNG's driver) over the first `prefix` points, with one landmark
    per POINTS_PER_CELL points as RNNG's run of this workload uses.  Edges/s of the sample:
    RNNG's cost per edge grows with n (the Voronoi step alone is n x landmarks), so the
    sample's rate is an upper bound of its full-size rate."""
    import oracle
    oracle.build()
    full = oracle.num_threads()
    if threads:
        oracle.set_threads(threads)
    xs = np.ascontiguousarray(x[:prefix])
    m = centres or max(1, xs.shape[0] // POINTS_PER_CELL)
    t0 = time.perf_counter()
    (u, v, w), info = oracle.landmark_l2(xs, radius, num_centers=m)
    dt = time.perf_counter() - t0
    if threads:
        oracle.set_threads(full)
    return {"value": u.size / dt, "edges": int(u.size), "seconds": dt, "points": int(xs.shape[0]),
            "landmarks": m, "threads": info["threads"], "host_cores": os.cpu_count(),
            "phases_s": {k: round(info[k], 3) for k in oracle.LANDMARK_PHASES}}


K3_PREFIX = 8_000   # strings of the edit-distance CPU sample: 200 whole families of 40
K3_FAMILY = 40      # strings per family; RNNG's run of the workload: 5,000 landmarks for 200k strings


def cpu_edit_leg(seqs, radius, prefix: int = K3_PREFIX) -> dict:
    """RNNG's landmark pipeline under edit distance (its driver's `-D edit` path, restated in
    oracle/landmark.c) over the first `prefix` strings, with one landmark per family's worth
    of strings.  The strings come family by family, so the prefix keeps each string's
    relatives; RNNG's cost per edge grows with n (Voronoi is n x landmarks edit distances),
    so the sample's rate is an upper bound of its full-size rate."""
    import oracle
    from rnng_gb300 import synth
    oracle.build()
    atoms, offsets = synth.pack_seqs(seqs[:prefix])
    m = max(1, prefix // K3_FAMILY)
    t0 = time.perf_counter()
    (u, v, w), info = oracle.landmark_edit(atoms, offsets, radius, num_centers=m)
    dt = time.perf_counter() - t0
    return {"value": u.size / dt, "edges": int(u.size), "seconds": dt, "points": prefix, "landmarks": m,
            "threads": info["threads"], "host_cores": os.cpu_count(),
            "phases_s": {k: round(info[k], 3) for k in oracle.LANDMARK_PHASES}}


def cpu_rips_leg(x, radius, landmarks_per_500k: int = 1024) -> dict:
    """The Rips workload on the host: RNNG's landmark epsilon graph (oracle/landmark.c, its
    driver's 1,024 landmarks) over all points, then the filtration - every clique up to a
    triangle with its value, sorted by (value, id) as RNNG's merge does (oracle orc_rips,
    one thread).  Simplices/s of the whole job."""
    import oracle
    oracle.build()
    n = x.shape[0]
    m = max(1, n * landmarks_per_500k // 500_000)
    t0 = time.perf_counter()
    (u, v, w), info = oracle.landmark_l2(x, radius, num_centers=m)
    t1 = time.perf_counter()
    ids, _ = oracle.rips(n, u, v, w, 2)
    t2 = time.perf_counter()
    phases = {k: round(info[k], 3) for k in oracle.LANDMARK_PHASES}
    phases["filtration"] = round(t2 - t1, 3)
    return {"value": ids.size / (t2 - t0), "simplices": int(ids.size), "edges": int(u.size), "graph_s": t1 - t0,
            "rips_s": t2 - t1, "points": n, "landmarks": m, "threads": info["threads"],
            "host_cores": os.cpu_count(), "phases_s": phases}


def landmark_sample_text(leg: dict) -> str:
    return (f"RNNG's landmark pipeline (oracle/landmark.c) on the first {leg['points']} points, "
            f"{leg['landmarks']} landmarks, {leg['threads']} host threads of {leg['host_cores']} cores: "
            f"{leg['edges']} edges in {leg['seconds']:.2f} s")


def cpu_leg(x, radius, budget_s: float = 20.0, threads: int | None = None) -> dict:
    """Times the brute-force restatement on a bounded sample of the workload (a second,
    labelled CPU number beside RNNG's algorithm).

    The oracle evaluates the reference predicate (sequential FP32 L2 <= radius) for a
    strided sample of query rows against all points; the measured time per pair
    evaluation is scaled to the whole job (n (n-1) / 2 pair evaluations for the
    |E| edges the GPU found) to give edges/s.
    """
    import oracle
    oracle.build()
    if threads:
        oracle.set_threads(threads)
    cores = oracle.num_threads()
    n = x.shape[0]
    # calibrate the sample to about budget_s of work
    rows = 64
    t0 = time.perf_counter()
    oracle.cross_l2(x, x[:: n // rows][:rows], radius)
    t_cal = time.perf_counter() - t0
    rows = int(max(64, min(20000, rows * budget_s / max(t_cal, 1e-3))))
    idx = np.linspace(0, n - 1, rows).astype(np.int64)
    t0 = time.perf_counter()
    u, v, w = oracle.cross_l2(x, x[idx], radius)
    dt = time.perf_counter() - t0
    pair_time = dt / (rows * n)
    # every sampled row also matches itself (distance 0)
    mean_degree = (u.size - rows) / rows
    return {"pair_time_s": pair_time, "cores": cores, "rows": rows, "seconds": dt, "mean_degree": mean_degree}


def cpu_value(leg: dict, edges: int, n: int) -> float:
    return edges / (leg["pair_time_s"] * n * (n - 1) / 2)


def fp64_error(x, u, v, w, chunk: int = 1 << 19) -> float:
    """max |w - L2 in float64| over the emitted edges: how far the reference's FP32
    arithmetic (which the path reproduces bit for bit) is from the exact distance."""
    err = 0.0
    for s in range(0, u.size, chunk):
        a = x[u[s:s + chunk]].astype(np.float64)
        a -= x[v[s:s + chunk]]
        d64 = np.sqrt(np.einsum("ij,ij->i", a, a))
        err = max(err, float(np.max(np.abs(w[s:s + chunk].astype(np.float64) - d64))))
    return err


def peaks_bf16():
    """(burst, sustained, source) bf16 TFLOP/s from the measured peaks, else the fallback."""
    try:
        p = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(p["bf16_tflops"]), float(p["bf16_tflops_sustained"]), "of measured"
    except (OSError, KeyError, ValueError):
        return 1900.0, 1700.0, "of fallback"


def max_over_ranks(ms: float, dist, device) -> float:
    """The slowest rank's time: every replica does the full workload, the job's time is
    the maximum (dist is torch.distributed or None for one process)."""
    if dist is None:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(units_per_rank: int, world: int, steps: int, ms: float) -> float:
    """Whole-job throughput: the units all ranks processed over the slowest rank's time."""
    return world * units_per_rank * steps / (ms / 1e3)


# ----------------------------------------------------------------------------- main

def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--fp32-steps", type=int, default=2)
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--points", type=int, default=N_POINTS,
                    help="points of the descriptor workload (smaller sizes are for ncu captures only)")
    ap.add_argument("--k5-points", type=int, default=5_000_000,
                    help="points of the K5 workload (smaller sizes are for ncu captures only)")
    ap.add_argument("--workload", default="k2", choices=["k1", "k2", "k3", "k4", "k5", "k2-dropin"],
                    help="k2 (default) is the headline; k1, k3, k4, k5 print the same line for the other "
                         "configurations (see SECONDARY)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    if args.workload == "k2-dropin":
        if rank == 0:
            run_dropin(args)
        return
    if args.workload != "k2":
        run_secondary(args, world, rank, local)
        return

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")

    import rnng_gb300
    x, radius = workload(args.points)
    n, d = x.shape
    ctx = rnng_gb300.Context(local)
    xd = torch.from_numpy(x).to(f"cuda:{local}")
    stream = torch.cuda.ExternalStream(ctx.stream(), device=f"cuda:{local}")
    flags_dev = rnng_gb300.INPUT_DEVICE | rnng_gb300.OUTPUT_DEVICE

    def step(mode):
        e = ctx.eps_graph_l2_raw(xd.data_ptr(), None, n, d, radius, mode, flags_dev)
        return e.count

    # ---- BF16 tensor-core form: warm-up, then K timed steps on the library's stream
    clocks = ClockSampler(local)
    clocks.start()
    for _ in range(args.warmup):
        edges = step(1)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    gram_ms, launches, tile_pairs, cands = [], [], [], []
    torch.cuda.synchronize()
    clocks.begin()
    ev0.record(stream)
    for _ in range(args.steps):
        edges = step(1)
        st = ctx.stats()
        gram_ms.append(st["ms_gram"])
        launches.append(st["kernel_launches"])
        tile_pairs.append(st["tile_pairs"])
        cands.append(st["candidates"])
    ev1.record(stream)
    torch.cuda.synchronize()
    clocks.end()
    clk = clocks.stop()
    ms = max_over_ranks(ev0.elapsed_time(ev1), dist, f"cuda:{local}")
    ms_step = ms / args.steps
    value = job_value(edges, world, args.steps, ms)
    last = ctx.stats()

    # ---- plain FP32 form (same partition and pruning), a few steps
    fp32 = None
    if args.fp32_steps > 0:
        step(0)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.fp32_steps):
            edges32 = step(0)
        e1.record(stream)
        torch.cuda.synchronize()
        ms32 = e0.elapsed_time(e1) / args.fp32_steps
        assert edges32 == edges, "FP32 and BF16 forms found different edge counts"
        fp32 = {"value": edges / (ms32 / 1e3), "ms_per_step": ms32,
                "bf16_speedup": ms32 / ms_step}

    # ---- end to end through the C ABI with host buffers (pinned input, host result)
    xh = torch.from_numpy(x).pin_memory()
    ctx.eps_graph_l2_raw(xh.data_ptr(), None, n, d, radius, 1, 0)
    t_e2e = []
    for _ in range(max(1, args.e2e_steps)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e = ctx.eps_graph_l2_raw(xh.data_ptr(), None, n, d, radius, 1, 0)
        t_e2e.append(time.perf_counter() - t0)
        assert e.count == edges
    e2e_s = statistics.median(t_e2e)
    st_e2e = ctx.stats()  # the last end-to-end call's copy times (CUDA events on the library's stream)
    err64 = fp64_error(x, *ctx._edges_out(e)) if rank == 0 else None
    e2e = {"value": world * edges / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(n * d * 4),
           "d2h_bytes_per_step": int(edges * (8 + 8 + 4)), "ms_per_step": e2e_s * 1e3,
           "ms_h2d": round(st_e2e["ms_h2d"], 3), "ms_d2h": round(st_e2e["ms_d2h"], 3),
           "ms_device_total": round(st_e2e["ms_total"], 3)}

    # ---- roofline of the dominant kernel (tcgen05 Gram tiles)
    burst, sustained, src = peaks_bf16()
    pairs = last["pairs_evaluated"]
    g_ms = statistics.median(gram_ms)
    achieved = 2.0 * d * pairs / (g_ms / 1e3) / 1e12
    traffic = read_profile_traffic() if n == N_POINTS else None  # the committed capture is of the 1M workload
    roofline = {"bound": "tensor", "kernel": "k_gram_bf16", "achieved": achieved, "peak": burst, "unit": "TFLOP/s",
                "frac": achieved / burst, "peak_source": src + " (burst bf16: the kernel runs in ms-long launches)",
                "peak_sustained": sustained, "frac_sustained": achieved / sustained, "traffic": traffic,
                "flops_per_launch": 2.0 * d * pairs, "ms_per_launch": g_ms,
                "algorithmic": "2*d flops per evaluated point pair (x.y), pairs = surviving tile pairs * 128 * 128"}

    # ---- CPU baselines (rank 0 only): RNNG's algorithm on a prefix, and brute force
    cpu, brute = None, None
    if rank == 0 and not args.no_cpu:
        leg = cpu_landmark_leg(x, radius)
        cpu = {"value": leg["value"], "unit": UNIT, "cores": leg["threads"], "kind": "port",
               "algorithm": "RNNG landmark pipeline (Voronoi cells + cover trees + ghosts)",
               "sample": landmark_sample_text(leg), "phases_s": leg["phases_s"]}
        bl = cpu_leg(x, radius, budget_s=8.0)
        brute = {"value": cpu_value(bl, edges, n), "unit": UNIT, "cores": bl["cores"],
                 "sample": f"{bl['rows']} strided query rows x all {n} points with the oracle's reference "
                           f"predicate ({bl['seconds']:.1f} s), time per pair scaled to n(n-1)/2 pairs"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "bf16", "data": "synthetic (seeded numpy, see rnng_gb300/synth.py)",
                "config": config({"parallelism": "replicas" if world > 1 else "single-gpu",
                                  "edges": int(edges), "super_pairs": int(last["super_pairs"]),
                                  "tile_pairs": int(last["tile_pairs"]),
                                  "tile_pairs_all": int(last["tile_pairs_all"]),
                                  "candidates": int(last["candidates"]),
                                  "prune": {"tensor_cores": bool(last["prune_tensor"]),
                                            "widen": round(float(last["prune_widen"]), 4)},
                                  "stage_ms": {k: round(last[k], 3) for k in
                                               ("ms_partition", "ms_bounds", "ms_prune", "ms_tiles", "ms_recheck",
                                                "ms_finalize")},
                                  "gram": {k: int(last[k]) for k in ("gram_nt", "gram_chunk", "gram_slots")}}, n),
                "fp32_direct": fp32, "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu,
                "cpu_bruteforce": brute,
                "max_abs_err_fp64": err64, "gpu_launches": int(sum(launches)), "clocks": clk}
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    ctx.close()


# ----------------------------------------------------------------------------- other configurations

SECONDARY = {
    "k1": {"metric": "eps-graph edges/s, 20k x 8 f32 Gaussian mixture, eps 1.5", "unit": "edges/s"},
    "k3": {"metric": "eps-graph edges/s, 200k DNA strings, edit distance, eps 8", "unit": "edges/s"},
    "k4": {"metric": "Rips filtration simplices/s (<= 2-simplices), 500k torus points in R^16", "unit": "simplices/s"},
    "k5": {"metric": "eps-graph edges/s, 5M x 32 f32 Zipf Gaussian mixture", "unit": "edges/s"},
}


def run_secondary(args, world, rank, local):
    """K1, K3, K4, K5: one call of the path per step on device-resident input (value) and
    from host buffers (e2e), timed like the headline line."""
    import torch
    import rnng_gb300
    from rnng_gb300 import synth
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    ctx = rnng_gb300.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=f"cuda:{local}")
    dev = f"cuda:{local}"
    flags_dev = rnng_gb300.INPUT_DEVICE | rnng_gb300.OUTPUT_DEVICE
    wl = args.workload
    cfg = {}
    if wl in ("k1", "k5"):
        x = synth.l2_mixture() if wl == "k1" else synth.zipf_mixture(n=args.k5_points)
        radius = synth.EPS_K1 if wl == "k1" else synth.EPS_K5
        n, d = x.shape
        xd = torch.from_numpy(x).to(dev)
        xh = torch.from_numpy(x).pin_memory()
        cfg = {"workload": {"k1": "k1-gaussian-mixture-20kx8-f32", "k5": "k5-zipf-mixture-5Mx32-f32"}[wl],
               "points": n, "dim": d, "radius": float(radius)}
        step = lambda mode=1: ctx.eps_graph_l2_raw(xd.data_ptr(), None, n, d, radius, mode, flags_dev).count
        step_host_e = lambda: ctx.eps_graph_l2_raw(xh.data_ptr(), None, n, d, radius, 1, 0)
        step_host = lambda: step_host_e().count
        err_edges = lambda: ctx._edges_out(step_host_e())
        h2d = n * d * 4
        d2h_per_unit = 8 + 8 + 4
    elif wl == "k3":
        seqs = synth.dna_families()
        atoms, offsets = synth.pack_seqs(seqs)
        radius = synth.EPS_K3
        n = offsets.size - 1
        ad, od = torch.from_numpy(atoms).to(dev), torch.from_numpy(offsets).to(dev)
        ah, oh = torch.from_numpy(atoms).pin_memory(), torch.from_numpy(offsets).pin_memory()
        cfg = {"workload": "k3-dna-families-200k-edit", "strings": n, "atoms": int(atoms.size),
               "radius": float(radius)}
        step = lambda mode=1: ctx.eps_graph_edit_raw(ad.data_ptr(), od.data_ptr(), n, radius, flags_dev).count
        step_host = lambda: ctx.eps_graph_edit_raw(ah.data_ptr(), oh.data_ptr(), n, radius, 0).count
        err_edges = None  # integer Levenshtein distances: exact
        h2d = int(atoms.size + offsets.size * 8)
        d2h_per_unit = 8 + 8 + 4
    else:  # k4
        x = synth.torus16()
        radius = synth.EPS_K4
        n, d = x.shape
        xd = torch.from_numpy(x).to(dev)
        xh = torch.from_numpy(x).pin_memory()
        cfg = {"workload": "k4-torus16-500k-rips-maxdim2", "points": n, "dim": d, "radius": float(radius),
               "maxdim": 2}
        step = lambda mode=1: ctx.rips_l2_raw(xd.data_ptr(), n, d, radius, 2, mode, flags_dev).count
        step_host = lambda: ctx.rips_l2_raw(xh.data_ptr(), n, d, radius, 2, 1, 0).count
        # every filtration value is the value of one of the graph's edges (a max over edges)
        err_edges = lambda: ctx._edges_out(ctx.eps_graph_l2_raw(xh.data_ptr(), None, n, d, radius, 1, 0))
        h2d = n * d * 4
        d2h_per_unit = 8 + 4
    clocks = ClockSampler(local)
    clocks.start()
    for _ in range(args.warmup):
        units = step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches, stats = [], []
    torch.cuda.synchronize()
    clocks.begin()
    ev0.record(stream)
    for _ in range(args.steps):
        units = step()
        st = ctx.stats()
        launches.append(st["kernel_launches"])
        stats.append(st)
    ev1.record(stream)
    torch.cuda.synchronize()
    clocks.end()
    clk = clocks.stop()
    ms = max_over_ranks(ev0.elapsed_time(ev1), dist, dev)
    value = job_value(units, world, args.steps, ms)
    last = stats[-1]
    fp32 = None
    if wl in ("k1", "k5", "k4") and args.fp32_steps > 0:
        step(0)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.fp32_steps):
            u32 = step(0)
        e1.record(stream)
        torch.cuda.synchronize()
        ms32 = e0.elapsed_time(e1) / args.fp32_steps
        assert u32 == units, "FP32 and BF16 forms differ"
        fp32 = {"value": units / (ms32 / 1e3), "ms_per_step": ms32, "bf16_speedup": ms32 / (ms / args.steps)}
    step_host()
    t_e2e = []
    for _ in range(max(1, args.e2e_steps)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        u = step_host()
        t_e2e.append(time.perf_counter() - t0)
        assert u == units
    e2e_s = statistics.median(t_e2e)
    err64 = None
    if rank == 0:
        err64 = 0.0 if err_edges is None else fp64_error(x, *err_edges())
    cpu = None
    if rank == 0 and not args.no_cpu and wl in ("k1", "k5"):
        # k1: RNNG's systolic run is one cover tree over all points (one cell); k5: a prefix
        # with RNNG's 1,024 landmarks per 5M points
        leg = (cpu_landmark_leg(x, radius, prefix=n, centres=1) if wl == "k1"
               else cpu_landmark_leg(x, radius, prefix=LANDMARK_PREFIX,
                                     centres=max(1, LANDMARK_PREFIX * 1024 // 5_000_000)))
        cpu = {"value": leg["value"], "unit": SECONDARY[wl]["unit"],
               "cores": 1 if wl == "k1" else leg["threads"],  # one cell: one thread does the work
               "kind": "port",
               "algorithm": "RNNG cover-tree search" + (" (one cell: systolic)" if wl == "k1" else
                                                        " with landmark cells and ghosts"),
               "sample": landmark_sample_text(leg), "phases_s": leg["phases_s"]}
    if rank == 0 and not args.no_cpu and wl == "k3":
        leg = cpu_edit_leg(seqs, radius)
        cpu = {"value": leg["value"], "unit": SECONDARY[wl]["unit"], "cores": leg["threads"], "kind": "port",
               "algorithm": "RNNG cover-tree search under edit distance with landmark cells and ghosts",
               "sample": (f"RNNG's landmark pipeline under edit distance (oracle/landmark.c) on the first "
                          f"{leg['points']} strings ({leg['points'] // K3_FAMILY} whole families), {leg['landmarks']} "
                          f"landmarks (one per {K3_FAMILY} strings, as RNNG's run of this workload), "
                          f"{leg['threads']} host threads of {leg['host_cores']} cores: {leg['edges']} edges in "
                          f"{leg['seconds']:.2f} s"),
               "phases_s": leg["phases_s"]}
    if rank == 0 and not args.no_cpu and wl == "k4":
        leg = cpu_rips_leg(x, radius)
        cpu = {"value": leg["value"], "unit": SECONDARY[wl]["unit"], "cores": leg["threads"], "kind": "port",
               "algorithm": "RNNG landmark epsilon graph, then clique enumeration and (value, id) order",
               "sample": (f"the whole workload ({leg['points']} points): RNNG's landmark pipeline (oracle/landmark.c, "
                          f"{leg['landmarks']} landmarks, {leg['threads']} host threads of {leg['host_cores']} cores) "
                          f"{leg['edges']} edges in {leg['graph_s']:.2f} s, then the filtration of cliques up to "
                          f"triangles sorted by (value, id) (oracle orc_rips, one thread) in {leg['rips_s']:.2f} s: "
                          f"{leg['simplices']} simplices"),
               "phases_s": leg["phases_s"]}
        assert leg["simplices"] == units, (leg["simplices"], units)
    roofline = None
    if wl == "k3" and last["ms_gram"] > 0:
        # the filter: a Gram form over 512-byte E4M3 rows (thermometer-coded q-gram profiles)
        peak = 2 * 1900.0
        src = "2 x fallback bf16 (FP8 dense rate is twice BF16's)"
        try:
            peak = 2.0 * float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["bf16_tflops_sustained"])
            src = "2 x measured sustained bf16 (FP8 dense rate is twice BF16's)"
        except (OSError, KeyError, ValueError):
            pass
        flops = 2.0 * 512 * last["pairs_evaluated"]
        achieved = flops / (statistics.median(s["ms_gram"] for s in stats) / 1e3) / 1e12
        roofline = {"bound": "tensor", "kernel": "k_gram_bf16 (FP8 filter)", "achieved": achieved, "peak": peak,
                    "unit": "TFLOP/s", "frac": achieved / peak, "peak_source": src, "traffic": None,
                    "algorithmic": "2*512 ops per evaluated string pair (512 E4M3 profile bytes per string)"}
    if wl in ("k1", "k5") and last["ms_gram"] > 0:
        burst, sustained, src = peaks_bf16()
        # a K5 step is a third of a second of Gram work: the sustained peak applies
        peak, src = (sustained, src + " (sustained bf16)") if wl == "k5" else (burst, src + " (burst bf16)")
        dp = -(-d // 64) * 64
        ms_gram = statistics.median(s["ms_gram"] for s in stats)
        achieved = 2.0 * d * last["pairs_evaluated"] / (ms_gram / 1e3) / 1e12
        # the tensor cores multiply the padded width: dp - d columns are zeros or the folded column terms
        issued = 2.0 * dp * last["pairs_evaluated"] / (ms_gram / 1e3) / 1e12
        roofline = {"bound": "tensor", "kernel": "k_gram_bf16", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                    "frac": achieved / peak, "peak_source": src, "frac_burst": achieved / burst,
                    "frac_sustained": achieved / sustained, "traffic": None,
                    "algorithmic": "2*d flops per evaluated pair",
                    "mma_issued": {"achieved": issued, "frac": issued / peak,
                                   "counted": f"2*dp flops per evaluated pair (dp = {dp}, d padded to 64)"}}
    if rank == 0:
        cfg.update({"units": int(units), "parallelism": "replicas" if world > 1 else "single-gpu",
                    "stage_ms": {k: round(last[k], 3) for k in ("ms_partition", "ms_bounds", "ms_prune", "ms_tiles",
                                                                "ms_recheck", "ms_finalize", "ms_total")},
                    "super_pairs": int(last["super_pairs"]), "tile_pairs": int(last["tile_pairs"]),
                    "candidates": int(last["candidates"]),
                    "prune": {"tensor_cores": bool(last["prune_tensor"]), "widen": round(float(last["prune_widen"]), 4)}})
        line = {"metric": SECONDARY[wl]["metric"], "value": value, "unit": SECONDARY[wl]["unit"], "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "u8" if wl == "k3" else "bf16",
                "data": "synthetic (seeded numpy, see rnng_gb300/synth.py)", "config": cfg, "fp32_direct": fp32,
                "e2e": {"value": world * units / e2e_s, "unit": SECONDARY[wl]["unit"], "h2d_bytes_per_step": int(h2d),
                        "d2h_bytes_per_step": int(units * d2h_per_unit), "ms_per_step": e2e_s * 1e3},
                "roofline": roofline, "cpu_baseline": cpu, "max_abs_err_fp64": err64,
                "gpu_launches": int(sum(launches)), "clocks": clk}
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    ctx.close()


def run_dropin(args):
    """The headline workload through RNNG's own API: the landmark driver's calls (read_fvecs,
    selection_sample, VoronoiDiagram, coalesce_cells, add_ghost_points_systolic, per-cell
    CoverTree queries, Graph + redistribute_edges, write_file) compiled against the drop-in
    headers (oracle/ref_harness.cpp, graph mode; 1,000 landmarks as RNNG's run of this
    workload uses).  One run after a warm-up run; phase times from the harness."""
    import re
    import tempfile
    import rnng_gb300
    from rnng_gb300 import synth
    rnng_gb300.build.build()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "dropin"], check=True)
    harness = os.path.join(ROOT, "oracle", "_build", "dropin_harness")
    x, radius = workload(args.points)
    n = x.shape[0]
    with tempfile.TemporaryDirectory() as tmp:
        inp, out = os.path.join(tmp, "k2.fvecs"), os.path.join(tmp, "k2.mtx")
        synth.write_fvecs(inp, x)
        cmd = [harness, "graph", "l2", inp, repr(float(radius)), str(max(1, n // 1000)), "7", out]
        runs = []
        for _ in range(2):
            t0 = time.perf_counter()
            r = subprocess.run(cmd, capture_output=True, text=True, check=True)
            runs.append((time.perf_counter() - t0, r.stderr))
        wall, err = runs[-1]
        phases = {m.group(2): float(m.group(1)) for m in re.finditer(r"\[phase ([\d.]+)\] (.+)", err)}
        reported = int(re.search(r"edges=(\d+)", err).group(1))
    edges = (reported - n) // 2
    pipeline = sum(v for k, v in phases.items() if k not in ("read input", "wrote edges"))
    line = {"metric": "eps-graph edges/s through RNNG's API (landmark driver calls, drop-in headers), 1M x 128",
            "value": edges / pipeline, "unit": UNIT, "n_gpus": 1, "steps": 1, "warmup": 1,
            "ms_per_step": pipeline * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16", "data": "synthetic (seeded numpy, see rnng_gb300/synth.py)",
            "config": config({"path": "drop-in headers, oracle/ref_harness.cpp graph mode", "landmarks": n // 1000,
                              "edges": edges, "reported_edges": reported,
                              "phases_s": {k: round(v, 4) for k, v in phases.items()}}, n),
            "e2e": {"value": edges / wall, "unit": UNIT, "h2d_bytes_per_step": int(n * DIM * 4),
                    "d2h_bytes_per_step": int(reported * 20), "seconds": wall,
                    "note": "whole process: reads the .fvecs file, writes the text graph"}}
    print(json.dumps(line), flush=True)


def read_profile_traffic():
    """DRAM bytes per launch of k_gram_bf16 from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "k_gram_bf16__k2_1Mx128.md")
    try:
        for ln in open(p):
            if ln.startswith("dram_bytes_per_launch:"):
                return float(ln.split(":")[1].split()[0])
    except OSError:
        pass
    return None


def run_reference(args, world, rank):
    """Reference arm: RNNG's own algorithm for this path (its landmark pipeline, restated
    in oracle/landmark.c) on all host cores, each step one run over a prefix sample of
    the same workload (RNNG's C++ cannot be built on the GPU machine: its sources are not
    there)."""
    if rank != 0:
        return
    if args.workload != "k2":
        print(json.dumps({"impl": "reference", "unavailable": "the reference arm times the headline (k2) only"}))
        return
    x, radius = workload(args.points)
    n = x.shape[0]
    vals, leg = [], None
    for i in range(args.warmup + args.steps):
        leg = cpu_landmark_leg(x, radius)
        if i >= args.warmup:
            vals.append(leg["value"])
    value = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": leg["seconds"] * 1e3,
            "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded numpy, see rnng_gb300/synth.py)",
            "config": config(n=n), "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                                        "d2h_bytes_per_step": 0},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": leg["threads"], "kind": "port",
                             "algorithm": "RNNG landmark pipeline (Voronoi cells + cover trees + ghosts)",
                             "sample": landmark_sample_text(leg) + " per step"}}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
