#!/usr/bin/env python3
"""Benchmark of the connected-components solve on GB300.

Headline workload (one step = one CC solve): the random hyperbolic graph of
n = 2^26 vertices, expected average degree 16, degree exponent gamma = 2.6
(threshold model, input seed 1; about 1.095e9 directed CSR entries, uint32
ids), solved by the exp_contraction option
(ExponentialContraction::FindComponents, app/exp_contraction.cpp:104-105)
with the reference's default Config (beta 0.1, seq 1, algorithm seed
1001 = seed + 0 + 1000), one rank.  It is the largest configuration that fits
one GPU (-gen rhg -n 26 -d 16 -gamma 2.6).

  value     Gedges/s = directed CSR entries / device time of the solve, input
            resident in HBM (CUDA events on the library's stream)
  e2e       the same metric through the C ABI with pinned HOST buffers: the
            host->device copy of the CSR and the device->host copy of the
            labels are inside the timed region
  roofline  the dominant kernel's algorithmic bytes per launch / its average
            CUDA-event duration, against the measured HBM copy bandwidth
  cpu_baseline  the CPU restatement of ExponentialContraction (oracle/) with
            one rank per host core, on a bounded sample of the same graph (the
            subgraph induced by its first quarter of the vertices)

Inputs (4.9 GB CSR + 0.27 GB labels) are larger than the 129 MB L2, so no
flush is needed between steps.

--workload grid prints the same line for the 8192 x 8192 bond-percolation
grid (p = 0.5, uint32 ids); --workload gnm | rhg-options | batch | serve
print the other configurations' lines.

--impl reference times the CPU restatement of the reference algorithm
(oracle/, one rank per host core) on the same bounded sample of the same
graph, built by the oracle's own input path (no GPU library is loaded), and
prints the same JSON line with "impl": "reference".

Multi-GPU (torchrun, N ranks): every rank solves its own replica (a single
graph does not shard on this path: replicas only); value = N x E / max-over-
ranks time.
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

INPUT_SEED = 1
ALGO_SEED = 1001
BETA, SEQ = 0.1, 1
RHG_LOG2N, RHG_DEG, RHG_GAMMA = 26, 16.0, 2.6
GRID_SIDE, GRID_P = 8192, 0.5
UNIT = "Gedges/s"
FALLBACK_HBM = 6800.0
L2_BYTES = 129 * 1024 * 1024


# ---- the two single-graph workloads -------------------------------------------
class NoGC:
    """Python's cyclic garbage collector paused over a timed region (after one
    full collection), as timeit does: a full collection with torch loaded takes
    about 25 ms, which would land in whichever timed step it fell into."""

    def __enter__(self):
        gc.collect()
        self.was = gc.isenabled()
        gc.disable()
        return self

    def __exit__(self, *a):
        if self.was:
            gc.enable()


class Workload:
    """One graph family at one size: how each arm builds it and how the JSON
    line names it.  Both arms build the same graph bit for bit (the same
    generator code; the reference arm's copy is linked into the oracle)."""

    def __init__(self, name: str, args):
        self.name = name
        if name == "rhg":
            k = args.rhg_log2n
            self.n = 1 << k
            self.desc = (f"random hyperbolic graph n=2^{k}, avg degree {RHG_DEG:g}, gamma {RHG_GAMMA} "
                         f"(threshold model, seed {INPUT_SEED}), exp_contraction")
            self.metric = (f"Gedges/s per CC solve (exp_contraction, random hyperbolic graph n=2^{k}, "
                           f"d=16, gamma=2.6)")
            self.flags = f"-gen rhg -n {k} -d 16 -gamma 2.6"
        else:
            side = args.grid
            self.n = side * side
            self.desc = f"grid2d {side}x{side} p={GRID_P} (seed {INPUT_SEED}), exp_contraction"
            self.metric = f"Gedges/s per CC solve (exp_contraction, 2D bond percolation {side}x{side}, p=0.5)"
            self.flags = f"-gen grid_2d -n {side} -m {side} -p 0.5"
        self.args = args

    def ours_host(self):
        """The graph from the library's host generators (libccgen)."""
        import components_gb300 as cc
        if self.name == "rhg":
            return cc.gen_rhg(self.n, RHG_DEG, RHG_GAMMA, seed=INPUT_SEED, id_bytes=4)
        return cc.gen_grid(self.args.grid, self.args.grid, GRID_P, seed=INPUT_SEED, id_bytes=4)

    def ours_device(self, device):
        """The GPU arm's graph, built on the device by the library's device
        generators (the host generators' graph bit for bit), and its host copy
        (for the end-to-end steps and the checks)."""
        import components_gb300 as cc
        if self.name == "rhg":
            D = cc.gen_rhg_device(self.n, RHG_DEG, RHG_GAMMA, seed=INPUT_SEED, id_bytes=4, device=device)
        else:
            D = cc.gen_grid_device(self.args.grid, self.args.grid, GRID_P, seed=INPUT_SEED, id_bytes=4,
                                   device=device)
        H = cc.StaticGraph(D.row_ptr.cpu().numpy().view(np.uint64), D.col.cpu().numpy().view(np.uint32))
        return H, D

    def oracle(self):
        """The same graph through the oracle's own input path."""
        import oracle
        if self.name == "rhg":
            return oracle.gen_rhg(self.n, RHG_DEG, RHG_GAMMA, seed=INPUT_SEED, id_bytes=4)
        return oracle.gen_grid(self.args.grid, self.args.grid, GRID_P, seed=INPUT_SEED, id_bytes=4)

    def config(self, n: int, m: int, world: int) -> dict:
        """The config dict of the JSON line, identical in both arms."""
        return {"workload": self.desc, "reference_flags": self.flags, "n": n, "m_dir": m,
                "id_bytes": 4, "algo": "exp_contraction", "beta": BETA, "seq": SEQ,
                "algo_seed": ALGO_SEED, "parallelism": f"replicas x{world}",
                "l2": l2_note(8 * (n + 1) + 4 * m + 4 * n)}


def l2_note(nbytes: int) -> str:
    if nbytes > L2_BYTES:
        return f"inputs larger than L2 ({nbytes / 1e9:.2f} GB CSR+labels > 129 MB), no flush"
    return f"inputs of {nbytes / 1e6:.1f} MB fit L2 (a reduced size for profiling, not the config)"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x: float, world: int, device=None) -> float:
    """The slowest rank's value of x (every rank calls it; one rank: x)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_gedges(world: int, m: int, ms_per_step: float) -> float:
    """Gedges/s of the whole job: every rank solves its own m-entry replica."""
    return world * m / (ms_per_step * 1e-3) / 1e9


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    return FALLBACK_HBM, "fallback 6.8 TB/s (MEASURED_PEAKS.json absent)"


def traffic_from_profile(kernel: str, workload: str):
    """dram bytes per launch of `kernel` on `workload` from the committed ncu
    summaries (profiles/traffic.json)."""
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists():
        return None, None
    d = json.loads(p.read_text())
    e = d.get(workload, {}).get(kernel)
    if not e:
        return None, None
    return e.get("dram_bytes_per_launch"), e.get("source")


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.25)
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# The CPU baseline times a bounded sample of the workload: the subgraph induced
# by the first 1/CPU_SAMPLE_DIV of the vertices (on the hyperbolic graph a
# contiguous angular sector, on the grid a band of rows), which holds one
# solve to a few seconds on the host cores.
CPU_SAMPLE_DIV = 4


def cpu_sample(G):
    import oracle
    k = max(1, G.n // CPU_SAMPLE_DIV)
    S = oracle.induced_prefix(G, k)
    return S, (f"the subgraph induced by vertices [0, {k}) of the graph (1/{CPU_SAMPLE_DIV} of the "
               f"vertices, {S.m} of its {G.m} directed entries)")


def cpu_reference_run(G, steps: int, warmup: int):
    """Time the oracle's restatement of ExponentialContraction with one rank
    per host core (OpenMP threads) on G (any graph with numpy() and n).
    Returns (Gedges/s, mean seconds per solve, ranks)."""
    import ctypes as C
    import oracle
    threads = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    n, rp, col = oracle.csr_u64(G)
    out = np.empty(max(n, 1), np.uint64)
    rounds = C.c_uint64()
    times = []
    for i in range(warmup + steps):
        t0 = time.perf_counter()
        oracle.lib().or_exp_contraction(n, rp, col, threads, BETA, SEQ, 0, ALGO_SEED + i, out,
                                        C.byref(rounds))
        t = time.perf_counter() - t0
        if i >= warmup:
            times.append(t)
    m = int(rp[-1]) if n else 0
    mean = sum(times) / max(len(times), 1)
    return m / mean / 1e9, mean, threads


def reference_arm(args, wl: Workload, world: int) -> dict:
    """The reference arm: the oracle's restatement on the host cores, on the
    graph built by the oracle's own input path.  Imports nothing of
    components_gb300 and loads no GPU library."""
    import oracle
    oracle.build()
    H = wl.oracle()
    S, what = cpu_sample(H)
    gps, mean_s, threads = cpu_reference_run(S, max(args.steps, 1), args.warmup)
    sample = (f"{what} ({wl.flags}), one solve per step, {max(args.steps, 1)} steps after "
              f"{args.warmup} warm-up, {mean_s:.2f} s each; oracle/cc_oracle.c restatement of "
              f"ExponentialContraction (exponential_contraction.h:59-319) with {threads} ranks as "
              f"threads; Gedges/s = the sample's entries / its solve time")
    return {
        "impl": "reference", "metric": wl.metric, "value": gps, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": mean_s * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64", "data": "synthetic (seeded stand-in for KaGen)",
        "config": wl.config(H.n, H.m, world),
        "cpu_baseline": {"value": gps, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": gps, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def gpu_arm(args, wl: Workload, rank: int, world: int, local: int) -> dict | None:
    """The headline line of our arm (every rank solves its own replica)."""
    import torch
    import components_gb300 as cc

    t_gen = time.perf_counter()
    G, D = wl.ours_device(f"cuda:{local}")
    gen_s = time.perf_counter() - t_gen
    n, m = G.n, G.m
    conf = cc.Config(seed=ALGO_SEED, beta=BETA, sequential_limit=SEQ)
    ctx = cc.Context(local)
    ctx.set_tuning(hook_mode=args.hook_mode, tile_vertices=args.tile, tile_threads=args.tile_threads)
    stream = torch.cuda.ExternalStream(ctx.stream_handle)
    lab = torch.empty(n, dtype=torch.int32, device=f"cuda:{local}")
    solver = cc.ExponentialContraction(conf, 0, 1, ctx)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # ---- device-resident solve ---------------------------------------------
    for _ in range(args.warmup):
        solver.FindComponents(D, lab)
    ctx.set_profiling(True)
    barrier()
    with ClockSampler(local) as clocks, NoGC():
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            solver.FindComponents(D, lab)
        ev1.record(stream)
        barrier()
    # per-kernel CUDA-event times of the timed solves, summed by the library
    tot = ctx.profile_totals()
    ctx.set_profiling(False)
    launches = tot["kernel_launches"]
    kstats = tot["kernels"]
    solve_ms_mean = tot["solve_ms"] / max(tot["solves"], 1)
    elapsed_ms = max_over_ranks(ev0.elapsed_time(ev1), world, f"cuda:{local}")
    ms_per_step = elapsed_ms / args.steps
    value = whole_job_gedges(world, m, ms_per_step)
    clock = clocks.summary()
    got_dev = lab.cpu().numpy().view(np.uint32).copy()

    # ---- end to end through the C ABI with pinned host buffers ---------------
    Hp = G.pinned()
    hlab = torch.empty(n, dtype=torch.int32).pin_memory()
    # untimed warm-up of the end-to-end path: at least five calls (the first
    # timed steps after three had sometimes taken 1.5-2x a settled step)
    for _ in range(max(5, args.warmup)):
        solver.FindComponents(Hp, hlab)
    barrier()
    with NoGC():
        t0 = time.perf_counter()
        step_s = []
        for _ in range(args.steps):
            ts = time.perf_counter()
            solver.FindComponents(Hp, hlab)  # returns once the labels are in hlab
            step_s.append(time.perf_counter() - ts)
        barrier()
    e2e_s = (time.perf_counter() - t0) / args.steps
    e2e_st = solver.last_stats  # bytes the library moved over the host link in the last step
    e2e_s = max_over_ranks(e2e_s, world, f"cuda:{local}")
    e2e_value = whole_job_gedges(world, m, e2e_s * 1e3)
    got_host = hlab.numpy().view(np.uint32).copy()
    # per-kernel CUDA-event times of one more (untimed) end-to-end call
    ctx.set_profiling(True)
    solver.FindComponents(Hp, hlab)
    e2e_kernels = {k: round(v["ms"], 4) for k, v in solver.last_stats["kernels"].items()}
    e2e_solve_ms = solver.last_stats["solve_ms"]
    ctx.set_profiling(False)
    # the same call with the rows copied to the device in chunks instead of
    # read in place (what a caller with pageable buffers gets), for comparison
    ctx.set_host_reads(False)
    for _ in range(max(5, args.warmup)):
        solver.FindComponents(Hp, hlab)
    barrier()
    with NoGC():
        t0 = time.perf_counter()
        copied_s = []
        for _ in range(args.steps):
            ts = time.perf_counter()
            solver.FindComponents(Hp, hlab)
            copied_s.append(time.perf_counter() - ts)
        barrier()
    copied_mean = max_over_ranks((time.perf_counter() - t0) / args.steps, world, f"cuda:{local}")
    copied_st = solver.last_stats
    ctx.set_host_reads(True)
    got_copied = hlab.numpy().view(np.uint32).copy()
    del Hp

    # ---- roofline of the dominant kernel -------------------------------------
    top = max(kstats.items(), key=lambda kv: kv[1]["ms"]) if kstats else (None, None)
    peak, peak_src = peaks()
    roof = None
    if top[0]:
        name, k = top
        per_launch_bytes = k["bytes"] / max(k["launches"], 1)
        per_launch_ms = k["ms"] / max(k["launches"], 1)
        achieved = per_launch_bytes / (per_launch_ms * 1e-3) / 1e9
        traffic, traffic_src = traffic_from_profile(name, wl.name)
        roof = {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic,
                "algorithmic_bytes_per_launch": per_launch_bytes, "ms_per_launch": per_launch_ms,
                "peak_source": peak_src, "traffic_source": traffic_src}
    # per-solve roofline (the survey's B_solve / t_solve): the library's sum of
    # every launched kernel's algorithmic bytes over a solve, against the
    # solve's CUDA-event time
    solve_roof = None
    if tot.get("solves") and tot.get("bytes_algorithmic") and tot.get("solve_ms"):
        b_solve = tot["bytes_algorithmic"] / tot["solves"]
        t_solve = tot["solve_ms"] / tot["solves"]
        solve_roof = {"bytes_algorithmic_per_solve": b_solve, "ms_per_solve": t_solve,
                      "achieved": b_solve / (t_solve * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                      "frac": b_solve / (t_solve * 1e-3) / 1e9 / peak}
    ksum = max(sum(x["ms"] for x in kstats.values()), 1e-12)
    share = {k: v["ms"] / ksum for k, v in kstats.items()}
    per_kernel = {k: {"launches_per_solve": v["launches"] / max(tot["solves"], 1),
                      "ms_per_launch": v["ms"] / max(v["launches"], 1),
                      "frac": (v["bytes"] / max(v["launches"], 1) / (v["ms"] / max(v["launches"], 1) * 1e-3)
                               / 1e9 / peak) if v["bytes"] and v["ms"] > 0 else None}
                  for k, v in kstats.items()}

    if world > 1:
        torch.distributed.barrier()
    if rank != 0:
        return None

    # labels checked against the oracle's union-find once (outside the timed regions)
    checked = None
    if not args.no_check:
        import oracle
        oracle.build()
        want = oracle.uf_labels(G)
        checked = bool(np.array_equal(got_dev.astype(np.uint64), want)
                       and np.array_equal(got_host, got_dev) and np.array_equal(got_copied, got_dev))

    # ---- CPU baseline: the oracle restatement on a bounded sample -------------
    cpu = None
    if world == 1 and args.cpu_steps > 0:
        S, what = cpu_sample(G)
        gps, mean_s, threads = cpu_reference_run(S, args.cpu_steps, 1)
        cpu = {"value": gps, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{what}, {args.cpu_steps} timed solves after 1 warm-up "
                         f"({mean_s:.2f} s each); oracle/cc_oracle.c restatement of "
                         f"ExponentialContraction with {threads} ranks as threads"}

    return {
        "metric": wl.metric, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic (seeded stand-in for KaGen)",
        "config": wl.config(n, m, world),
        "virtual_ranks": 1,
        "e2e": {"value": e2e_value, "unit": UNIT,
                "h2d_bytes_per_step": int(e2e_st["h2d_bytes"]), "d2h_bytes_per_step": int(e2e_st["d2h_bytes"]),
                "input_bytes_per_step": 8 * (n + 1) + 4 * m,
                "h2d_note": "CSR in pinned host memory, read inside the timed call: by sampled linking "
                            "the kernels read it in place (the offsets, each row's link entries, the rows "
                            "outside the giant component; h2d_bytes counts the offsets and link entries, "
                            "the link moves whole sectors around them); otherwise it is copied (row "
                            "offsets of rows under 255 entries as one degree byte each when streamed "
                            "under the tiled pass)",
                "ms_per_step": e2e_s * 1e3,
                "ms_min_median_max": [min(step_s) * 1e3, statistics.median(step_s) * 1e3,
                                      max(step_s) * 1e3],
                "ms_steps": [round(x * 1e3, 3) for x in step_s],
                "kernels_ms_one_call": e2e_kernels, "solve_ms_one_call": e2e_solve_ms,
                "rows_copied": {"value": whole_job_gedges(world, m, copied_mean * 1e3), "unit": UNIT,
                                "ms_per_step": copied_mean * 1e3,
                                "ms_median": statistics.median(copied_s) * 1e3,
                                "h2d_bytes_per_step": int(copied_st["h2d_bytes"]),
                                "d2h_bytes_per_step": int(copied_st["d2h_bytes"])}},
        "gpu_launches": launches,
        "roofline": roof,
        "solve_roofline": solve_roof,
        "kernel_share": share,
        "per_kernel": per_kernel,
        "solve_ms_mean": solve_ms_mean,
        "generated_on_device_s": gen_s,
        "labels_match_oracle": checked,
        "clocks": clock,
        "cpu_baseline": cpu,
    }


# ---- the other configurations' lines -------------------------------------------
def _timed_solves(solver, D, lab, steps, warmup, ctx):
    for _ in range(warmup):
        solver.FindComponents(D, lab)
    ctx.set_profiling(True)
    ms, kern = [], {}
    for _ in range(steps):
        solver.FindComponents(D, lab)
        st = ctx.stats()
        ms.append(st["solve_ms"])
        for k, v in st["kernels"].items():
            a = kern.setdefault(k, {"launches": 0, "ms": 0.0, "bytes": 0})
            for f in a:
                a[f] += v[f]
    ctx.set_profiling(False)
    return ms, kern, st


def workload_options(args, name):
    """G(2^20, 2^22) with 64-bit ids, or the 2^k-vertex RHG (d = 16, gamma = 2.6):
    one JSON line per (algo option, virtual ranks)."""
    import torch
    import components_gb300 as cc
    import oracle
    t0 = time.time()
    if name == "gnm":
        G = cc.gen_gnm(1 << 20, 1 << 22, seed=INPUT_SEED, id_bytes=8)
        desc = "G(n=2^20, m=2^22) uniform endpoints, u64 ids"
        D = G.to_device("cuda:0")
    else:
        D = cc.gen_rhg_device(1 << args.rhg_log2n, RHG_DEG, RHG_GAMMA, seed=INPUT_SEED, id_bytes=4)
        G = cc.StaticGraph(D.row_ptr.cpu().numpy().view(np.uint64), D.col.cpu().numpy().view(np.uint32))
        desc = f"RHG n=2^{args.rhg_log2n}, d=16, gamma=2.6 (threshold model), u32 ids"
    gen_s = time.time() - t0
    want = oracle.uf_labels(G) if not args.no_check else None
    dt = torch.int32 if G.id_bytes == 4 else torch.int64
    lab = torch.empty(G.n, dtype=dt, device="cuda:0")
    peak, _ = peaks()
    lines = {"exp1": ("exp", 1, 1), "exp16": ("exp", 16, 1), "exp16seq0": ("exp", 16, 0),
             "allreduce": ("allreduce", 1, 1), "shortcuts": ("shortcuts", 1, 1), "local": ("local", 1, 1),
             "labels": ("labels", 1, 1)}
    for key in args.options.split(","):
        algo, P, seq = lines[key]
        ctx = cc.Context(0)
        solver = cc.SOLVERS[algo](cc.Config(seed=ALGO_SEED, sequential_limit=seq), 0, P, ctx)
        ms, kern, st = _timed_solves(solver, D, lab, args.steps, args.warmup, ctx)
        ok = None
        if want is not None:
            got = lab.cpu().numpy().view(np.uint32 if G.id_bytes == 4 else np.uint64)
            ok = bool(np.array_equal(got.astype(np.uint64), want))
        med = statistics.median(ms)
        roof = None
        if kern:
            top = max(kern.items(), key=lambda kv: kv[1]["ms"])
            per_ms = top[1]["ms"] / top[1]["launches"]
            ach = top[1]["bytes"] / top[1]["launches"] / (per_ms * 1e-3) / 1e9
            roof = {"kernel": top[0], "achieved_GBs": ach, "frac": ach / peak, "ms_per_launch": per_ms,
                    "per_kernel": {k: {"launches": v["launches"] // args.steps,
                                       "ms_per_launch": v["ms"] / v["launches"],
                                       "frac": (v["bytes"] / v["launches"]
                                                / (v["ms"] / v["launches"] * 1e-3) / 1e9 / peak)
                                       if v["bytes"] and v["ms"] > 0 else None}
                                   for k, v in kern.items()}}
        print(json.dumps({
            "workload": name, "graph": desc, "n": G.n, "m_dir": G.m, "algo": algo,
            "virtual_ranks": P, "seq": seq, "metric": "Gedges/s per CC solve",
            "value": G.m / (med * 1e-3) / 1e9, "unit": "Gedges/s", "solve_ms_median": med,
            "levels": st["levels"], "rounds": st["rounds"], "level_edges": st["level_edges"],
            "roofline": roof,
            "kernel_ms": {k: v["ms"] / args.steps for k, v in kern.items()},
            "labels_match_oracle": ok, "gen_s": gen_s}), flush=True)
        ctx.close()


def workload_batch(args):
    """4096 G(n, m) graphs, n log-uniform in [2^8, 2^18], degree uniform in
    [0.5, 8]: one batched solve (CUDA-graph replay) against 4096 plain
    cc_ctx_run launches on the same device-resident graphs."""
    import torch
    import components_gb300 as cc
    from components_gb300 import batch as B
    t0 = time.time()
    bt = B.gen_batch(args.batch_k, 8, 18, 0.5, 8.0, seed=INPUT_SEED)
    gen_s = time.time() - t0
    D = bt.to_device("cuda:0")
    ctx = cc.Context(0)
    tune = B.autotune(D, ctx, reps=2)
    lab = torch.empty(bt.total_n, dtype=torch.int32, device="cuda:0")
    for _ in range(args.warmup):
        B.batch_run(D, ctx, tune, lab)
    torch.cuda.synchronize()
    with NoGC():
        t0 = time.perf_counter()
        for _ in range(args.steps):
            B.batch_run(D, ctx, tune, lab)
        torch.cuda.synchronize()
        batched_s = (time.perf_counter() - t0) / args.steps
    batched = lab.cpu().numpy().view(np.uint32).copy()
    # plain path, looped in C++: one cc_ctx_run per graph, inputs already on the device
    conf = cc.Config(seed=ALGO_SEED)
    plain_c = torch.empty(bt.total_n, dtype=torch.int32, device="cuda:0")
    B.plain_run(D, ctx, plain_c, "exp", conf)  # warm-up (and the per-graph offsets)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    B.plain_run(D, ctx, plain_c, "exp", conf)
    torch.cuda.synchronize()
    plain_c_s = time.perf_counter() - t0
    same_c = bool(np.array_equal(plain_c.cpu().numpy().view(np.uint32), batched))
    # the same loop from Python (ctypes and tensor slicing per graph)
    v, r, c = bt.numpy()
    graphs = []
    for i in range(bt.k):
        a, b = int(v[i]), int(v[i + 1])
        rp = torch.from_numpy((r[a:b + 1] - r[a]).view(np.int64).copy()).to("cuda:0")
        col = D.col[int(r[a]):int(r[b])]
        graphs.append(cc.StaticGraph(rp, col))
    plain_lab = torch.empty(bt.total_n, dtype=torch.int32, device="cuda:0")
    solver = cc.ExponentialContraction(cc.Config(seed=ALGO_SEED), 0, 1, ctx)
    for i in range(min(bt.k, 64)):
        solver.FindComponents(graphs[i], plain_lab[int(v[i]):int(v[i + 1])])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(bt.k):
        solver.FindComponents(graphs[i], plain_lab[int(v[i]):int(v[i + 1])])
    torch.cuda.synchronize()
    plain_s = time.perf_counter() - t0
    same = bool(np.array_equal(plain_lab.cpu().numpy().view(np.uint32), batched))
    print(json.dumps({
        "workload": "batch", "graphs": bt.k, "total_n": bt.total_n, "total_m": bt.total_m,
        "metric": "graphs/s", "batched_graphs_per_s": bt.k / batched_s,
        "plain_graphs_per_s": bt.k / plain_c_s, "speedup": plain_c_s / batched_s,
        "plain_loop": "C++ (cc_batch_run_plain: one cc_ctx_run per graph)",
        "plain_python_graphs_per_s": bt.k / plain_s, "speedup_vs_python_loop": plain_s / batched_s,
        "batched_ms": batched_s * 1e3, "plain_ms": plain_c_s * 1e3, "plain_python_ms": plain_s * 1e3,
        "labels_bit_identical_c_loop": same_c,
        "batched_gedges_per_s": bt.total_m / batched_s / 1e9,
        "labels_bit_identical": same, "tuning": tune.as_dict(), "gen_s": gen_s}), flush=True)
    ctx.close()


def _to_host(D):
    import components_gb300 as cc
    rp = D.row_ptr.cpu().numpy().view(np.uint64)
    col = D.col.cpu().numpy()
    return cc.StaticGraph(rp, col.view(np.uint32 if col.itemsize == 4 else np.uint64))


def workload_serve(args):
    """Poisson stream of CC requests (GNM / 2D grid p = 0.5 / RHG gamma = 2.6,
    n log-uniform in [2^10, 2^22], degree uniform in [1, 16]) through the
    continuous-batching server, against the plain path (one cc_gpu_run per
    request with host buffers) on the same requests.  The pool of distinct
    graphs is built by the device generators and kept in page-locked host
    memory (requests arrive as host CSRs); the requests draw from it."""
    import torch
    import components_gb300 as cc
    from components_gb300.serve import Server
    rng = np.random.default_rng(INPUT_SEED)
    pool = []
    t0 = time.time()
    for i in range(args.serve_pool):
        kind = i % 3
        n = int(2 ** rng.uniform(10, args.serve_log2n_max))
        d = float(rng.uniform(1, 16))
        if kind == 0:
            D = cc.gen_gnm_device(n, max(1, int(n * d / 2)), seed=1000 + i, id_bytes=4)
        elif kind == 1:
            side = max(2, int(round(np.sqrt(n))))
            D = cc.gen_grid_device(side, side, 0.5, seed=1000 + i)
        else:
            D = cc.gen_rhg_device(n, d, 2.6, seed=1000 + i)
        pool.append(_to_host(D).pinned())  # page-locked: both paths copy at the link's rate
        del D
    torch.cuda.empty_cache()
    gen_s = time.time() - t0
    picks = [int(j) for j in rng.integers(0, len(pool), args.serve_requests)]
    reqs = [pool[j] for j in picks]
    edges = sum(G.m for G in reqs)
    # plain path, closed loop: one request after the other (one label array
    # kept per pool graph; repeated solves of a graph must agree with it)
    plain, plain_same = {}, True
    t0 = time.perf_counter()
    for j, G in zip(picks, reqs):
        lab = cc.find_components(G, "exp")
        if j in plain:
            plain_same &= bool(np.array_equal(lab, plain[j]))
        else:
            plain[j] = lab
    plain_s = time.perf_counter() - t0
    # served: capacity (closed loop: every request submitted at once), then an
    # open-loop Poisson stream at args.serve_load of that capacity
    with Server(budget_bytes=120 << 30) as srv:
        t0 = time.perf_counter()
        ts = [srv.submit(G) for G in reqs]
        for t in ts:
            srv.wait(t)
        cap_s = time.perf_counter() - t0
        open_loop = []
        same = plain_same
        for load in args.serve_load:
            rate = load * len(reqs) / cap_s
            gaps = rng.exponential(1.0 / rate, len(reqs))
            infos = [None] * len(reqs)
            tickets = [None] * len(reqs)
            submitted = threading.Semaphore(0)

            def producer():
                t_next = time.perf_counter()
                for i, G in enumerate(reqs):
                    t_next += gaps[i]
                    while True:  # sleep (releasing the GIL) until just before the arrival, then spin
                        dt = t_next - time.perf_counter()
                        if dt <= 0:
                            break
                        if dt > 5e-4:
                            time.sleep(dt - 3e-4)
                    tickets[i] = srv.submit(G)
                    submitted.release()

            def collector():
                # results are taken as they complete (a client collecting its
                # answers), which returns each request's memory to the HBM
                # budget; the wait blocks in C with the interpreter lock
                # released.  Labels are checked in a pass of their own below:
                # comparing them here held the interpreter lock for about
                # 0.2 ms a request and delayed the producer's arrivals.
                for i in range(len(reqs)):
                    submitted.acquire()
                    _, infos[i] = srv.wait(tickets[i])

            th = threading.Thread(target=producer)
            tc = threading.Thread(target=collector)
            th.start()
            tc.start()
            th.join()
            tc.join()
            served_s = max(x["done_s"] for x in infos) - min(x["submit_s"] for x in infos)
            lat = np.array([(x["done_s"] - x["submit_s"]) * 1e3 for x in infos])
            open_loop.append({"offered_fraction_of_burst_capacity": load, "arrival_rate_per_s": rate,
                              "served_graphs_per_s": len(reqs) / served_s,
                              "p50_ms": float(np.percentile(lat, 50)),
                              "p99_ms": float(np.percentile(lat, 99))})
        st = srv.stats()
        # every request once more through the server (untimed, all submitted
        # at once), each result checked against the graph solved alone
        ts = [srv.submit(G) for G in reqs]
        for i, t in enumerate(ts):
            lab, _ = srv.wait(t)
            same &= bool(np.array_equal(lab, plain[picks[i]]))
    low = open_loop[0]
    print(json.dumps({
        "workload": "serve", "requests": len(reqs), "pool_graphs": len(pool),
        "edges_total": edges, "metric": "p50/p99 latency (ms) and graphs/s",
        "capacity_graphs_per_s": len(reqs) / cap_s, "plain_graphs_per_s": len(reqs) / plain_s,
        "capacity_vs_plain": plain_s / cap_s,
        "p50_ms": low["p50_ms"], "p99_ms": low["p99_ms"], "open_loop": open_loop,
        "batches": st["batches"], "peak_hbm_bytes": st["peak_bytes_in_use"],
        "labels_same_alone_and_in_mix": same, "gen_s": gen_s,
        "sample": f"{len(reqs)} Poisson requests drawn from {len(pool)} distinct seeded graphs "
                  f"(device generators), n log-uniform in [2^10, 2^{args.serve_log2n_max:g}], "
                  "degree uniform in [1, 16]; the configuration's 100k-request stream is sampled "
                  "to keep the run within minutes"}), flush=True)


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--no-check", action="store_true")
    ap.add_argument("--workload", default="rhg",
                    choices=["rhg", "grid", "gnm", "rhg-options", "batch", "serve"],
                    help="rhg (the headline line) or grid print the contract line; the others "
                         "print their own lines")
    ap.add_argument("--rhg-log2n", type=int, default=RHG_LOG2N,
                    help="RHG size (default 2^26; smaller sizes are for ncu captures)")
    ap.add_argument("--grid", type=int, default=GRID_SIDE,
                    help="grid side (default 8192; smaller sides are for ncu captures)")
    ap.add_argument("--hook-mode", type=int, default=0,
                    help="hook schedule (cc_tuning.hook_mode: 0 auto, 1 global, 2 tiled, 3 sampled)")
    ap.add_argument("--tile", type=int, default=0, help="cc_tuning.tile_vertices (0 = default)")
    ap.add_argument("--tile-threads", type=int, default=0, help="cc_tuning.tile_threads")
    ap.add_argument("--options", default="exp1,exp16,exp16seq0,allreduce,shortcuts,local",
                    help="--workload gnm | rhg-options: the option lines to run, comma-separated")
    ap.add_argument("--batch-k", type=int, default=4096)
    ap.add_argument("--serve-requests", type=int, default=12000)
    ap.add_argument("--serve-pool", type=int, default=1200)
    ap.add_argument("--serve-log2n-max", type=float, default=22)
    ap.add_argument("--serve-load", type=float, nargs="+", default=[0.5, 0.8],
                    help="open-loop arrival rates as fractions of the burst capacity")
    return ap.parse_args(argv)


def main(argv=None):
    args = parse_args(argv)
    rank, world, local = dist_env()

    if args.impl == "reference":
        # rank 0 alone runs the CPU reference; the other ranks exit without work
        if rank != 0:
            return 0
        wl = Workload(args.workload if args.workload in ("rhg", "grid") else "rhg", args)
        print(json.dumps(reference_arm(args, wl, world)), flush=True)
        return 0

    import torch
    import __graft_entry__ as ge
    if args.workload not in ("rhg", "grid"):
        ge.build()
        torch.cuda.set_device(0)
        if args.workload == "gnm":
            workload_options(args, "gnm")
        elif args.workload == "rhg-options":
            workload_options(args, "rhg")
        elif args.workload == "batch":
            workload_batch(args)
        else:
            workload_serve(args)
        return 0

    if rank == 0 or world == 1:
        ge.build()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        dist.barrier()
        ge.build()
    torch.cuda.set_device(local)
    line = gpu_arm(args, Workload(args.workload, args), rank, world, local)
    if line is not None:
        print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
