#!/usr/bin/env python3
"""Barnes-Hut layout throughput (vertex-iterations/s) on one GB300.

Workload (default): random geometric graph, 1,000,000 points uniform in the
unit square, mean degree 6, largest connected component (986,822 vertices,
2,977,701 edges), uniform init in [-3,3]^2, algo 4 (BarnesHutApproximation),
bht 1.2, batch 256.  One step = one iteration of the layout over the whole
graph (tree build, repulsion of every vertex, attraction + minibatch updates).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

value      device-resident throughput: n * K / (sum of CUDA-event times of the
           K steps); L2 flushed (256 MB write) before every timed step.
e2e        the same through the C ABI with host buffers: per step, copy the
           coordinates from pinned host memory, run the iteration, copy them
           back (host wall clock).
roofline   dominant kernel (the repulsion traversal), bound by instruction
           issue: warp instructions per launch (live record visits x the
           instructions per visit of its committed ncu capture) over
           152 SMs x 4 schedulers x the sampled SM clock; beside it the
           step's algorithmic bytes (build, traversal, sweep) over the step
           time against the measured HBM copy bandwidth.
cpu_baseline  the FP64 oracle port (reference Makefile optimisation flags)
           on all host cores, a bounded sample of iterations from the same start.

With --impl reference the reference's CPU implementation is timed on the same
workload (oracle/_ref/BatchLayout when it exists and runs here, else the port).
Multi-GPU: independent replicas (the layout has no data-parallel split that
avoids a per-batch all-gather), one per rank, value = sum over ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "1M-vertex BH layout: s to plain-energy (learned vs plain), vertex-iters/s"
UNIT = "vertex-iters/s"
WORKLOADS = {
    "rgg1m": dict(algo=4, batch=256, theta=1.2,
                  desc="random geometric graph, 1,000,000 points in the unit square, mean degree 6, "
                       "largest component; uniform init in [-3,3]^2; algo 4 (Barnes-Hut), bht 1.2, batch 256"),
    "chunglu100k": dict(algo=2, batch=256, theta=1.2,
                        desc="Chung-Lu power-law graph, 100,000 vertices, exponent 2.5, mean degree 10, "
                             "largest component; disc init; algo 2 (all-pairs minibatch), batch 256"),
    "grid64": dict(algo=2, batch=256, theta=1.2,
                   desc="64x64 triangulated grid (4,096 vertices, 12,033 edges); disc init; algo 2, batch 256"),
    "greedy100k": dict(algo=5, batch=256, theta=1.2, graph="chunglu100k", iters_per_step=10,
                       desc="the 100,000-vertex Chung-Lu graph of chunglu100k; algo 5 (greedy approximation), "
                            "batch 256; one step = 10 iterations in the reference's phase split (9 with the "
                            "depth-first-walk repulsion, 1 all-pairs with unit-vector repulsion)"),
    "sd100k": dict(algo=7, batch=256, theta=1.2, graph="chunglu100k",
                   desc="the 100,000-vertex Chung-Lu graph of chunglu100k; algo 7 (SD: attraction over every "
                        "CSR neighbour, all-pairs repulsion), batch 256"),
    "batched256": dict(algo="batched", batch=256, theta=1.2, iterations=30, graphs=256,
                       desc="profiling case of the batched launch: the first 256 graphs of the 2,048-graph mix "
                            "(same generator and seed), 30 iterations"),
    "batched2048": dict(algo="batched", batch=256, theta=1.2, iterations=300, graphs=2048,
                        desc="2,048 graphs, sizes log-uniform in 200-20,000 vertices, a third each of triangulated "
                             "grids, random geometric graphs (mean degree 6) and Chung-Lu graphs (exponent 2.5, "
                             "mean degree 8), disc init per graph; 300 iterations of algo 2 below 5,000 vertices "
                             "and algo 4 (bht 1.2) from there, batch 256; one persistent launch replayed as a "
                             "CUDA graph"),
}
REF_BINARY_NOTE = ("the reference binary (oracle/_ref/BatchLayout, built from the reference's sources with its "
                   "Makefile flags) is an x86-64 build that does not travel to this Arm host and the reference "
                   "sources are not here to rebuild it; the port restates the same FP64 arithmetic and is pinned "
                   "bit-exact to the reference (strict flags) by the golden-vector tests")
KERNEL_FOR_ALGO = {4: "traverse_kernel", 2: "minibatch_kernel", 3: "minibatch_kernel", 8: "minibatch_kernel",
                   7: "minibatch_kernel", 5: "greedy_iteration_kernel"}
DECAY = {2: 0.999, 4: 0.999, 7: 0.999, 3: 0.99, 8: 0.99, 5: 0.99}


def replica_throughput(dist, ws, units_per_step, steps, total_ms, device):
    """Whole-job throughput of `ws` independent replicas that each ran
    `steps` steps of `units_per_step` units: the job takes as long as its
    slowest rank (all-reduce MAX of the timed milliseconds).  Returns
    (units per second, job milliseconds)."""
    if dist:
        import torch
        t = torch.tensor([float(total_ms)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    return ws * units_per_step * steps / (total_ms / 1e3), total_ms


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """nvidia-smi sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return None
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for k, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(k)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        return None


def traffic_from_profile(kernel: str, workload: str):
    """dram bytes per launch from the committed ncu summary, if there is one."""
    return profile_figure(kernel, workload, "dram_bytes_per_launch")


def profile_figure(kernel: str, workload: str, key: str):
    """A `key: value` figure from the committed ncu summary of the kernel."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_{workload}.md")
    if not os.path.exists(path):
        return None
    m = re.search(re.escape(key) + r":\s*([0-9.eE+]+)", open(path).read())
    return float(m.group(1)) if m else None


def allpairs_fraction(B, torch, device: int, flush, iterations: int = 3) -> dict:
    """All-pairs minibatch (algo 2) on the 100,000-vertex Chung-Lu graph: the
    minibatch kernel's time per iteration (CUDA events on the library's
    stream, L2 flushed before each iteration) and its fraction of the FP32
    FMA peak (10 flops per ordered pair, n^2 pairs per iteration)."""
    g, xy = load_workload("chunglu100k")
    with B.Algorithms(g.rowptr, g.colids, device=device) as a:
        a.nCoordinates = xy
        a.run_resident(2, 1, 256, 1.2, 1.0, want_energy=True)  # warm-up (builds the cursor table)
        a.kernel_time("minibatch_kernel")
        step = 0.999
        for _ in range(iterations):
            flush.zero_()
            torch.cuda.synchronize()
            a.run_resident(2, 1, 256, 1.2, step, want_energy=True)
            step *= 0.999
        torch.cuda.synchronize()
        ms, cnt = a.kernel_time()
    per_it = ms / max(cnt, 1)
    flops = 10.0 * float(g.n) * g.n
    peak = 152 * 128 * 2 * 2070e6 / 1e12
    tflops = flops / (per_it * 1e-3) / 1e12
    return {"workload": "chunglu100k: " + WORKLOADS["chunglu100k"]["desc"], "vertices": g.n,
            "ms_per_iteration": per_it, "iterations": cnt, "tflops": tflops, "peak_tflops": peak,
            "frac": tflops / peak,
            "pairs_per_clock_per_sm": float(g.n) * g.n / (per_it * 1e-3) / 152 / 2070e6,
            "note": "minibatch_kernel per iteration; peak = nominal FP32 FMA rate, 152 SMs x 128 lanes x 2 "
                    "flops x 2,070 MHz; the kernel's reciprocal (one MUFU operation per pair at 16 per clock "
                    "per SM) caps it at 16 pairs per clock per SM, 0.625 of this peak"}


def bh_roofline(g, kernel, workload, visits, kernel_s, step_s, sm_mhz, pk):
    """Roofline of the Barnes-Hut traversal and of the whole step.

    The traversal reads its tree records from L1/L2 (under 1 % of the record
    bytes reach DRAM), so its bound is instruction issue: warp instructions
    per launch = live record visits x (warp instructions per visit of the
    committed ncu capture of this kernel), over 152 SMs x 4 schedulers x the
    median SM clock sampled during the timed steps.  The record bytes (16 B
    per visit) are kept as a labelled secondary figure, and the step's
    algorithmic bytes (tree build, traversal, level sweep) over the step time
    give the HBM fraction of the whole iteration."""
    hbm = pk["hbm_gbs"] if pk else 6800.0
    hbm_src = "measured (MEASURED_PEAKS.json hbm_gbs)" if pk else "fallback 6.8 TB/s"
    inst_prof = profile_figure(kernel, workload, "warp_instructions_per_launch")
    visits_prof = profile_figure(kernel, workload, "record_visits_per_launch")
    n, nnz = float(g.n), float(g.nnz)
    # per iteration: Morton keys (read 8 B, write 8 B), 4 LSD passes over
    # (key 8 B + vertex 4 B) read and written, sorted positions and tree nodes
    # (~2n nodes of 24 B), pre-order records (2n x 16 B + FP64 centroid 16 B)
    build = n * 16 + 4 * n * 24 + n * 8 + 2 * n * 24 + 2 * n * 32
    traversal = visits * 16.0 + nnz * 12 + n * 24
    sweep = n * 24 + nnz * 12
    step_bytes = build + traversal + sweep
    step = {"bound": "hbm", "achieved": step_bytes / step_s / 1e9, "peak": hbm, "unit": "GB/s",
            "frac": step_bytes / step_s / 1e9 / hbm, "algorithmic_bytes_per_step": step_bytes,
            "parts": {"build": build, "traversal": traversal, "sweep": sweep},
            "note": "tree build + traversal (record visits x 16 B + CSR term) + level sweep, over ms_per_step; "
                    "peak " + hbm_src}
    records = {"achieved": visits * 16.0 / kernel_s / 1e9, "unit": "GB/s", "bytes_per_launch": visits * 16.0,
               "frac_of_hbm": visits * 16.0 / kernel_s / 1e9 / hbm,
               "note": "record visits x 16 B per launch over the traversal time; over 99 % of these bytes "
                       "hit L1/L2, so this is not a DRAM figure"}
    if inst_prof and visits_prof:
        inst = visits * inst_prof / visits_prof
        peak = 152 * 4 * sm_mhz * 1e6 / 1e9
        return {"bound": "issue", "achieved": inst / kernel_s / 1e9, "peak": peak, "unit": "Gwarp-inst/s",
                "frac": inst / kernel_s / 1e9 / peak, "traffic": traffic_from_profile(kernel, workload),
                "kernel": kernel, "kernel_ms_per_launch": kernel_s * 1e3, "record_visits_per_launch": visits,
                "warp_instructions_per_launch": inst,
                "instructions_source": f"live record visits x {inst_prof / visits_prof:.4f} warp instructions per "
                                       f"visit (smsp__inst_executed.sum / visits of the ncu capture in "
                                       f"profiles/{kernel}_{workload}.md)",
                "peak_source": f"152 SMs x 4 schedulers x 1 warp instruction per clock x {sm_mhz:.0f} MHz "
                               "(median SM clock sampled during the timed steps)",
                "record_bytes": records, "step": step}
    return {"bound": "hbm", "achieved": step["achieved"], "peak": hbm, "unit": "GB/s", "frac": step["frac"],
            "traffic": traffic_from_profile(kernel, workload), "kernel": "whole step", "record_bytes": records,
            "step": step, "peak_source": hbm_src}


def load_workload(name: str):
    from batchlayoutcode_gb300 import graphs as G
    return G.cached_workload(WORKLOADS.get(name, {}).get("graph", name))


def load_batched(seed: int = 1, graphs: int = 2048):
    """The 2,048-graph mix (its first `graphs` graphs), cached as one .npz of
    concatenated arrays."""
    import numpy as np
    from batchlayoutcode_gb300 import graphs as G
    cache = os.path.join(ROOT, "batchlayoutcode_gb300", "_build", "workloads", f"batched2048_s{seed}.npz")
    if os.path.exists(cache):
        with np.load(cache) as z:
            vo, eo, rp, ci, xy, algo = (z[k] for k in ("vertex_offset", "edge_offset", "rowptr", "colids", "xy",
                                                       "algo"))
        count = min(graphs, vo.shape[0] - 1)
        gl = [(rp[vo[k] + k: vo[k + 1] + k + 1], ci[eo[k]:eo[k + 1]]) for k in range(count)]
        xys = [xy[vo[k]:vo[k + 1]] for k in range(count)]
        return gl, xys, algo[:count]
    gs, xys, algo = G.batched_mix(2048, 200, 20000, seed)
    vo = np.zeros(len(gs) + 1, np.int64)
    vo[1:] = np.cumsum([g.n for g in gs])
    eo = np.zeros(len(gs) + 1, np.int64)
    eo[1:] = np.cumsum([g.colids.shape[0] for g in gs])
    os.makedirs(os.path.dirname(cache), exist_ok=True)
    np.savez(cache, vertex_offset=vo, edge_offset=eo, rowptr=np.concatenate([g.rowptr for g in gs]),
             colids=np.concatenate([g.colids for g in gs]), xy=np.concatenate(xys), algo=algo)
    return [(g.rowptr, g.colids) for g in gs[:graphs]], xys[:graphs], algo[:graphs]


def batched_sample(graphs, algo, iterations):
    """Every 64th graph of the size-sorted mix (32 graphs spanning the size
    range) at all iterations: 10-30 s of CPU work."""
    import numpy as np
    order = np.argsort([len(rp) for rp, _ in graphs])
    pick = order[32::64]
    return [int(k) for k in pick], iterations


def cpu_baseline_batched(graphs, xys, algo, w, threads=None):
    import oracle
    pick, it = batched_sample(graphs, algo, w["iterations"])
    t0 = time.perf_counter()
    vi = 0
    for k in pick:
        rp, ci = graphs[k]
        oracle.layout(int(algo[k]), rp, ci, xys[k].astype("float64"), it, w["batch"], w["theta"],
                      nthreads=threads, fast=True)
        vi += (len(rp) - 1) * it
    dt = time.perf_counter() - t0
    return vi / dt, dt, len(pick), it


def cpu_baseline_port(g, xy, w, iters: int, threads: int | None = None):
    import oracle
    t0 = time.perf_counter()
    _, e, loops = oracle.layout(w["algo"], g.rowptr, g.colids, xy.astype("float64"), iters, w["batch"],
                                w["theta"], nthreads=threads, fast=True)
    dt = time.perf_counter() - t0
    return g.n * iters / dt, dt


def baseline_iters(w, n):
    # about 10-30 s of CPU work on a 16-core host
    if w["algo"] == 4:
        return max(2, min(50, int(2.0e7 / max(n, 1))))
    if w.get("iters_per_step", 1) > 1:  # whole steps, so that the phase split matches
        return w["iters_per_step"]
    return max(1, min(600, int(2.0e11 / max(n * n, 1))))


def workload_config(args, w, g) -> dict:
    """The `config` object of both arms' lines (the same keys and values, so
    that the two lines describe one workload)."""
    ips = w.get("iters_per_step", 1)
    return {"workload": f"{args.workload}: {w['desc']}", "vertices": g.n, "edges": g.nnz // 2,
            "step": (f"{ips} layout iterations" if ips > 1 else "one layout iteration") + " over the whole graph",
            "l2": "GPU steps: L2 flushed before every timed step (256 MB write)"}


def run_reference(args, w, g, xy):
    """Reference CPU implementation on the same workload."""
    cores = os.cpu_count() or 1
    ref_bin = os.path.join(ROOT, "oracle", "_ref", "BatchLayout")
    steps = args.steps + args.warmup
    iters_per_step = 1
    kind = "port"
    sample = None
    value = None
    if os.path.exists(ref_bin) and os.access(ref_bin, os.X_OK):
        try:
            from batchlayoutcode_gb300 import graphs as G
            with tempfile.TemporaryDirectory() as td:
                mtx, initf = os.path.join(td, "w.mtx"), os.path.join(td, "w.initf")
                G.write_mtx(g, mtx)
                G.write_initf(xy, initf)
                it = baseline_iters(w, g.n) if w.get("iters_per_step", 1) > 1 else \
                    max(1, min(steps, baseline_iters(w, g.n)))
                out = subprocess.run([ref_bin, "-input", mtx, "-output", td + "/", "-iter", str(it), "-algo",
                                      str(w["algo"]), "-batch", str(w["batch"]), "-bht", str(w["theta"]),
                                      "-initf", initf, "-threads", str(cores)], cwd=td, capture_output=True,
                                     text=True, timeout=1800)
                m = re.search(r"Wall time required:([0-9.eE+-]+)", out.stdout)
                if out.returncode == 0 and m:
                    secs = float(m.group(1))
                    value = g.n * it / secs
                    kind = "reference"
                    sample = f"{it} iterations of algo {w['algo']} (reference binary built from source, " \
                             f"stock flags), reported wall time incl. file init"
        except (OSError, subprocess.SubprocessError):
            value = None
    if value is None:
        it = baseline_iters(w, g.n) if w.get("iters_per_step", 1) > 1 else \
            max(1, min(steps, baseline_iters(w, g.n))) * iters_per_step
        value, secs = cpu_baseline_port(g, xy, w, it, cores)
        sample = f"{it} iterations of algo {w['algo']} with the FP64 port (oracle/oracle.cpp, reference " \
                 f"Makefile optimisation flags), same start, {cores} OpenMP threads"
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args, w, g),
            "parallelism": f"host CPU, {cores} threads",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample,
                             "why_port": None if kind == "reference" else REF_BINARY_NOTE},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def time_to_energy(B, g, w, iterations: int = 600):
    """Seconds to the plain run's final energy (+0.5%): the plain GPU run
    (greedy DFS start, `iterations` Barnes-Hut iterations from STEP 1) against
    the learned start refined by Barnes-Hut until that energy (greedy
    fallback), and the same pipeline with a zero network (pivot-MDS shape)."""
    import numpy as np
    from batchlayoutcode_gb300 import learned as LR
    params, sm = LR.load_model()
    with B.Algorithms(g.rowptr, g.colids, init=0) as a:
        e_plain, plain_s = a.BarnesHutApproximation(iterations, 0, w["batch"], w["theta"], 0)
    target = e_plain * 1.005
    with B.Algorithms(g.rowptr, g.colids, init=0) as a:
        a.kernel_time("mpnn_forward")
        r = a.learnedLayout(params, sm, iterations, target, w["batch"], w["theta"], LR.STEP0)
        fwd_ms, fwd_n = a.kernel_time()
    with B.Algorithms(g.rowptr, g.colids, init=0) as a:
        r0 = a.learnedLayout(np.zeros_like(params), sm, iterations, target, w["batch"], w["theta"], LR.STEP0)
    # the plain run from the breadth-first greedy start built on the device
    with B.Algorithms(g.rowptr, g.colids, init=4) as a:
        e_bfs, bfs_s = a.BarnesHutApproximation(iterations, 0, w["batch"], w["theta"], 0)
    # what the network itself buys: the lowest energy the same pipeline with a
    # zero network (the pivot-MDS shape) reaches in its first 100 refinement
    # iterations, then the iterations and seconds each start needs to reach it
    floor_its = 100
    with B.Algorithms(g.rowptr, g.colids, init=0) as a:
        a.learnedInit(np.zeros_like(params), sm)
        es, step = [], LR.STEP0
        for _ in range(floor_its):
            es.append(a.barnes_hut_iteration(w["batch"], w["theta"], step))
            step *= 0.999
    floor = min(es) * 1.005
    with B.Algorithms(g.rowptr, g.colids, init=0) as a:
        rf = a.learnedLayout(params, sm, floor_its, floor, w["batch"], w["theta"], LR.STEP0)
    with B.Algorithms(g.rowptr, g.colids, init=0) as a:
        rf0 = a.learnedLayout(np.zeros_like(params), sm, floor_its, floor, w["batch"], w["theta"], LR.STEP0)
    network_gain = {
        "target": f"lowest energy of the zero-network pipeline in its first {floor_its} refinement iterations x 1.005",
        "target_energy": floor, "zero_network_best_iteration": int(np.argmin(es)) + 1,
        "learned_iterations": rf["iterations"], "learned_s": rf["seconds"], "learned_fell_back": rf["fell_back"],
        "mds_only_iterations": rf0["iterations"], "mds_only_s": rf0["seconds"], "mds_only_fell_back": rf0["fell_back"],
        "speedup": rf0["seconds"] / rf["seconds"] if rf["seconds"] > 0 and not rf["fell_back"] else None,
    }
    flops = 2.0 * g.n * (32 * 64 + 2 * 128 * 64)
    return {
        "plain_energy": e_plain, "plain_s": plain_s,
        "learned_s": r["seconds"], "learned_energy": r["energy"], "learned_iterations": r["iterations"],
        "learned_start_s": r["init_seconds"], "fell_back": r["fell_back"],
        "speedup": plain_s / r["seconds"] if r["seconds"] > 0 else None,
        "mds_only_s": r0["seconds"], "mds_only_iterations": r0["iterations"], "mds_only_energy": r0["energy"],
        "bfs_start_plain_s": bfs_s, "bfs_start_plain_energy": e_bfs,
        "mpnn_forward_ms": fwd_ms, "mpnn_forward_tflops": flops / (fwd_ms * 1e-3) / 1e12 if fwd_ms > 0 else None,
        "target": "plain run's final energy x 1.005",
        "network_gain": network_gain,
        "note": "wall seconds through the C ABI, starts included (greedy DFS on the host; features, network "
                "and scale on the device); refinement STEP from 0.3; model batchlayoutcode_gb300/weights/"
                "mpnn_bh.blw (48 graphs of 1k-100k vertices); mds_only = the same pipeline with a zero network; "
                "bfs_start_plain = the plain run from the breadth-first start built on the device (bl_bfs_init)",
    }


def run_reference_batched(args, w):
    """The reference lays out one graph per process: run its binary (else the
    port) graph by graph over the bounded sample with all host threads."""
    graphs, xys, algo = load_batched(graphs=w["graphs"])
    cores = os.cpu_count() or 1
    pick, it = batched_sample(graphs, algo, w["iterations"])
    ref_bin = os.path.join(ROOT, "oracle", "_ref", "BatchLayout")
    value, kind, sample = None, "port", None
    if os.path.exists(ref_bin) and os.access(ref_bin, os.X_OK):
        try:
            from batchlayoutcode_gb300 import graphs as G
            secs, vi = 0.0, 0
            with tempfile.TemporaryDirectory() as td:
                for k in pick:
                    rp, ci = graphs[k]
                    g = G.Graph(n=len(rp) - 1, rowptr=rp, colids=ci)
                    mtx, initf = os.path.join(td, "w.mtx"), os.path.join(td, "w.initf")
                    G.write_mtx(g, mtx)
                    G.write_initf(xys[k], initf)
                    out = subprocess.run([ref_bin, "-input", mtx, "-output", td + "/", "-iter", str(it), "-algo",
                                          str(int(algo[k])), "-batch", str(w["batch"]), "-bht", str(w["theta"]),
                                          "-initf", initf, "-threads", str(cores)], cwd=td, capture_output=True,
                                         text=True, timeout=1800)
                    m = re.search(r"Wall time required:([0-9.eE+-]+)", out.stdout)
                    if out.returncode != 0 or not m:
                        raise subprocess.SubprocessError("reference run failed")
                    secs += float(m.group(1))
                    vi += g.n * it
            value, kind = vi / secs, "reference"
            sample = (f"{len(pick)} graphs of the mix (every 64th by size) x {it} iterations, one reference "
                      f"process per graph (binary built from source, stock flags), summed reported wall times")
        except (OSError, subprocess.SubprocessError):
            value = None
    if value is None:
        value, secs, npick, it = cpu_baseline_batched(graphs, xys, algo, w, cores)
        sample = (f"{npick} graphs of the mix (every 64th by size) x {it} iterations with the FP64 port "
                  f"(oracle/oracle.cpp, reference Makefile optimisation flags), {cores} OpenMP threads")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": batched_config(args, w, graphs, algo),
            "parallelism": f"host CPU, {cores} threads",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample,
                             "why_port": None if kind == "reference" else REF_BINARY_NOTE},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def batched_config(args, w, graphs, algo) -> dict:
    import numpy as np
    algo = np.asarray(algo)
    small = algo != 4
    return {"workload": f"{args.workload}: {w['desc']}", "graphs": len(graphs),
            "vertices": int(sum(len(rp) - 1 for rp, _ in graphs)),
            "minibatch_graphs": int(small.sum()), "barnes_hut_graphs": int((~small).sum()),
            "step": f"one batched layout: {w['iterations']} iterations of every graph",
            "l2": "GPU steps: L2 flushed before every timed step (256 MB write)"}


def run_batched(args, w, ws, rank, local):
    """One step = the whole batched layout (every graph, all iterations)."""
    import ctypes as C

    import numpy as np
    import torch

    dist = None
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    device = local if ws > 1 else 0
    import batchlayoutcode_gb300 as B
    B.build()
    graphs, xys, algo = load_batched(graphs=w["graphs"])
    iters, batch, theta = w["iterations"], w["batch"], w["theta"]
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        v, secs, npick, it = cpu_baseline_batched(graphs, xys, algo, w)
        cpu = {"value": v, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
               "sample": f"{npick} graphs of the mix (every 64th by size) x {it} iterations from the same starts, "
                         f"FP64 port (oracle/oracle.cpp) with the reference Makefile's optimisation flags, "
                         f"{os.cpu_count()} OpenMP threads, {secs:.1f} s"}
    bl = B.BatchedLayout(graphs, algo, xys, device=device)
    nv = int(bl.vertex_offset[-1])
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{device}")
    for _ in range(args.warmup):
        bl.run(iters, batch, theta)
    launches0 = bl.kernel_launches()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    times = []
    with Clocks(device) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            times.append(bl.run(iters, batch, theta))
    torch.cuda.synchronize()
    cyc = bl.graph_cycles().astype(np.float64)
    launches = bl.kernel_launches() - launches0
    value, total_ms = replica_throughput(dist, ws, nv * iters, args.steps, 1e3 * sum(times), f"cuda:{device}")
    total_s = total_ms / 1e3
    clocks = clk.summary()
    sizes = bl.sizes
    small = algo != 4
    pairs = float(np.sum(sizes[small].astype(np.float64) ** 2)) * iters
    avg_s = total_s / args.steps
    sm_mhz = (clocks or {}).get("sm_max_mhz") or 2070.0
    peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
    achieved = 10.0 * pairs / avg_s / 1e12
    roof = {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
            "traffic": traffic_from_profile("batched_kernel", args.workload), "kernel": "batched_kernel",
            "kernel_ms_per_launch": avg_s * 1e3, "launches": args.steps,
            "algorithmic_flops_per_launch": 10.0 * pairs,
            "note": "flops of the minibatch graphs' pair sweeps only (10 per pair and iteration); the "
                    "Barnes-Hut graphs' time is in the denominator, so this is a lower bound",
            "peak_source": "nominal FP32 FMA peak: 152 SMs x 128 lanes x 2 flops x max SM clock"}
    # end to end through the C ABI: host arrays in pinned memory, upload,
    # run, read back, every step
    L = bl._L

    def pinned(a, dtype):
        t = torch.empty(a.shape, dtype=dtype, pin_memory=True)
        t.copy_(torch.from_numpy(np.ascontiguousarray(a)))
        return t
    h_vo = pinned(bl.vertex_offset, torch.int32)
    h_eo = pinned(bl.edge_offset, torch.int64)
    h_rp = pinned(bl.rowptr, torch.int32)
    h_ci = pinned(bl.colids, torch.int32)
    h_al = pinned(bl.algo, torch.int32)
    h_xy = torch.empty((nv, 2), dtype=torch.float64, pin_memory=True)
    h_e = torch.empty(len(sizes), dtype=torch.float64, pin_memory=True)
    ip = C.POINTER(C.c_int)
    dp = C.POINTER(C.c_double)
    ctx = L.bl_batch_create(device)
    e2e_steps = max(3, min(args.steps, 5))
    secs = C.c_double()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        h_xy.copy_(torch.from_numpy(bl.xy0))
        rc = L.bl_batched_layout(ctx, len(sizes), C.cast(h_vo.data_ptr(), ip),
                                 C.cast(h_eo.data_ptr(), C.POINTER(C.c_longlong)), C.cast(h_rp.data_ptr(), ip),
                                 C.cast(h_ci.data_ptr(), ip), C.cast(h_al.data_ptr(), ip),
                                 C.cast(h_xy.data_ptr(), dp), iters, batch, theta, 1.0,
                                 C.cast(h_e.data_ptr(), dp), C.byref(secs))
        if rc != 0:
            raise RuntimeError(L.bl_last_error(ctx).decode())
    e2e_s = time.perf_counter() - t0
    L.bl_destroy(ctx)
    h2d = 16 * nv + 4 * (len(bl.rowptr) + len(bl.colids) + 2 * len(sizes)) + 8 * len(sizes)
    e2e = {"value": ws * nv * iters * e2e_steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": 16 * nv + 8 * len(sizes), "steps": e2e_steps,
           "note": "bl_batched_layout per step: host preparation, upload, autotuning, the launch, read-back"}
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_s * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": batched_config(args, w, graphs, algo),
            "parallelism": "replicas" if ws > 1 else "single GPU",
            "autotuned_parts": bl.parts().tolist(),
            "block_ms": {"max_minibatch_graph": float(cyc[small].max() / sm_mhz / 1e3),
                         "max_barnes_hut_graph": float(cyc[~small].max() / sm_mhz / 1e3)
                         if (~small).any() else 0.0,
                         "sum_minibatch": float(cyc[small].sum() / sm_mhz / 1e3),
                         "sum_barnes_hut": float(cyc[~small].sum() / sm_mhz / 1e3),
                         "note": "clock64 cycles per graph / max SM clock"},
            "e2e": e2e, "gpu_launches": launches, "roofline": roof, "cpu_baseline": cpu, "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    bl.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()


# Labels the library times with CUDA events around each stage of a
# Barnes-Hut iteration (direct launches, not the replayed graph).
BH_STAGES = ["frame_morton", "lsd_passes", "radix_sort", "gather_tree", "chain_kernel", "centroid_top",
             "centroid_kernel", "traverse_kernel", "sweep_kernel"]


def stage_times(a, w, flush, steps, warmup):
    """Live microseconds per stage of one Barnes-Hut iteration (L2 flushed
    before every iteration), and the iteration with direct launches and as
    the replayed graph."""
    import torch
    batch, theta = w["batch"], w["theta"]
    step = 1.0
    a.set_graph_mode(False)
    for _ in range(warmup):
        a.run_resident(4, 1, batch, theta, step, want_energy=False)
        step *= 0.999
    out = {"unit": "us", "iterations_per_stage": steps, "stages": {}}
    for lab in BH_STAGES:
        a.kernel_time(lab)
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            a.run_resident(4, 1, batch, theta, step, want_energy=False)
            step *= 0.999
        torch.cuda.synchronize()
        ms, cnt = a.kernel_time()
        out["stages"][lab] = round(ms / max(cnt, 1) * 1000, 1)
    for mode in (False, True):
        a.set_graph_mode(mode)
        ts = []
        for _ in range(steps + 2):
            flush.zero_()
            torch.cuda.synchronize()
            a.run_resident(4, 1, batch, theta, step, want_energy=False)
            step *= 0.999
            ts.append(a.last_run_ms())
        ts = sorted(ts[2:])
        out["graph_iteration" if mode else "direct_iteration"] = round(sum(ts) / len(ts) * 1000, 1)
    out["note"] = ("lsd_passes is part of radix_sort (which adds the runs of equal high halves), centroid_top "
                   "(the nodes that span blocks) part of centroid_kernel; the other stages of a direct "
                   "iteration add up to direct_iteration")
    return out


def io_times(reps: int = 3) -> dict:
    """Host-side input and output of the 1M-vertex workload: the MatrixMarket
    text of the random geometric graph (lower triangle, pattern symmetric)
    parsed into the sorted, mirrored CSR (parallel slices), the same through
    the binary CSR cache (first call parses and writes the cache, later calls
    read it), and the 1M-line `x y id` output file written with the %g
    formatting of writeToFile.  Median wall time of `reps` calls each."""
    import numpy as np
    from batchlayoutcode_gb300 import _lib, graphs as G
    g, xy = load_workload("rgg1m")
    tmp = tempfile.mkdtemp(prefix="blio")
    mtx = os.path.join(tmp, "rgg1m.mtx")
    G.write_mtx(g, mtx)
    mtx_bytes = os.path.getsize(mtx)

    def med(f):
        ts = []
        for _ in range(reps):
            t = time.perf_counter()
            out = f()
            ts.append(time.perf_counter() - t)
        return statistics.median(ts), out

    t_parse, (rp, ci, _) = med(lambda: _lib.read_matrix_market(mtx))
    assert np.array_equal(rp, g.rowptr) and np.array_equal(ci, g.colids)
    cache = os.path.join(tmp, "cache")
    os.makedirs(cache)
    t = time.perf_counter()
    _, _, info = _lib.read_matrix_market(mtx, cache)
    t_miss = time.perf_counter() - t
    assert not info["cached"]
    t_hit, (rp2, ci2, info2) = med(lambda: _lib.read_matrix_market(mtx, cache))
    assert info2["cached"] and np.array_equal(rp2, g.rowptr) and np.array_equal(ci2, g.colids)
    outd = os.path.join(tmp, "out") + os.sep
    os.makedirs(outd)
    xy64 = np.ascontiguousarray(xy, dtype=np.float64)
    t_write, path = med(lambda: _lib.write_coordinates(mtx, outd, "BHMINB", xy64))
    out_bytes = os.path.getsize(path)
    import shutil
    shutil.rmtree(tmp, ignore_errors=True)
    ms = lambda x: round(x * 1e3, 2)
    return {"workload": "rgg1m (%d vertices, %d CSR entries)" % (g.n, g.colids.size),
            "host_threads": os.cpu_count(), "reps": reps,
            "parse_mtx_ms": ms(t_parse), "mtx_bytes": mtx_bytes,
            "parse_mtx_MBps": round(mtx_bytes / t_parse / 1e6, 1),
            "csr_cache_miss_ms": ms(t_miss), "csr_cache_hit_ms": ms(t_hit),
            "write_coordinates_ms": ms(t_write), "output_bytes": out_bytes,
            "write_MBps": round(out_bytes / t_write / 1e6, 1)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="rgg1m", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--no-allpairs", action="store_true",
                    help="skip the all-pairs minibatch figure on the 100k Chung-Lu graph in the default line")
    ap.add_argument("--stages", action="store_true",
                    help="Barnes-Hut workloads: print the live time of every stage of one iteration and exit")
    ap.add_argument("--traverse-probe", action="store_true",
                    help="Barnes-Hut workloads: after --warmup iterations print the traversal's record visits, "
                         "then run one iteration (its traverse_kernel launch walks the same tree) and exit")
    ap.add_argument("--io", action="store_true",
                    help="host only: time the MatrixMarket reader, the binary CSR cache and the output writer "
                         "on the 1M-vertex graph, print one JSON line and exit")
    args = ap.parse_args()
    if args.io:
        print(json.dumps({"io": io_times()}))
        return
    args.warmup = max(3, args.warmup)
    ws, rank, local = dist_env()
    w = WORKLOADS[args.workload]

    if args.impl == "reference":
        if rank != 0:
            return
        if w["algo"] == "batched":
            run_reference_batched(args, w)
            return
        g, xy = load_workload(args.workload)
        run_reference(args, w, g, xy)
        return
    if w["algo"] == "batched":
        run_batched(args, w, ws, rank, local)
        return

    import numpy as np
    import torch

    dist = None
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    device = local if ws > 1 else 0

    import batchlayoutcode_gb300 as B
    B.build()
    g, xy = load_workload(args.workload)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        it = baseline_iters(w, g.n)
        v, secs = cpu_baseline_port(g, xy, w, it)
        cpu = {"value": v, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
               "sample": f"{it} iterations of algo {w['algo']} on the same graph from the same start, FP64 port "
                         f"(oracle/oracle.cpp) with the reference Makefile's optimisation flags, "
                         f"{os.cpu_count()} OpenMP threads, {secs:.1f} s"}

    a = B.Algorithms(g.rowptr, g.colids, device=device)
    a.nCoordinates = xy
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{device}")
    if args.stages and w["algo"] == 4:
        print(json.dumps(stage_times(a, w, flush, args.steps, args.warmup)))
        return
    if args.traverse_probe and w["algo"] == 4:
        # `warmup` iterations, the record visits of the repulsion walk at that
        # state (the counting instance), then one iteration whose traversal
        # launch (the timed instance) walks the same tree: an ncu capture of
        # that launch gives the warp instructions for exactly these visits
        a.set_graph_mode(False)  # direct launches: traverse_kernel<false> launch number warmup + 1 is the one
        a.run_resident(4, args.warmup, w["batch"], w["theta"], 1.0, want_energy=False)
        _, (visits, exact) = a.bh_repulsion(w["theta"])
        a.barnes_hut_iteration(w["batch"], w["theta"], 0.999 ** args.warmup)
        print(json.dumps({"traverse_probe": {"workload": args.workload, "iterations_before": args.warmup,
                                             "record_visits": visits, "fp64_retests": exact}}))
        return
    algo, batch, theta = w["algo"], w["batch"], w["theta"]
    ips = w.get("iters_per_step", 1)
    decay = DECAY[algo] ** ips
    step = 1.0
    # Barnes-Hut steps replay the captured iteration (a CUDA graph, captured
    # during the warm-up); the energy is not read back inside the timed steps
    graph = algo == 4
    a.set_graph_mode(graph)
    for _ in range(args.warmup):
        a.run_resident(algo, ips, batch, theta, step, want_energy=not graph)
        step *= decay

    kernel = KERNEL_FOR_ALGO[algo]
    visits_before = None
    if algo == 4:
        _, (visits_before, _) = a.bh_repulsion(theta)
    if not graph:
        a.kernel_time(kernel)  # start timing the dominant kernel
    launches0 = a.kernel_launches()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    times = []
    with Clocks(device) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            a.run_resident(algo, ips, batch, theta, step, want_energy=not graph)
            times.append(a.last_run_ms())
            step *= decay
    torch.cuda.synchronize()
    launches = a.kernel_launches() - launches0
    if graph:
        # per-kernel CUDA events cannot sit inside the replayed graph: time the
        # dominant kernel over direct launches of the same kind of steps
        a.set_graph_mode(False)
        a.kernel_time(kernel)
        kstep = step
        for _ in range(min(args.steps, 10)):
            flush.zero_()
            torch.cuda.synchronize()
            a.run_resident(algo, 1, batch, theta, kstep, want_energy=False)
            kstep *= decay
        torch.cuda.synchronize()
    kern_ms, kern_count = a.kernel_time()
    value, total_ms = replica_throughput(dist, ws, g.n * ips, args.steps, sum(times), f"cuda:{device}")
    clocks = clk.summary()

    # algorithmic bytes of the dominant kernel per launch
    roof = None
    pk = peaks()
    if algo == 4:
        _, (visits_after, _) = a.bh_repulsion(theta)
        visits = 0.5 * (visits_before + visits_after)
        avg_s = kern_ms / max(kern_count, 1) / 1e3
        sm_mhz = (clocks or {}).get("sm_mhz") or (pk or {}).get("sm_max_mhz", 2070.0)
        roof = bh_roofline(g, kernel, args.workload, visits, avg_s, total_ms / args.steps / 1e3, sm_mhz, pk)
    elif algo == 5:
        # per first-phase iteration and vertex: rowptr (8 B), walk offsets
        # (16 B), own position (8 B), force write + read (32 B), position
        # write (8 B); per CSR entry: colid + neighbour position (12 B); per
        # walk pair: (source, count) + source position (16 B)
        off, _, _ = a.greedy_walks()
        npairs = float(off[-1])
        first = min(ips, int(ips * 0.8) + 1)  # walk-phase iterations per launch
        alg_bytes = first * (72.0 * g.n + 12.0 * g.nnz + 16.0 * npairs)
        avg_s = kern_ms / max(kern_count, 1) / 1e3
        achieved = alg_bytes / avg_s / 1e9
        peak = pk["hbm_gbs"] if pk else 6800.0
        roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic_from_profile(kernel, args.workload), "kernel": kernel,
                "kernel_ms_per_launch": avg_s * 1e3, "launches": kern_count,
                "algorithmic_bytes_per_launch": alg_bytes, "walk_pairs": npairs,
                "iterations_per_launch": first,
                "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if pk else "fallback",
                "note": "one cluster runs the batches in sequence, one cluster barrier per batch; "
                        "positions stay in L2, so the kernel is bound by barrier and gather latency"}
    else:
        pairs = float(g.n) * g.n
        avg_s = kern_ms / max(kern_count, 1) / 1e3
        achieved = 10.0 * pairs / avg_s / 1e12
        sm_mhz = (clocks or {}).get("sm_max_mhz") or (pk or {}).get("sm_max_mhz", 2070.0)
        peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
        roof = {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                "traffic": traffic_from_profile(kernel, args.workload), "kernel": kernel,
                "kernel_ms_per_launch": avg_s * 1e3, "launches": kern_count,
                "algorithmic_flops_per_launch": 10.0 * pairs,
                "peak_source": "nominal FP32 FMA peak: 152 SMs x 128 lanes x 2 flops x max SM clock"}

    tte = None
    if algo == 4 and rank == 0 and not args.no_learned:
        tte = time_to_energy(B, g, w)
    allpairs = None
    if algo == 4 and rank == 0 and not args.no_allpairs:
        allpairs = allpairs_fraction(B, torch, device, flush)

    # end to end through the C ABI with pinned host buffers: every step copies
    # its input coordinates in and its result out (the two buffers take turns)
    a.set_graph_mode(True)  # the library's default mode
    host = [torch.empty((g.n, 2), dtype=torch.float64, pin_memory=True) for _ in range(2)]
    host[0].copy_(torch.from_numpy(a.nCoordinates))
    e2e_steps = max(3, min(args.steps, 10))
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        a.set_coordinates_ptr(host[k & 1].data_ptr())
        if algo == 4:
            a.barnes_hut_iteration(batch, theta, step)
        elif algo == 5:
            a.run_resident(algo, ips, batch, theta, step)
        else:
            a.minibatch_iteration(algo, batch, step)
        a.get_coordinates_ptr(host[(k + 1) & 1].data_ptr())
    e2e_s = time.perf_counter() - t0
    e2e = {"value": ws * g.n * ips * e2e_steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 16 * g.n,
           "d2h_bytes_per_step": 16 * g.n + 8, "steps": e2e_steps}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(args, w, g),
            "parallelism": "replicas" if ws > 1 else "single GPU",
            "step_launch": (f"replay of the captured iteration, a CUDA graph of its {launches // args.steps} "
                            "kernel launches") if graph else "direct launches",
            "e2e": e2e, "gpu_launches": launches, "roofline": roof, "cpu_baseline": cpu, "clocks": clocks,
            "time_to_energy": tte, "allpairs_chunglu100k": allpairs,
        }
        print(json.dumps(line), flush=True)
    a.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
