"""Benchmark: GPU BVH build throughput (Mtris/s) and HBM-roofline fraction on one GB300.

Default workload: 10,000,000 clustered triangles (64 Gaussian clusters, sigma 0.02, edges
logU[1e-4,1e-2], seed 1), LBVH with 63-bit Morton codes.  One step = one full build from
device-resident SoA input to device-resident BVHNode output.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

Inputs (360 MB of vertices, plus ~2 GB of workspace written per build) are larger than the
129 MB L2, so no explicit flush is done between steps.  Under torchrun each rank builds its own
replica (the single-mesh build does not shard).
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

PEAKS_PATH = os.path.join(ROOT, "MEASURED_PEAKS.json")
METRIC = "build Mtris/s (device-resident) + %HBM roofline; batched vs plain; serve p50/p99 ms"
FALLBACK_HBM = 6800.0

WORKLOADS = {
    # name: (generator, kwargs, algo, morton_bits, radius, description)
    "c1_lbvh63": ("clustered", {"n": 10_000_000, "seed": 1}, "lbvh", 63, 0,
                  "10M clustered triangles, LBVH 63-bit Morton"),
    "c1_lbvh30": ("clustered", {"n": 10_000_000, "seed": 1}, "lbvh", 30, 0,
                  "10M clustered triangles, LBVH 30-bit Morton"),
    "c1_ploc25": ("clustered", {"n": 10_000_000, "seed": 1}, "ploc", 30, 25,
                  "10M clustered triangles, PLOC radius 25"),
    "c1_lbvhplus": ("clustered", {"n": 10_000_000, "seed": 1}, "lbvh_plus", 60, 0,
                    "10M clustered triangles, LBVH+ 60-bit, 1 treelet pass"),
    "c1_lbvhplus3": ("clustered", {"n": 10_000_000, "seed": 1}, "lbvh_plus", 60, 0,
                     "10M clustered triangles, LBVH+ 60-bit, 3 treelet passes"),
    "c1_lbvh63_4m": ("clustered", {"n": 4_000_000, "seed": 1}, "lbvh", 63, 0,
                     "4M clustered triangles (config 1 distribution), LBVH 63-bit; profiling size"),
    "c1_lbvhplus_2m": ("clustered", {"n": 2_000_000, "seed": 1}, "lbvh_plus", 60, 0,
                       "2M clustered triangles (config 1 distribution), LBVH+ 60-bit, 1 pass; profiling size"),
    "c1_ploc25_2m": ("clustered", {"n": 2_000_000, "seed": 1}, "ploc", 30, 25,
                     "2M clustered triangles (config 1 distribution), PLOC radius 25; profiling size"),
    "c2a_ploc25": ("icosphere", {"levels": 8, "seed": 2}, "ploc", 30, 25,
                   "1,310,720-triangle displaced icosphere (0.05 fBm), PLOC radius 25"),
    "c2a_lbvhplus": ("icosphere", {"levels": 8, "seed": 2}, "lbvh_plus", 60, 0,
                     "1,310,720-triangle displaced icosphere (0.05 fBm), LBVH+ 60-bit, 1 treelet pass"),
    "c2b_ploc25": ("strands", {"n_strands": 20000, "segments": 100, "seed": 3}, "ploc", 30, 25,
                   "2,000,000 thin triangles on 20,000 random-walk strands, PLOC radius 25"),
    "c2a_ploc10": ("icosphere", {"levels": 8, "seed": 2}, "ploc", 30, 10,
                   "1,310,720-triangle displaced icosphere (0.05 fBm), PLOC radius 10"),
    "c2a_ploc100": ("icosphere", {"levels": 8, "seed": 2}, "ploc", 30, 100,
                    "1,310,720-triangle displaced icosphere (0.05 fBm), PLOC radius 100"),
    "c2b_ploc10": ("strands", {"n_strands": 20000, "segments": 100, "seed": 3}, "ploc", 30, 10,
                   "2,000,000 thin triangles on 20,000 random-walk strands, PLOC radius 10"),
    "c2b_ploc100": ("strands", {"n_strands": 20000, "segments": 100, "seed": 3}, "ploc", 30, 100,
                    "2,000,000 thin triangles on 20,000 random-walk strands, PLOC radius 100"),
    "c2b_lbvhplus": ("strands", {"n_strands": 20000, "segments": 100, "seed": 3}, "lbvh_plus", 60, 0,
                     "2,000,000 thin triangles on 20,000 random-walk strands, LBVH+ 60-bit, 1 treelet pass"),
    "c3_batched": ("batch", {"meshes": 4096, "lo": 64, "hi": 262144}, "lbvh_batched", 30, 0,
                   "4,096 meshes, triangle counts logU[64, 262144], each built by LBVH-30 in one batched launch "
                   "sequence replayed as a CUDA graph"),
    "c3_batched_ploc25": ("batch", {"meshes": 4096, "lo": 64, "hi": 262144}, "ploc_batched", 30, 25,
                          "4,096 meshes, triangle counts logU[64, 262144], each built by PLOC r=25 in one batched "
                          "build (one CUDA graph launch: keys, sort, clustering loop as a conditional node)"),
    "c4_serve": ("serve", {"rate": 2000.0, "duration_s": 3.0, "lo": 1000, "hi": 2_000_000, "rays": 65536,
                           "pool": 32, "budget_gb": 40, "slots": 16}, "serve", 30, 0,
                 "Poisson stream (2,000 req/s) of build+trace requests, meshes logU[1e3, 2e6] triangles, "
                 "65,536 rays each, 40 GB HBM budget"),
    "c4_serve_batched": ("serve", {"rate": 2000.0, "duration_s": 3.0, "lo": 1000, "hi": 2_000_000, "rays": 65536,
                                   "pool": 32, "budget_gb": 40, "slots": 8}, "serve_batched", 30, 0,
                         "config 4's stream served in batched ticks: every waiting request that fits joins one "
                         "gather + batched LBVH build + traversal + scatter launch sequence"),
    "c0_lbvh30": ("uniform_small", {"n": 100_000, "seed": 0}, "lbvh", 30, 0,
                  "100k uniform triangles, LBVH 30-bit"),
}
# LBVH+ treelet passes per workload (1 where not listed: the reference's own count)
TREELET_ROUNDS = {"c1_lbvhplus3": 3}


def treelet_rounds(name: str) -> int:
    return TREELET_ROUNDS.get(name, 1) if WORKLOADS[name][2] == "lbvh_plus" else 0


def bytes_per_tri(algo: str, bits: int, rounds: int = 0, cluster_sum_per_tri: float = 0.0) -> float:
    """Algorithmic HBM bytes per triangle of a whole build.  LBVH: B(K) = 276 + 3kb + 2D(kb+4)
    with D = ceil(K/8) 8-bit digits (the bytes an 8-bit LSD sort of the whole key moves; the
    library's 64-bit sort moves fewer, so B(K) is a property of the problem, not of this
    implementation).  LBVH+: B(60) + 144 per treelet pass.  PLOC: 264 + 160 * (live clusters
    summed over iterations) / n."""
    if algo == "ploc":
        return 264.0 + 160.0 * cluster_sum_per_tri
    kb = 4 if bits == 30 else 8
    d = (bits + 7) // 8
    b = 276 + 3 * kb + 2 * d * (kb + 4)
    return b + 144.0 * rounds if algo == "lbvh_plus" else b


def stage_bytes_per_tri(stage: str, algo: str, bits: int, rounds: int = 0, cluster_sum_per_tri: float = 0.0):
    """Algorithmic bytes per triangle of one build stage: the split of B(K) above, except that the
    Morton stage also counts the 32-byte triangle box it writes for the emission's gather (B(K)
    counts that gather as 36 bytes of vertices inside the emission stage, as this split does too),
    so the LBVH stages sum to B(K) + 32."""
    kb = 4 if bits == 30 else 8
    d = (bits + 7) // 8
    if stage == "scene_bounds":
        return 36.0
    if stage == "morton_boxes_hist":
        return 36.0 + kb + 4 + 32.0
    # 60/63-bit codes: the run fix-up at the end of the sort stage also writes the delta bytes, so
    # the delta's key read and byte write (kb + 1) move from the emission stage to the sort stage
    delta = kb + 1 if bits != 30 and algo != "ploc" else 0
    if stage == "onesweep_sort":
        return kb + 2.0 * d * (kb + 4) + delta
    if stage == "emit_refit":  # PLOC: leaf nodes + cluster init in this slot
        return 116.0 if algo == "ploc" else kb + 4 + 36 + 48 + 12 + 48 + 4 + 48 - delta
    if algo == "ploc":
        return 160.0 * cluster_sum_per_tri
    return 144.0 * rounds


def impl_stage_bytes_per_tri(stage: str, algo: str, bits: int, rounds: int = 0,
                             cluster_sum_per_tri: float = 0.0) -> float:
    """Bytes per triangle this implementation moves in a stage (its own buffers, not the problem's
    B(K) split): bounds 36 read; Morton 36 read + 4 key + (60/63-bit: 4 low bits) + 32 box
    written; sort: 4 passes over 32-bit (key, index) pairs, 12 B in the first (no index read) and
    16 B in each other, + for 60/63-bit codes the run fix-up's 8 B read, 1 B delta write and about
    4 B of low-bit gathers and index moves; emission: 4 index + 32 box gathered + 48 leaf + 48
    internal node + 1 delta (30-bit: 4 key read, the delta bytes stay in shared memory).  Stages
    this accounting does not split (the treelet pass, the PLOC loop and its cluster init) report
    their algorithmic bytes."""
    split = bits != 30 and algo != "ploc"
    if stage == "scene_bounds":
        return 36.0
    if stage == "morton_boxes_hist":
        return 36.0 + 4 + (4 if split else 0) + 32.0
    if stage == "onesweep_sort":
        return 12.0 + 3 * 16.0 + (13.0 if split else 0.0)
    if stage == "emit_refit" and algo != "ploc":
        return 4.0 + 32 + 48 + 48 + (1.0 if split else 4.0)
    return stage_bytes_per_tri(stage, algo, bits, rounds, cluster_sum_per_tri)


def kernels_per_build(algo: str, bits: int, rounds: int = 0, ploc_iterations: int = 0, tree_height: int = 0) -> int:
    """Launches of this library's kernels in one build: bounds, Morton, 4 onesweep passes, the run
    fix-up of 60/63-bit codes (short runs, listed long runs; it writes the delta bytes too),
    emission (which computes the delta bytes of 30-bit codes) + frontier climb;
    per treelet pass five (heights, counts, offsets, grouping by height, the fallback check) plus
    growth, DP and loop control per tree level; PLOC adds cluster init, 4 per clustering iteration
    launched one kernel per phase (neighbours, tile counts + scan, merge + compaction, loop
    control) and the root fix
    (its 30-bit prefix stops after the sort).  A PLOC build reports its exact count itself (some
    iterations run inside its middle-iterations and tail kernels); this is the count when every
    iteration is launched per phase."""
    if algo == "ploc":
        return 2 + 4 + 1 + 4 * ploc_iterations + 1
    n = 2 + 4 + (2 if bits != 30 else 0) + 2
    return n + (rounds * (5 + 3 * tree_height) if algo == "lbvh_plus" else 0)


def batched_kernels_per_build(meshes: int, ploc_iterations: int = -1) -> int:
    """Launches in one batched build: per-mesh box init, bounds and Morton, ceil(K/8) onesweep
    passes over the K = 30 + mesh-bits keys (4 when K > 32, followed by the two run fix-up
    kernels), then LBVH: delta + emission + frontier climb; PLOC (ploc_iterations >= 0): leaf and
    cluster init, 5 per iteration (neighbours, tile counts + scan, per-mesh ranks, merge +
    compaction, loop control) and the per-mesh root fix."""
    mbits = 1
    while mbits < 34 and (1 << mbits) < meshes:
        mbits += 1
    kbits = 30 + mbits
    passes = 4 if kbits > 32 else (kbits + 7) // 8
    prefix = 3 + passes + (2 if kbits > 32 else 0)
    if ploc_iterations >= 0:
        return prefix + 1 + 5 * ploc_iterations + 1
    return prefix + 3


STAGE_KERNELS = {
    "scene_bounds": "k_bounds",
    "morton_boxes_hist": "k_morton",
    "onesweep_sort": "k_onesweep x4 (+ k_fixrun_split_short/_long for 60/63-bit codes)",
    "emit_refit": "k_emit (with the delta bytes of 30-bit codes) + k_emit_climb",
    "treelet_or_ploc_loop": "LBVH+: k_tl_heights, k_tl_count, k_tl_offsets, k_tl_scatter, then k_tl_grow +"
                            " k_tl_dp per tree height; PLOC: k_ploc_nn, k_ploc_count, k_ploc_scatter, k_ploc_step"
                            " per iteration + k_ploc_root",
}

# DRAM bytes per triangle (dram__bytes_read.sum + dram__bytes_write.sum over the stage's kernels)
# from one ncu capture of a smaller case of the same distribution, whose buffers exceed the L2;
# the stage's traffic grows with the triangle count, so a launch over n triangles moves about
# n times this.  Keyed by (algorithm, Morton bits, stage).
MEASURED_TRAFFIC_PER_TRI = {
    ("lbvh", 63, "emit_refit"): (191.6, "one ncu capture of k_emit + k_emit_climb on 4M triangles of the same "
                                        "distribution: 766 MB / 4M triangles, scaled by the triangle count"),
}


def hbm_peak():
    try:
        with open(PEAKS_PATH) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 20 ms for as long as the sampler is
    open; each sample is stamped with the host clock when it arrives, so any window (the timed
    region, or the whole measurement phase around it) can be summarised afterwards."""

    PERIOD_MS = 20

    def __init__(self, gpu_index: int = 0):
        self.gpu = gpu_index
        self.proc = None
        self.samples = []  # (host time, csv line)
        self.marks = {}

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", str(self.PERIOD_MS)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # measure only once nvidia-smi is producing samples (it takes a moment to start)
            t0 = time.perf_counter()
            while not self.samples and self.proc.poll() is None and time.perf_counter() - t0 < 3.0:
                time.sleep(0.01)
        except Exception:
            self.proc = None
        self.mark("open")
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append((time.perf_counter(), line.strip()))

    def mark(self, name):
        self.marks[name] = time.perf_counter()

    def __exit__(self, *a):
        self.mark("close")
        if self.proc:
            time.sleep(2.0 * self.PERIOD_MS / 1e3)  # the sample covering the last moments
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def _summarise(self, t0, t1):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ts, line in self.samples:
            if ts < t0 or ts > t1:
                continue
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return sm, mx, reasons

    def summary(self, start="timed_start", end="timed_end", fallback=("open", "close"), min_samples=3):
        """Median SM clock, its maximum and the throttle reasons seen between two marks.  With
        fewer than min_samples there (a short timed region), the fallback window -- the whole
        phase of identical builds around it -- is summarised instead and named in `window`."""
        t0, t1 = self.marks.get(start, 0.0), self.marks.get(end, 0.0)
        sm, mx, reasons = self._summarise(t0, t1 + self.PERIOD_MS / 1e3)
        window = "timed region"
        if len(sm) < min_samples and fallback:
            f0, f1 = self.marks.get(fallback[0], 0.0), self.marks.get(fallback[1], time.perf_counter())
            sm, mx, reasons = self._summarise(f0, f1 + self.PERIOD_MS / 1e3)
            window = (f"{fallback[0]}..{fallback[1]}: the timed region ({(t1 - t0) * 1e3:.0f} ms) and the "
                      f"warm-up and stage-timing builds around it ({(f1 - f0) * 1e3:.0f} ms in all)")
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0, "window": window}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm), "window": window, "period_ms": self.PERIOD_MS}


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def make_mesh(name):
    from bvh_gb300 import meshgen
    gen, kw, *_ = WORKLOADS[name]
    return getattr(meshgen, gen)(**kw)


def cpu_baseline(name, mesh, budget_s=12.0):
    """The CPU oracle (same algorithm, OpenMP on every host core) on a bounded sample."""
    from oracle import oracle as O
    _, _, algo, bits, radius, _ = WORKLOADS[name]
    n_sample = min(mesh.size(), 1_000_000)
    arrays = [a[:n_sample] for a in mesh.arrays()]
    cores = O.threads()
    t0 = time.perf_counter()
    reps = 0
    while True:
        if algo == "ploc":
            O.ploc(arrays, radius)
        elif algo == "lbvh_plus":
            O.lbvh_plus(arrays, bits, treelet_rounds(name))
        else:
            O.lbvh(arrays, bits)
        reps += 1
        if time.perf_counter() - t0 > budget_s or reps >= 20:
            break
    dt = (time.perf_counter() - t0) / reps
    out = {"value": round(n_sample / dt / 1e6, 3), "unit": "Mtris/s", "cores": cores, "kind": "port",
           "sample": f"first {n_sample:,} triangles of the workload, {reps} builds, oracle/bvh_oracle.c (OpenMP)"}
    # the same build on one thread (a smaller sample), and the host evaluator (SAH + depth
    # statistics, single-threaded as BVHEvaluator is) on an LBVH of the sample
    n1 = min(n_sample, 250_000)
    a1 = [a[:n1] for a in arrays]
    try:
        O.set_threads(1)
        t1 = time.perf_counter()
        if algo == "ploc":
            O.ploc(a1, radius)
        elif algo == "lbvh_plus":
            O.lbvh_plus(a1, bits, treelet_rounds(name))
        else:
            O.lbvh(a1, bits)
        dt1 = time.perf_counter() - t1
    finally:
        O.set_threads(cores)
    out["one_thread"] = {"value": round(n1 / dt1 / 1e6, 3), "unit": "Mtris/s", "cores": 1,
                         "sample": f"first {n1:,} triangles, 1 build"}
    nodes, _, _ = O.lbvh(arrays, 30)
    t2 = time.perf_counter()
    O.sah(nodes)
    O.depth_stats(nodes)
    dt2 = time.perf_counter() - t2
    out["evaluator"] = {"ms": round(dt2 * 1e3, 2), "nodes": int(nodes.shape[0]), "cores": 1,
                        "what": "SAH + depth statistics (the restatement of BVHEvaluator, pinned bit-equal to it) "
                                f"over an LBVH-30 of the first {n_sample:,} triangles"}
    return out


def run_ours(args):
    import torch
    import torch.distributed as dist

    import bvh_gb300
    from bvh_gb300 import _capi as C, meshgen

    ws, rank, local = dist_info()
    if ws > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    gen, kw, algo, bits, radius, desc = WORKLOADS[args.workload]
    mesh = make_mesh(args.workload)
    n = mesh.size()
    algo_id = {"lbvh": C.ALGO_LBVH, "lbvh_plus": C.ALGO_LBVH_PLUS, "ploc": C.ALGO_PLOC}[algo]
    ctx = bvh_gb300.Context(local)
    params = ctx.params(algo_id, morton_bits=bits, ploc_radius=radius or 25,
                        treelet_rounds=max(1, treelet_rounds(args.workload)),
                        host_loops=getattr(args, "host_loops", False))
    d_in = [torch.from_numpy(a).to(dev) for a in mesh.arrays()]
    ptrs = [t.data_ptr() for t in d_in]
    stream = torch.cuda.Stream(device=dev)
    s = stream.cuda_stream
    ctx.reserve(n, algo_id)
    # launch shapes for this algorithm and size (the tree is checked to stay the same); choices
    # that change the tree (radius, treelet passes, Morton bits) come back with their SAH
    tuning = None if args.no_autotune else ctx.autotune_build(ptrs, n, params, s)

    # --- device-resident build throughput -------------------------------------------------
    # The clock sampler runs through the warm-up, the timed region and the stage-timing builds
    # (all identical builds), so a short timed region still gets a clock record.
    with torch.cuda.stream(stream), ClockSampler(local) as clk:
        for _ in range(args.warmup):
            ctx.build_device(ptrs, n, params, s)
        ctx.sync()
        stages = []
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        if ws > 1:
            dist.barrier()
        clk.mark("timed_start")
        ev0.record(stream)
        for _ in range(args.steps):
            ctx.build_device(ptrs, n, params, s)
        ev1.record(stream)
        torch.cuda.synchronize(dev)
        clk.mark("timed_end")
        if ws > 1:
            dist.barrier()
        ctx.sync()
        # per-stage device times from the library's stage events, one build at a time
        for _ in range(min(args.steps, 10)):
            tree = ctx.build_device(ptrs, n, params, s)
            t = ctx.last_timing()
            stages.append((t.bounds_ms, t.morton_ms, t.sort_ms, t.emit_ms, t.optimize_ms, t.total_ms))
            ploc_iters, ploc_csum = int(t.ploc_iterations), int(t.ploc_cluster_sum)
            build_launches = int(t.kernel_launches)
            tree_height = int(t.tree_height)
        # a short timed region gets few clock samples: keep building (untimed, the same build)
        # until the sampled window around it spans at least 150 ms
        while time.perf_counter() - clk.marks["open"] < 0.15:
            for _ in range(8):
                ctx.build_device(ptrs, n, params, s)
            torch.cuda.synchronize(dev)
    elapsed_ms = ev0.elapsed_time(ev1)
    if ws > 1:
        tt = torch.tensor([elapsed_ms], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        elapsed_ms = float(tt.item())
    ms_per_step = elapsed_ms / args.steps
    value = n * args.steps * ws / (elapsed_ms / 1e3) / 1e6

    st = np.array(stages, np.float64)
    med = np.median(st, axis=0)
    peak, peak_kind = hbm_peak()
    rounds = treelet_rounds(args.workload)
    csum = ploc_csum / n if algo == "ploc" else 0.0
    # dominant stage: the largest share of device time (stage events on the launching stream)
    shares = {"scene_bounds": med[0], "morton_boxes_hist": med[1], "onesweep_sort": med[2], "emit_refit": med[3],
              "treelet_or_ploc_loop": med[4]}
    dom = max(shares, key=shares.get)
    per_unit = stage_bytes_per_tri(dom, algo, bits, rounds, csum)
    achieved = per_unit * n / (shares[dom] / 1e3) / 1e9
    whole = bytes_per_tri(algo, bits, rounds, csum)
    build_gbs = whole * n / (med[5] / 1e3) / 1e9
    kernels = "k_ploc_init" if (algo == "ploc" and dom == "emit_refit") else STAGE_KERNELS[dom]
    measured = MEASURED_TRAFFIC_PER_TRI.get((algo, bits, dom))
    traffic = round(measured[0] * n) if measured else None
    roofline = {"bound": "hbm", "kernel": dom, "kernels": kernels, "achieved": round(achieved, 1),
                "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic,
                "traffic_source": measured[1] if measured else "no capture of this stage at this workload",
                "peak_kind": f"of {peak_kind}", "algorithmic_bytes_per_tri": round(per_unit, 2),
                "whole_build": {"bytes_per_tri": round(whole, 2), "achieved": round(build_gbs, 1),
                                "frac": round(build_gbs / peak, 4), "median_build_ms": round(med[5], 4)},
                # secondary: the compulsory input and output alone (36 B in, 2 x 48 B nodes, 4 B index)
                "io_floor": {"bytes_per_tri": 136, "achieved": round(136.0 * n / (med[5] / 1e3) / 1e9, 1),
                             "frac": round(136.0 * n / (med[5] / 1e3) / 1e9 / peak, 4)}}
    if algo == "ploc":
        roofline["ploc"] = {"iterations": ploc_iters, "cluster_sum": ploc_csum}
    # every stage against the measured peak, in the problem's bytes and in the bytes this
    # implementation moves
    roofline["stages"] = {}
    for k, ms in shares.items():
        if ms <= 0.005:
            continue
        alg = stage_bytes_per_tri(k, algo, bits, rounds, csum)
        imp = impl_stage_bytes_per_tri(k, algo, bits, rounds, csum)
        roofline["stages"][k] = {"ms": round(ms, 4), "algorithmic_bytes_per_tri": round(alg, 2),
                                 "frac_algorithmic": round(alg * n / (ms / 1e3) / 1e9 / peak, 4),
                                 "implementation_bytes_per_tri": round(imp, 2),
                                 "frac_implementation": round(imp * n / (ms / 1e3) / 1e9 / peak, 4)}
    stage_ms = {k: round(v, 4) for k, v in shares.items()}

    # --- tree quality: evaluator statistics on the GPU, 1920x1080 pinhole primary rays -----
    quality = None
    with torch.cuda.stream(stream):
        quality = ctx.evaluate(tree.nodes, tree.n_nodes, s)
        root = np.zeros(1, C.NODE_DTYPE)
        xs, ys, zs = mesh.arrays()[0::3], mesh.arrays()[1::3], mesh.arrays()[2::3]
        root["min"][0] = [min(a.min() for a in xs), min(a.min() for a in ys), min(a.min() for a in zs)]
        root["max"][0] = [max(a.max() for a in xs), max(a.max() for a in ys), max(a.max() for a in zs)]
        cam = bvh_gb300.auto_camera(root[0])
        W, Hh = 1920, 1080
        hits = [torch.empty(W * Hh, dtype=torch.float32, device=dev)] + \
               [torch.empty(W * Hh, dtype=torch.int32, device=dev) for _ in range(4)]
        hp = [h.data_ptr() for h in hits]
        ctx.trace_pinhole(tree.nodes, tree.n_nodes, ptrs, n, cam, W, Hh, hp, s)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(3):
            ctx.trace_pinhole(tree.nodes, tree.n_nodes, ptrs, n, cam, W, Hh, hp, s)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        tr_ms = e0.elapsed_time(e1) / 3
        quality.update({"pinhole_rays": W * Hh, "avg_nodes_visited": round(float(hits[2].double().mean()), 3),
                        "hit_fraction": round(float((hits[1] >= 0).double().mean()), 4),
                        "trace_ms": round(tr_ms, 3), "trace_mrays_per_s": round(W * Hh / (tr_ms / 1e3) / 1e6, 1)})
        quality["sah"] = round(quality["sah"], 3)
        quality["avg_leaf_depth"] = round(quality["avg_leaf_depth"], 3)
        if gen in ("icosphere", "strands"):
            # surface-like meshes: 1M rays from a sphere around the mesh toward points in its box
            ro, rd = meshgen.sphere_rays(mesh, 1_000_000, seed=7)
            nr = ro.shape[0]
            rays = [torch.from_numpy(np.ascontiguousarray(a)).to(dev)
                    for a in (ro[:, 0], ro[:, 1], ro[:, 2], rd[:, 0], rd[:, 1], rd[:, 2])]
            sh = [torch.empty(nr, dtype=torch.float32, device=dev)] + \
                 [torch.empty(nr, dtype=torch.int32, device=dev) for _ in range(4)]
            rp, shp = [r.data_ptr() for r in rays], [h.data_ptr() for h in sh]
            ctx.trace(tree.nodes, tree.n_nodes, ptrs, n, rp, nr, shp, s)
            e0.record(stream)
            for _ in range(3):
                ctx.trace(tree.nodes, tree.n_nodes, ptrs, n, rp, nr, shp, s)
            e1.record(stream)
            torch.cuda.synchronize(dev)
            sr_ms = e0.elapsed_time(e1) / 3
            quality["sphere_rays"] = {"rays": nr, "avg_nodes_visited": round(float(sh[2].double().mean()), 3),
                                      "hit_fraction": round(float((sh[1] >= 0).double().mean()), 4),
                                      "trace_ms": round(sr_ms, 3),
                                      "trace_mrays_per_s": round(nr / (sr_ms / 1e3) / 1e6, 1)}

    # --- end to end through the C ABI with pinned host buffers ----------------------------
    h_in = [torch.from_numpy(a).pin_memory() for a in mesh.arrays()]
    m_host = C.mesh_struct([t.data_ptr() for t in h_in], n)
    h_nodes = torch.empty((2 * n - 1) * 48, dtype=torch.uint8).pin_memory()
    h_idx = torch.empty(n * 4, dtype=torch.uint8).pin_memory()
    import ctypes
    nn = ctypes.c_uint32(0)
    lib = ctx.lib

    def e2e_once():
        rc = lib.bvh_build_host(ctx.handle, ctypes.byref(m_host), ctypes.byref(params), ctypes.c_void_p(s),
                                ctypes.c_void_p(h_nodes.data_ptr()), ctypes.c_void_p(h_idx.data_ptr()),
                                ctypes.byref(nn))
        C.check(rc, "bvh_build_host")

    for _ in range(max(1, args.warmup)):
        e2e_once()
    e2e_steps = max(1, min(args.steps, 10))
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_once()
    torch.cuda.synchronize(dev)
    e2e_ms = (time.perf_counter() - t0) * 1e3 / e2e_steps
    e2e = {"value": round(n * ws / (e2e_ms / 1e3) / 1e6, 2), "unit": "Mtris/s", "h2d_bytes_per_step": 36 * n,
           "d2h_bytes_per_step": 48 * (2 * n - 1) + 4 * n, "ms_per_step": round(e2e_ms, 3),
           "host_memory": "pinned (page-locked) input and output buffers"}
    extras = {}
    if args.workload == "c1_lbvh63" and not args.no_extras and ws == 1:
        # the same call on ordinary pageable memory: what the BVHBuilder adapter hands over
        # (std::vector / numpy arrays), so the speed-up a drop-in caller gets
        p_in = mesh.arrays()
        m_page = C.mesh_struct([a.ctypes.data for a in p_in], n)
        p_nodes = np.empty((2 * n - 1) * 48, np.uint8)
        p_idx = np.empty(n, np.uint32)

        def e2e_pageable_once():
            C.check(lib.bvh_build_host(ctx.handle, ctypes.byref(m_page), ctypes.byref(params), ctypes.c_void_p(s),
                                       ctypes.c_void_p(p_nodes.ctypes.data), ctypes.c_void_p(p_idx.ctypes.data),
                                       ctypes.byref(nn)), "bvh_build_host")

        e2e_pageable_once()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            e2e_pageable_once()
        torch.cuda.synchronize(dev)
        pg_ms = (time.perf_counter() - t0) * 1e3 / e2e_steps
        extras["e2e_pageable"] = {"value": round(n / (pg_ms / 1e3) / 1e6, 2), "unit": "Mtris/s",
                                  "ms_per_step": round(pg_ms, 3), "steps": e2e_steps,
                                  "h2d_bytes_per_step": 36 * n, "d2h_bytes_per_step": 48 * (2 * n - 1) + 4 * n,
                                  "host_memory": "pageable numpy arrays (as a std::vector-backed TriangleMesh)"}
        # the same mesh with the reference LBVH's own 30-bit codes: the same-configuration number
        p30 = ctx.params(C.ALGO_LBVH, morton_bits=30)
        with torch.cuda.stream(stream):
            for _ in range(args.warmup):
                ctx.build_device(ptrs, n, p30, s)
            torch.cuda.synchronize(dev)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(args.steps):
                ctx.build_device(ptrs, n, p30, s)
            e1.record(stream)
            torch.cuda.synchronize(dev)
        ms30 = e0.elapsed_time(e1) / args.steps
        extras["lbvh30"] = {"value": round(n / (ms30 / 1e3) / 1e6, 2), "unit": "Mtris/s",
                            "ms_per_step": round(ms30, 4), "steps": args.steps,
                            "what": "the same 10M mesh, LBVH with 30-bit Morton codes (the configuration of the "
                                    "reference's LBVHBuilderCUDA, which the reference arm times)"}

    # parity of the timed result against the oracle is covered by tests; record SAH here
    line = {
        "metric": METRIC,
        "value": round(value, 2), "unit": "Mtris/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms_per_step, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+u64", "data": "synthetic (seeded generator, bvh_gb300/meshgen.py)",
        "config": {"workload": args.workload, "description": desc, "triangles": n, "algorithm": algo,
                   "morton_bits": bits, "ploc_radius": radius or None, "parallelism": f"replicas x{ws}",
                   "l2": "inputs (360 MB) and per-build writes exceed the 129 MB L2; no flush"},
        "stage_ms_median": stage_ms,
        "quality": quality,
        "roofline": roofline,
        "e2e": e2e,
        # PLOC's and LBVH+'s loops run on the device: those builds report their own launches
        "gpu_launches": args.steps * (build_launches if algo in ("ploc", "lbvh_plus") and build_launches > 0
                                      else kernels_per_build(algo, bits, rounds, ploc_iters, tree_height)),
        "clocks": clk.summary(),
        "autotune": tuning,
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.workload, mesh)
    ctx.close()
    if extras:
        line.update(extras)
        del d_in, h_in, h_nodes, h_idx
        torch.cuda.empty_cache()
        # the metric's other halves: batched vs plain at equal trees (config 3), serving p50/p99
        # (config 4, a shortened stream), each a measurement of its own
        line["batched"] = measure_batched(max(3, min(args.steps, 10)), args.warmup, local, rank,
                                          autotune=not args.no_autotune)
        line["batched_ploc"] = measure_batched(3, args.warmup, local, rank, autotune=False, algo="ploc", radius=25)
        line["serve"] = measure_serve(1.0, local, rank)
        for k in ("latencies_ms", "span_s", "tris", "rays"):
            line["serve"].pop(k)
        line["serve"]["mode"] = "per-request slots (16 streams, one build + trace per request)"
        line["serve_batched"] = measure_serve(1.0, local, rank, batched=True, slots=8, batch_requests=8)
        for k in ("latencies_ms", "span_s", "tris", "rays"):
            line["serve_batched"].pop(k)
        line["serve_batched"]["mode"] = ("batched ticks (8 slots, up to 8 requests per batch; each batch: one "
                                         "gather, one batched LBVH build, one traversal launch, one scatter)")
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()


def measure_batched(steps, warmup, local=0, rank=0, autotune=True, algo="lbvh", radius=25, check_meshes=16,
                    world=1, barrier=None):
    """Config 3: 4,096 meshes (counts logU[64, 262144]) in one batched, graph-replayed build vs a
    per-mesh loop of single builds on the same GPU and the same device-resident data.  Also checks
    that sampled meshes' trees equal their single builds bit for bit.  With world > 1 ranks the
    batch has 4,096 x world meshes, shared out by shard.assign (balanced by triangle count, no
    collective on the data path); this rank builds its share, and `barrier` brackets the timed
    region."""
    import ctypes
    import torch

    import bvh_gb300
    from bvh_gb300 import _capi as C
    from bvh_gb300 import meshgen, shard

    dev = torch.device("cuda", local)
    kw = WORKLOADS["c3_batched"][1]
    if world > 1:
        all_counts = meshgen.batch_counts(kw["meshes"] * world, kw["lo"], kw["hi"], seed=4)
        mine = shard.assign(all_counts, world)[rank]
        counts = all_counts[mine]
        mesh, offsets = meshgen.batch_subset(all_counts, mine, seed=5)
    else:
        counts = meshgen.batch_counts(kw["meshes"], kw["lo"], kw["hi"], seed=4)
        mesh, offsets = meshgen.batch(counts, seed=5)
    n = mesh.size()
    count = offsets.shape[0] - 1
    ctx = bvh_gb300.Context(local)
    algo_id = C.ALGO_PLOC if algo == "ploc" else C.ALGO_LBVH
    params = ctx.params(algo_id, ploc_radius=radius)
    tuning = ctx.autotune(min(n, 1 << 26)) if autotune else None
    d_in = [torch.from_numpy(a).to(dev) for a in mesh.arrays()]
    ptrs = [t.data_ptr() for t in d_in]
    stream = torch.cuda.Stream(device=dev)
    s = stream.cuda_stream
    with torch.cuda.stream(stream), ClockSampler(local) as clk:
        for _ in range(warmup):
            ctx.build_batched(ptrs, offsets, params, s, use_graph=True)
        ctx.sync()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        if barrier:
            barrier()
        clk.mark("timed_start")
        ev0.record(stream)
        for _ in range(steps):
            ctx.build_batched(ptrs, offsets, params, s, use_graph=True)
        ev1.record(stream)
        torch.cuda.synchronize(dev)
        clk.mark("timed_end")
        if barrier:
            barrier()
        ms = ev0.elapsed_time(ev1) / steps
        # stage breakdown without the graph
        tree = ctx.build_batched(ptrs, offsets, params, s, use_graph=False)
        t = ctx.last_timing()
        iters, csum = int(t.ploc_iterations), int(t.ploc_cluster_sum)
        stages = {"seg_bounds": round(t.bounds_ms, 4), "seg_morton_hist": round(t.morton_ms, 4),
                  "onesweep_sort": round(t.sort_ms, 4), "delta_emit_refit": round(t.emit_ms, 4),
                  "ploc_loop": round(t.optimize_ms, 4)}
        # plain per-mesh loop of single-mesh builds on the same device-resident data
        single = bvh_gb300.Context(local)
        single.reserve(int(counts.max()), algo_id)
        single.set_tuning(ctx.tuning())
        loop_reps = 2
        for m in range(count):
            a = int(offsets[m])
            single.build_device([p + 4 * a for p in ptrs], int(counts[m]), params, s)
        torch.cuda.synchronize(dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(loop_reps):
            for m in range(count):
                a = int(offsets[m])
                single.build_device([p + 4 * a for p in ptrs], int(counts[m]), params, s)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        loop_ms = e0.elapsed_time(e1) / loop_reps
        # sampled meshes (the largest, the smallest, others spread over the batch) against their
        # single builds, bit for bit; each mesh's part of the batched tree is read back alone
        picks = sorted({int(np.argmax(counts)), int(np.argmin(counts))} |
                       {int(x) for x in np.linspace(0, count - 1, max(2, check_meshes - 2)).astype(int)})
        equal = True
        for m in picks:
            a, c = int(offsets[m]), int(counts[m])
            first = 2 * a - m
            sub = C.Tree()
            sub.nodes = tree.nodes + 48 * first
            sub.indices = tree.indices + 4 * a
            sub.n_nodes, sub.n_prims = 2 * c - 1, c
            bn = np.zeros(2 * c - 1, C.NODE_DTYPE)
            bi = np.zeros(c, np.uint32)
            C.check(ctx.lib.bvh_tree_download(ctx.handle, ctypes.byref(sub), ctypes.c_void_p(s),
                                              ctypes.c_void_p(bn.ctypes.data), ctypes.c_void_p(bi.ctypes.data)))
            one = single.build_device([p + 4 * a for p in ptrs], c, params, s)
            single.sync()
            sn, si = single.download(one, s)
            same = (np.array_equal(bi, si) and np.array_equal(bn["left"], sn["left"])
                    and np.array_equal(bn["right"], sn["right"])
                    and np.array_equal(bn["min"].view(np.uint32), sn["min"].view(np.uint32))
                    and np.array_equal(bn["max"].view(np.uint32), sn["max"].view(np.uint32)))
            equal = equal and same
        single.close()
    value = n / (ms / 1e3) / 1e6
    loop_value = n / (loop_ms / 1e3) / 1e6
    peak, peak_kind = hbm_peak()
    # 42-bit segmented keys (kb = 8, D = 6): LBVH B = 276 + 3*8 + 2*6*(8+4) = 444; PLOC: its prefix
    # with those keys (36 + 48 + 152) + leaf and cluster init 116 = 352, + 160 per live cluster
    # per iteration
    bpt = 444.0 if algo != "ploc" else 352.0 + 160.0 * csum / n
    # e2e: pinned host SoA -> device, batched build, nodes + indices back to pinned host memory
    h_in = [torch.from_numpy(a).pin_memory() for a in mesh.arrays()]
    n_nodes = 2 * n - count
    h_nodes = torch.empty(n_nodes * 48, dtype=torch.uint8).pin_memory()
    h_idx = torch.empty(n * 4, dtype=torch.uint8).pin_memory()
    e2e_steps = max(1, min(steps, 5))

    def e2e_once():
        with torch.cuda.stream(stream):
            for d, h in zip(d_in, h_in):
                d.copy_(h, non_blocking=True)
            tr = ctx.build_batched(ptrs, offsets, params, s, use_graph=True)
            C.check(ctx.lib.bvh_tree_download(ctx.handle, ctypes.byref(tr), ctypes.c_void_p(s),
                                              ctypes.c_void_p(h_nodes.data_ptr()), ctypes.c_void_p(h_idx.data_ptr())))

    e2e_once()
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_once()
    torch.cuda.synchronize(dev)
    e2e_ms = (time.perf_counter() - t0) * 1e3 / e2e_steps
    ctx.close()
    out = {"value": round(value, 2), "unit": "Mtris/s", "ms_per_step": round(ms, 4), "steps": steps,
           "meshes": count, "triangles": n, "min_mesh": int(counts.min()), "max_mesh": int(counts.max()),
           "algorithm": "PLOC r=%d" % radius if algo == "ploc" else "LBVH 30-bit",
           "per_mesh_loop": {"value": round(loop_value, 2), "unit": "Mtris/s", "ms_per_step": round(loop_ms, 3)},
           "speedup_batched_over_loop": round(value / loop_value, 2),
           "equal_to_single_builds": {"meshes_checked": len(picks), "all_equal": bool(equal)},
           "stage_ms": stages,
           "e2e": {"value": round(n / (e2e_ms / 1e3) / 1e6, 2), "unit": "Mtris/s", "h2d_bytes_per_step": 36 * n,
                   "d2h_bytes_per_step": 48 * n_nodes + 4 * n, "ms_per_step": round(e2e_ms, 3)},
           "gpu_launches": steps * batched_kernels_per_build(count, iters if algo == "ploc" else -1),
           "clocks": clk.summary(), "autotune": tuning}
    if algo == "ploc":
        out["ploc"] = {"iterations": iters, "cluster_sum": csum, "radius": radius}
    if bpt:
        achieved = bpt * n / (ms / 1e3) / 1e9
        out["algorithmic_bytes_per_tri"] = round(bpt, 2)
        out["roofline"] = {"bound": "hbm", "kernel": "whole batched build", "achieved": round(achieved, 1),
                           "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": None,
                           "peak_kind": f"of {peak_kind}", "algorithmic_bytes_per_tri": bpt}
    return out


def run_batched(args):
    """Config 3 as its own bench line.  Under torchrun: 4,096 meshes per rank, shared out by
    shard.assign; value = all ranks' triangles / the slowest rank's time."""
    import torch
    import torch.distributed as dist
    ws, rank, local = dist_info()
    torch.cuda.set_device(local)
    barrier = None
    if ws > 1:
        dist.init_process_group("nccl")
        barrier = dist.barrier
    gen, kw, algo, bits, radius, desc = WORKLOADS[args.workload]
    b = measure_batched(args.steps, args.warmup, local, rank, autotune=not args.no_autotune,
                        algo="ploc" if algo == "ploc_batched" else "lbvh", radius=radius or 25, world=ws,
                        barrier=barrier)
    ms, tris, meshes = b["ms_per_step"], b["triangles"], b["meshes"]
    if ws > 1:
        t = torch.tensor([ms], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        u = torch.tensor([tris, meshes], dtype=torch.float64, device="cuda")
        dist.all_reduce(u, op=dist.ReduceOp.SUM)
        tris, meshes = int(u[0].item()), int(u[1].item())
    line = {
        "metric": "batched build Mtris/s (device-resident) vs per-mesh loop",
        "value": round(tris / (ms / 1e3) / 1e6, 2), "unit": "Mtris/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+u64", "data": "synthetic (seeded generator, bvh_gb300/meshgen.py)",
        "config": {"workload": args.workload, "description": desc, "meshes": meshes, "triangles": tris,
                   "min_mesh": b["min_mesh"], "max_mesh": b["max_mesh"],
                   "parallelism": f"shards x{ws} (shard.assign: 4,096 meshes per rank, balanced by triangles)"
                   if ws > 1 else "1 GPU",
                   "l2": "inputs (4.8 GB) exceed the 129 MB L2; no flush"},
    }
    for k in ("per_mesh_loop", "speedup_batched_over_loop", "equal_to_single_builds", "stage_ms", "roofline",
              "e2e", "gpu_launches", "clocks", "autotune"):
        if k in b:
            line[k] = b[k]
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()


def measure_serve(duration_s=None, local=0, rank=0, world=1, barrier=None, **server_opts):
    """Config 4: a Poisson stream (2,000 req/s) of build+trace requests (meshes logU[1e3, 2e6]
    triangles from a pool of clustered and strand meshes, 65,536 rays each) through the server;
    p50/p90/p99 latency from submission to completion, aggregate Mtris/s and Mrays/s.  With
    world > 1 ranks the stream carries 2,000 x world req/s and shard.stream_share gives each rank
    its balanced share (no collective on the data path); `barrier` aligns the ranks' clocks."""
    import threading as th

    import torch

    from bvh_gb300 import meshgen, shard
    from bvh_gb300.serve import Server

    kw = dict(WORKLOADS["c4_serve"][1])
    if duration_s:
        kw["duration_s"] = duration_s
    g = np.random.default_rng(7)  # the same pool and stream on every rank
    sizes = np.exp(g.uniform(np.log(kw["lo"]), np.log(kw["hi"]), kw["pool"])).astype(np.int64)
    pool = []
    for k, n in enumerate(sizes):
        if k % 2:
            m = meshgen.strands(max(1, int(n) // 100), 100, seed=300 + k)
        else:
            m = meshgen.clustered(int(n), seed=300 + k)
        ro, rd = meshgen.sphere_rays(m, kw["rays"], seed=400 + k)
        mesh_h = [torch.from_numpy(a).pin_memory() for a in m.arrays()]
        rays_h = [torch.from_numpy(np.ascontiguousarray(x)).pin_memory()
                  for x in (ro[:, 0], ro[:, 1], ro[:, 2], rd[:, 0], rd[:, 1], rd[:, 2])]
        pool.append((m.size(), mesh_h, rays_h))
    nr = kw["rays"]
    free_hits = [[torch.empty(nr, dtype=torch.float32).pin_memory()] +
                 [torch.empty(nr, dtype=torch.int32).pin_memory() for _ in range(4)] for _ in range(512)]
    opts = dict(budget_bytes=kw["budget_gb"] << 30, slots=kw["slots"], morton_bits=30, device=local,
                max_triangles=int(max(p[0] for p in pool)), max_rays=nr)
    opts.update(server_opts)
    sv = Server(**opts)
    results = []
    in_use = {}
    lock = th.Lock()
    stop = th.Event()

    def poller():
        while not stop.is_set() or in_use:
            for r in sv.poll(256, 5):
                with lock:
                    free_hits.append(in_use.pop(r["tag"]))
                results.append(r)

    pt = th.Thread(target=poller, daemon=True)
    pt.start()

    def submit(tag, k):
        while True:
            with lock:
                if free_hits:
                    h = free_hits.pop()
                    in_use[tag] = h
                    break
            time.sleep(0.0001)
        n, mesh_h, rays_h = pool[k]
        sv.submit(tag, mesh_h, rays_h, h)

    # warm-up: every pool mesh once
    for k in range(len(pool)):
        submit(10_000_000 + k, k)
    while len(results) < len(pool):
        time.sleep(0.01)
    results.clear()
    n_all = int(kw["rate"] * world * kw["duration_s"])
    arrivals = np.cumsum(g.exponential(1.0 / (kw["rate"] * world), n_all))
    picks = g.integers(0, len(pool), n_all)
    mine = shard.stream_share(sizes[picks], world, rank) if world > 1 else np.arange(n_all)
    n_req = len(mine)
    if barrier:
        barrier()
    with ClockSampler(local) as clk:
        clk.mark("timed_start")
        t0 = time.perf_counter()
        for tag, q in enumerate(mine):
            delay = t0 + arrivals[q] - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            submit(tag, int(picks[q]))
        while len(results) < n_req:
            time.sleep(0.005)
        clk.mark("timed_end")
    stop.set()
    pt.join(timeout=10)
    st = sv.stats()
    sv.close()
    lat = np.array([(r["t_done_ns"] - r["t_submit_ns"]) / 1e6 for r in results])
    queue_ms = np.array([(r["t_admit_ns"] - r["t_submit_ns"]) / 1e6 for r in results])
    tris = sum(r["triangles"] for r in results)
    rays = sum(r["rays"] for r in results)
    span = (max(r["t_done_ns"] for r in results) - min(r["t_submit_ns"] for r in results)) / 1e9
    ok = all(r["status"] == 0 for r in results)
    return {
        "latencies_ms": lat, "span_s": span, "tris": tris, "rays": rays,
        "requests": n_req, "rate_per_s": kw["rate"], "duration_s": kw["duration_s"], "pool_meshes": len(pool),
        "slots": opts["slots"], "budget_gb": kw["budget_gb"], "rays_per_request": nr,
        "offered_mtris_per_s": round(float(np.mean(sizes)) * kw["rate"] / 1e6, 1),
        "latency_ms": {"p50": round(float(np.percentile(lat, 50)), 3), "p90": round(float(np.percentile(lat, 90)), 3),
                       "p99": round(float(np.percentile(lat, 99)), 3), "max": round(float(lat.max()), 3),
                       "mean": round(float(lat.mean()), 3),
                       "queue_p50": round(float(np.percentile(queue_ms, 50)), 3),
                       "queue_p99": round(float(np.percentile(queue_ms, 99)), 3)},
        "throughput": {"mtris_per_s": round(tris / span / 1e6, 1), "mrays_per_s": round(rays / span / 1e6, 1),
                       "requests_per_s": round(n_req / span, 1), "all_ok": ok},
        "server": {k: int(v) for k, v in st.items()},
        "e2e": {"value": round(tris / span / 1e6, 1), "unit": "Mtris/s",
                "h2d_bytes_per_step": int(np.mean([36 * pool[int(picks[q])][0] + 24 * nr for q in mine])),
                "d2h_bytes_per_step": 20 * nr},
        "clocks": clk.summary(),
    }


def run_serve(args):
    """Config 4 as its own bench line.  Under torchrun: 2,000 req/s per rank, the stream shared
    out by shard.stream_share; latencies are gathered from every rank."""
    import torch
    import torch.distributed as dist
    ws, rank, local = dist_info()
    torch.cuda.set_device(local)
    barrier = None
    if ws > 1:
        dist.init_process_group("nccl")
        barrier = dist.barrier
    gen, kw, algo, bits, radius, desc = WORKLOADS[args.workload]
    extra = dict(batched=True, batch_requests=8) if algo == "serve_batched" else {}
    r = measure_serve(None, local, rank, world=ws, barrier=barrier, slots=kw["slots"], **extra)
    if ws > 1:  # every rank's latencies and totals
        parts = [None] * ws
        dist.all_gather_object(parts, (list(r["latencies_ms"]), r["span_s"], r["tris"], r["rays"], r["requests"]))
        lat = np.concatenate([np.asarray(p[0]) for p in parts])
        span = max(p[1] for p in parts)
        r["latency_ms"].update({"p50": round(float(np.percentile(lat, 50)), 3),
                                "p90": round(float(np.percentile(lat, 90)), 3),
                                "p99": round(float(np.percentile(lat, 99)), 3), "max": round(float(lat.max()), 3),
                                "mean": round(float(lat.mean()), 3)})
        r["throughput"]["mtris_per_s"] = round(sum(p[2] for p in parts) / span / 1e6, 1)
        r["throughput"]["mrays_per_s"] = round(sum(p[3] for p in parts) / span / 1e6, 1)
        r["requests"] = sum(p[4] for p in parts)
        r["e2e"]["value"] = r["throughput"]["mtris_per_s"]
    line = {
        "metric": "serve p50/p99 request latency (ms) + aggregate Mtris/s and Mrays/s",
        "value": r["latency_ms"]["p50"], "unit": "ms (p50 latency)", "n_gpus": ws,
        "steps": r["requests"], "warmup": r["pool_meshes"], "ms_per_step": r["latency_ms"]["mean"],
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32+u32",
        "data": "synthetic (seeded pool of clustered/strand meshes, bvh_gb300/meshgen.py)",
        "config": {"workload": args.workload, "description": desc, "requests": r["requests"],
                   "rate_per_s": r["rate_per_s"], "pool_meshes": r["pool_meshes"], "slots": r["slots"],
                   "budget_gb": r["budget_gb"], "rays_per_request": r["rays_per_request"],
                   "offered_mtris_per_s": r["offered_mtris_per_s"],
                   "parallelism": f"shards x{ws} (shard.stream_share: 2,000 req/s per rank)" if ws > 1 else "1 GPU"},
        "latency_ms": r["latency_ms"], "throughput": r["throughput"], "server": r["server"], "e2e": r["e2e"],
        "gpu_launches": r["requests"] * 14, "clocks": r["clocks"],
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()


def run_reference_batched(args, ref, sample_meshes: int = 256):
    """Config 3 on the reference: it has no batched builder, so its LBVH builder runs once per
    mesh (the loop a BLAS build would need), on a bounded sample of the batch's meshes."""
    from bvh_gb300 import meshgen
    gen, kw, algo, bits, radius, desc = WORKLOADS[args.workload]
    counts = meshgen.batch_counts(kw["meshes"], kw["lo"], kw["hi"], seed=4)
    mesh, offsets = meshgen.batch(counts, seed=5)
    arrays = mesh.arrays()
    k = min(sample_meshes, counts.shape[0])
    parts = [[a[offsets[m]:offsets[m + 1]] for a in arrays] for m in range(k)]
    R = ref.RefRunner(fast=True)
    ploc = algo == "ploc_batched"

    def one(part):  # (getLastBuildTimeMS, wall ms of build())
        if ploc:
            _, _, _, ms, _ = R.ploc(part, radius)
            return float(ms[0]), float(ms[5])
        _, _, ms = R.lbvh(part)
        return float(ms[0]), float(ms[6])

    for m in range(min(8, k)):
        one(parts[m])
    tris = int(offsets[k])
    builds, walls = [], []
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            b = w = 0.0
            for m in range(k):
                bm, wm = one(parts[m])
                b += bm
                w += wm
            builds.append(b)
            walls.append(w)
    b = float(np.mean(builds))
    w = float(np.mean(walls))
    value = tris / (b / 1e3) / 1e6
    print(json.dumps({
        "impl": "reference", "metric": "batched build Mtris/s (device-resident) vs per-mesh loop",
        "value": round(value, 2), "unit": "Mtris/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(b, 3), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+u32", "data": "synthetic (seeded generator, bvh_gb300/meshgen.py)",
        "config": {"workload": args.workload, "description": desc, "meshes_sampled": k, "triangles_sampled": tris,
                   "reference_builder": (f"PLOCBuilderCUDA(r={radius})" if ploc else "LBVHBuilderCUDA (30-bit)")
                                        + " once per mesh: the reference has no batched builder",
                   "how": "the reference's own kernels (its .cu files compiled unmodified, Release flags) "
                          "replayed in its host order; value from the sum of its getLastBuildTimeMS"},
        "e2e": {"value": round(tris / (w / 1e3) / 1e6, 2), "unit": "Mtris/s", "h2d_bytes_per_step": 36 * tris,
                "d2h_bytes_per_step": 48 * (2 * tris - k) + 4 * tris, "ms_per_step": round(w, 3),
                "note": "wall time of the per-mesh build() calls: upload, kernels, download, AoS conversion"},
        "cpu_baseline": {"value": round(value, 2), "unit": "Mtris/s", "cores": 1, "kind": "reference",
                         "sample": f"first {k} of {counts.shape[0]} meshes ({tris:,} triangles) on the GPU "
                                   "(the reference path is CUDA)"},
        "clocks": clk.summary(),
    }), flush=True)


def run_reference(args):
    ws, rank, local = dist_info()
    if rank != 0:
        return
    from oracle import ref
    if not ref.runner_available():
        print(json.dumps({"impl": "reference", "unavailable": "reference kernels (oracle/_ref fatbins) not built"}))
        return
    gen, kw, algo, bits, radius, desc = WORKLOADS[args.workload]
    if algo in ("serve", "serve_batched"):
        print(json.dumps({"impl": "reference", "unavailable": "the reference has no serving path (no request "
                          "queue, admission or overlapped builds); nothing of it can run this workload"}))
        return
    if algo in ("lbvh_batched", "ploc_batched"):
        run_reference_batched(args, ref)
        return
    mesh = make_mesh(args.workload)
    n = mesh.size()
    R = ref.RefRunner(fast=True)
    arrays = mesh.arrays()

    def once():
        if algo == "ploc":
            nodes, idx, it, ms, rc = R.ploc(arrays, radius)
            once.ploc_stages = {"init_incl_upload": float(ms[1]), "neighbour_search": float(ms[2]),
                                "merge": float(ms[3]), "scan_compact": float(ms[4]), "iterations": int(it)}
            return ms[0], ms[5]
        if algo == "lbvh_plus":
            nodes, idx, ms = R.lbvh_plus(arrays)
            return ms[0], ms[7]
        nodes, idx, ms = R.lbvh(arrays)
        once.stages = [float(x) for x in ms[1:6]]
        return ms[0], ms[6]

    for _ in range(args.warmup):
        once()
    builds, walls = [], []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            b, w = once()
            builds.append(b)
            walls.append(w)
    b = float(np.mean(builds))
    w = float(np.mean(walls))
    value = n / (b / 1e3) / 1e6
    ref_algo = {"lbvh": "LBVHBuilderCUDA (30-bit Morton, CUB radix sort)",
                "lbvh_plus": "LBVHPlusBuilderCUDA (60-bit, Thrust sort, 1 treelet pass)",
                "ploc": f"PLOCBuilderCUDA(r={radius})"}[algo]
    if treelet_rounds(args.workload) > 1:
        ref_algo += f"; the reference has no multi-pass LBVH+, so this is its 1-pass build, not the " \
                    f"workload's {treelet_rounds(args.workload)} passes"
    line = {
        "impl": "reference", "metric": METRIC,
        "value": round(value, 2), "unit": "Mtris/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(b, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+u32", "data": "synthetic (seeded generator, bvh_gb300/meshgen.py)",
        "config": {"workload": args.workload, "description": desc, "triangles": n,
                   "reference_builder": ref_algo,
                   "how": "the reference's own kernels (its .cu files compiled unmodified, Release flags) "
                          "replayed in its host order with CUB/Thrust; value from its getLastBuildTimeMS"},
        # the reference's public call takes a host mesh and returns host vectors: its own upload
        # (36 B/tri) and download (nodes + indices) happen inside build()
        "e2e": {"value": round(n / (w / 1e3) / 1e6, 2), "unit": "Mtris/s", "h2d_bytes_per_step": 36 * n,
                "d2h_bytes_per_step": 48 * (2 * n - 1) + 4 * n, "ms_per_step": round(w, 3),
                "note": "wall time of the whole build() call: upload, kernels, download, AoS conversion"},
        "cpu_baseline": {"value": round(value, 2), "unit": "Mtris/s", "cores": 1, "kind": "reference",
                         "sample": f"whole workload on the GPU, {args.steps} builds (the reference path is CUDA)"},
        "clocks": clk.summary(),
    }
    if getattr(once, "ploc_stages", None):
        line["stage_ms_last"] = {k: (round(v, 4) if isinstance(v, float) else v) for k, v in once.ploc_stages.items()}
    if getattr(once, "stages", None):
        line["stage_ms_last"] = dict(zip(["bounds", "morton", "sort", "topology", "refit"],
                                         [round(x, 4) for x in once.stages]))
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="c1_lbvh63")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="default workload only: skip the pageable e2e, LBVH-30, batched and serving blocks")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default sort variants")
    ap.add_argument("--host-loops", action="store_true",
                    help="drive the PLOC / LBVH+ device loops from the host (for profilers; slower)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif WORKLOADS[args.workload][2] in ("lbvh_batched", "ploc_batched"):
        run_batched(args)
    elif WORKLOADS[args.workload][2] in ("serve", "serve_batched"):
        run_serve(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
