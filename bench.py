#!/usr/bin/env python3
"""Benchmark of the plain WoB hot path on one GB300.

Workload (the largest single-GPU configuration of the headline metric): 3D interior Robin problem
(du/dn + 2u = h), direct BIE, backward estimator with uniform boundary sampling, on an icosphere
subdivided to 81,920 triangles and displaced by 0.15 * sum_{l<=4} c_lm Y_lm (c_lm ~ N(0,1), seed
0); exact solution u = 1/(4 pi |x - s|), s = (3, 0.5, 0); evaluation points on a 512 x 512 grid of
the z = 0 slice over [-1.3, 1.3]^2, kept when inside the surface; 4096 paths per point, 16 bounces,
FP32 walks, FP64 sums, Philox seed 0.

A step is one pass over every evaluation point with 4096 new paths (path_offset advances, as the
reference's iteration loop does). Metric: bounces per second (a bounce is one executed iteration of
the bounce loop, estimator.cuh:252); the RMSE against the exact solution after all timed steps is
reported beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference algorithm on the host cores: the CPU restatement under
oracle/ with all host threads, on a bounded sample of the same workload. (The reference's own
estimator compiles only where its source tree is present, with stand-ins for its empty Eigen and
lbvh submodules -- oracle/_ref, the source of the committed reference fixtures the restatement is
checked against; that tree is not on the GPU machine.)
"""
from __future__ import annotations

import argparse
import dataclasses
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

METRIC = "bounces/s; time to RMSE 1e-3 vs analytic, plain vs learned-CV WoB, 1 GB300"
UNIT = "bounces/s"
PATHS = 4096
PATH_LENGTH = 16
GRID = 512
EXTENT = 2.6
SEED = 0
# Algorithmic bytes per bounce of this workload: two uniform boundary samples, each one element
# record (76 B) plus one sampling-table entry (8 B).
BYTES_PER_BOUNCE = 2 * (76 + 8)
# DRAM bytes (read + write) of one full-size walk launch of this workload, measured by ncu on the
# timed launch itself (dram__bytes_read.sum + dram__bytes_write.sum, one pass; 15,653,120 +
# 931,584 B, profiles/launches_robin3d_default_bench.md). The scene (5.2 MB of records, 1.3 MB of
# guides) stays in L2, so DRAM traffic is the scene once plus the points and sums, not a
# per-bounce quantity; it applies to the default (full) workload only.
TRAFFIC_BYTES_PER_LAUNCH = 15_653_120 + 931_584
WORKLOAD = ("3D interior Robin (du/dn + 2u = h), direct BIE, backward estimator, uniform sampling; "
            "displaced icosphere 81920 triangles; 512x512 z=0 slice over [-1.3,1.3]^2, inside points; "
            "4096 paths x 16 bounces per point per step")
PROBE_DIR = np.array([0.48, 0.57, 0.66])
DL2D_WORKLOAD = ("2D interior Dirichlet, double-layer BIE, backward estimator, line-intersection sampling; star "
                 "r = 1 + 0.3 cos 5t, 1024 segments, g = e^x cos y; 128x128 grid over [-1.3,1.3]^2, 7960 interior "
                 "points; 1024 paths x 8 bounces per point per step")


# 2D double-layer star: per bounce one infinite-line query, N_node = 31.51 nodes visited and
# N_prim = 4.51 primitives tested by the reference's binary LBVH (oracle/roofline_constants.py):
# 8 N_node + 14 N_prim + 30 FLOP and 16 N_node + 44 N_prim + 8 bytes.
DL2D_FLOP_PER_BOUNCE = 8 * 31.51 + 14 * 4.51 + 30
DL2D_BYTES_PER_BOUNCE = 16 * 31.51 + 44 * 4.51 + 8


def fp32_roofline(bounces_per_s, clk):
    """FP32-issue roofline of the 2D line-intersection walk: algorithmic FLOP per bounce x bounces/s
    against the nominal FP32 rate 152 SMs x 128 lanes x 2 (FMA) x the SM clock seen in the run."""
    mhz = (clk or {}).get("sm_mhz") or 2070.0
    peak = 152 * 128 * 2 * mhz * 1e6 / 1e12
    achieved = DL2D_FLOP_PER_BOUNCE * bounces_per_s / 1e12
    return {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
            "peak_source": "nominal: 152 SMs x 128 FP32 lanes x 2 x median SM clock (no measured FP32 peak)",
            "traffic": None, "algorithmic_flop_per_bounce": DL2D_FLOP_PER_BOUNCE,
            "algorithmic_bytes_per_bounce": DL2D_BYTES_PER_BOUNCE,
            "bytes_view_gbs": DL2D_BYTES_PER_BOUNCE * bounces_per_s / 1e9}


def build_scene_arrays():
    from wobtoolbox_gb300 import workloads as W
    return W.robin_sphere_scene(subdiv=6, seed=SEED, alpha=2.0, source=(3.0, 0.5, 0.0))


def params():
    import wobtoolbox_gb300 as wob
    return wob.EstimatorParams(bie_model=wob.Direct, domain=wob.InteriorDomain, estimator=wob.BackwardEstimator,
                               problem=wob.RobinProblem, path_length=PATH_LENGTH, num_sample_paths=PATHS,
                               seed=SEED)


def probe_dirs(n):
    d = np.tile(PROBE_DIR / np.linalg.norm(PROBE_DIR), (n, 1)).astype(np.float32)
    return d


def exact(points, sc):
    from wobtoolbox_gb300 import workloads as W
    return W.point_sources(points, sc["source"], sc["strengths"])[:, 0]


def cpu_sample(sc, n_points, seed=1):
    """A fixed pseudo-random sample of inside slice points, classified with the oracle's
    brute-force half-line parity test."""
    from oracle import oracle_py as O
    from wobtoolbox_gb300 import workloads as W
    cand = W.slice_points_z0(GRID, EXTENT)
    perm = np.random.default_rng(seed).permutation(len(cand))
    el = O.Elements(sc["verts"], sc["normals"], sc["bvals"], sc["types"], sc["alphas"])
    chosen = []
    for s in range(0, len(perm), 256):
        pts = cand[perm[s:s + 256]]
        d = probe_dirs(len(pts))
        counts, _, hp = O.line_query(el, pts, d)
        for i in range(len(pts)):
            m = min(int(counts[i]), 64)
            t = ((hp[i, :m] - pts[i]) * d[i]).sum(1)
            if (t > 0).sum() % 2 == 1:
                chosen.append(perm[s + i])
        if len(chosen) >= n_points:
            break
    return np.ascontiguousarray(cand[np.array(chosen[:n_points])])


def time_cpu(sc, sample_pts, paths, threads=0, path_offset=0):
    """Runs the oracle on the sample; returns (seconds, bounces, threads used)."""
    from oracle import oracle_py as O
    import wobtoolbox_gb300 as wob
    import dataclasses
    p = dataclasses.replace(params(), num_sample_paths=paths, path_offset=path_offset)
    el = O.Elements(sc["verts"], sc["normals"], sc["bvals"], sc["types"], sc["alphas"])
    t0 = time.perf_counter()
    _, _, b, _ = O.solve_domain(el, p, sample_pts, n_threads=threads)
    return time.perf_counter() - t0, b, O.max_threads()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_init(args):
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    elif torch.cuda.is_available():
        torch.cuda.set_device(0)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def run_reference(args):
    """CPU arm: the reference algorithm (oracle restatement) on all host threads."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle_py as O
    O.build()
    sc = build_scene_arrays()
    sample_pts = cpu_sample(sc, args.ref_points)
    paths = args.cpu_paths
    for w in range(args.warmup):
        time_cpu(sc, sample_pts, paths, path_offset=w * paths)
    secs, bounces = 0.0, 0
    for k in range(args.steps):
        dt, b, threads = time_cpu(sc, sample_pts, paths, path_offset=(args.warmup + k) * paths)
        secs += dt
        bounces += b
    value = bounces / secs
    sample = f"{len(sample_pts)} inside slice points x {paths} paths x {PATH_LENGTH} bounces per step"
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "sample": sample},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "nproc": os.cpu_count(), "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's own CPU/OpenMP build needs its submodules (Eigen, lbvh, libigl, json), which the "
                "reference tree leaves empty; its code is compiled only against stand-ins for the parity fixtures "
                "(timing that build would time the brute-force BVH stand-in), so this arm times the C++ "
                "restatement of its algorithm under oracle/ on all host threads",
    }
    print(json.dumps(out), flush=True)


def slice_inside(scene, cand, dev):
    """Inside test of points against a closed 3D scene on the GPU: an odd number of crossings of a
    half-line (probe_dirs) through the point. Returns a numpy bool mask."""
    import torch
    n_c = len(cand)
    d_c = torch.from_numpy(np.ascontiguousarray(cand)).to(dev)
    d_dir = torch.from_numpy(probe_dirs(n_c)).to(dev)
    counts = torch.zeros(n_c, dtype=torch.int32, device=dev)
    hits = torch.zeros(n_c, 64, dtype=torch.int32, device=dev)
    hp = torch.zeros(n_c, 64, 3, dtype=torch.float32, device=dev)
    scene.line_query(d_c, d_dir, n_c, counts, hits, hp)
    m = torch.clamp(counts, max=64)
    valid = torch.arange(64, device=dev)[None, :] < m[:, None]
    t = ((hp - d_c[:, None, :]) * d_dir[:, None, :]).sum(-1)
    crossings = ((t > 0) & valid).sum(1)
    return (crossings % 2 == 1).cpu().numpy()


def run_ours(args):
    import torch
    import wobtoolbox_gb300 as wob
    from wobtoolbox_gb300 import workloads as W

    rank, world, local = dist_init(args)
    wob.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    if args.workload == "dl2d":
        sc = W.star_dirichlet_scene()
        scene = wob.SceneHost(sc["verts"], sc["normals"], sc["bvals"], sc["types"], sc["alphas"])
        pts = sc["points"]
        paths = 1024
        p = wob.EstimatorParams(bie_model=wob.IndirectDoubleLayer, domain=wob.InteriorDomain,
                                estimator=wob.BackwardEstimator, problem=wob.DirichletProblem, path_length=8,
                                num_sample_paths=paths, seed=SEED)
        exact_u = W.exp_cos(pts)[:, 0]
        workload = DL2D_WORKLOAD
        bytes_per_bounce = None  # FP32-issue bound: see the roofline object below
    else:
        sc = build_scene_arrays()
        scene = wob.SceneHost(sc["verts"], sc["normals"], sc["bvals"], sc["types"], sc["alphas"])
        cand = W.slice_points_z0(GRID, EXTENT)
        pts = np.ascontiguousarray(cand[slice_inside(scene, cand, dev)])
        paths = PATHS
        p = params()
        exact_u = None
        workload = WORKLOAD
        bytes_per_bounce = BYTES_PER_BOUNCE
    if args.small:  # profiling case: every 16th point, 512 paths
        pts = np.ascontiguousarray(pts[::16])
        paths = 512
        if exact_u is not None:
            exact_u = exact_u[::16]
    n_pts = len(pts)
    D = pts.shape[1]
    d_pts = torch.from_numpy(pts).to(dev)
    d_sum = torch.zeros(n_pts, D + 1, dtype=torch.float64, device=dev)
    d_sq = torch.zeros(n_pts, D + 1, dtype=torch.float64, device=dev)
    d_b = torch.zeros(1, dtype=torch.int64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > 129 MB L2
    stream = torch.cuda.current_stream()
    p = dataclasses.replace(p, num_sample_paths=paths)
    base_offset = rank * (1 << 40)

    def step(k, sum_buf=d_sum, sq_buf=d_sq):
        scene.solve_domain(dataclasses.replace(p, path_offset=base_offset + k * paths), d_pts, n_pts, sum_buf,
                           sq_buf, d_b, stream)

    tuned = scene.autotune_domain(p, d_pts, n_pts, stream)
    for w in range(args.warmup):
        step(w)
    torch.cuda.synchronize()
    d_sum.zero_()
    d_sq.zero_()
    d_b.zero_()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        for k in range(args.steps):
            flush.fill_(float(k))  # evict the scene from L2 between timed steps (not timed)
            starts[k].record(stream)
            step(args.warmup + k)
            ends[k].record(stream)
        torch.cuda.synchronize()
    barrier(world)
    kernel_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    local_s = sum(kernel_ms) / 1e3
    bounces_local = int(d_b.item())
    # every rank learns of a traversal-limit hit on any rank before the collectives below, so all
    # ranks stop together instead of some waiting in all_reduce
    if max_over_ranks(float(scene.poll_error()), world):
        raise RuntimeError("device traversal limit hit on some rank")
    total_s = max_over_ranks(local_s, world)
    bounces_all = sum_over_ranks(bounces_local, world)
    value = bounces_all / total_s

    # accuracy after all timed steps (args.steps * 4096 paths per point)
    s = d_sum.cpu().numpy()
    n_paths_total = args.steps * paths
    u = s[:, 0] / n_paths_total
    if exact_u is None:
        exact_u = exact(pts, sc)
    rmse = float(np.sqrt(np.mean((u - exact_u) ** 2)))
    err = np.sort(np.abs(u - exact_u))
    error_spread = {"median_point_error": float(err[len(err) // 2]),
                    "rmse_best_99pct_points": float(np.sqrt(np.mean(err[:int(0.99 * len(err))] ** 2)))}

    # end to end through the C ABI with host buffers (copies in the timed region)
    pts_pinned = torch.from_numpy(pts).pin_memory()
    h_sum = np.zeros((n_pts, D + 1))
    h_sq = np.zeros((n_pts, D + 1))
    e2e_p = dataclasses.replace(p, path_offset=base_offset + (1 << 30))
    import ctypes as C
    lib = wob.load()
    bb = C.c_uint64(0)
    cp = e2e_p.to_c()
    for w in range(1):
        wob.check(lib.wob_solve_domain_host(scene.handle, C.byref(cp), pts_pinned.data_ptr(), n_pts,
                                            h_sum.ctypes.data, h_sq.ctypes.data, C.byref(bb)))
    barrier(world)
    e2e_steps = max(1, min(args.steps, 3))
    t0 = time.perf_counter()
    b0 = bb.value
    for k in range(e2e_steps):
        cp.path_offset = base_offset + (1 << 30) + (k + 1) * paths
        wob.check(lib.wob_solve_domain_host(scene.handle, C.byref(cp), pts_pinned.data_ptr(), n_pts,
                                            h_sum.ctypes.data, h_sq.ctypes.data, C.byref(bb)))
    e2e_local = time.perf_counter() - t0
    e2e_s = max_over_ranks(e2e_local, world)
    e2e_bounces = sum_over_ranks(bb.value - b0, world)
    e2e_value = e2e_bounces / e2e_s

    out = None
    if rank == 0:
        avg_ms = sum(kernel_ms) / len(kernel_ms)
        bounces_per_launch = bounces_local / args.steps
        achieved = (bytes_per_bounce or 0) * bounces_per_launch / (avg_ms / 1e3) / 1e9
        peaks = {}
        try:
            with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
                peaks = json.load(f)
        except OSError:
            pass
        peak = float(peaks.get("hbm_gbs", 6800.0))
        clk = clocks.summary()
        gather = None
        if bytes_per_bounce:
            # the walk's own ceiling: random guide + 64-byte record gathers over tables of this
            # scene's sizes (L2-resident), measured now on this GPU (wob_measure_gather_peak)
            import ctypes as C
            sps, gms = C.c_double(0.0), C.c_float(0.0)
            wob.check(wob.load().wob_measure_gather_peak(scene.n_elems, min(scene.n_elems, 1 << 22), 4096,
                                                         C.byref(sps), C.byref(gms)))
            per_sample = bytes_per_bounce / 2  # two uniform samples per bounce
            gather = {"samples_per_s": sps.value, "ms": gms.value,
                      "peak_gbs": sps.value * per_sample / 1e9}
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * total_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": workload, "elements": int(len(sc["verts"])), "points": n_pts,
                       "paths_per_point_per_step": paths, "path_length": p.path_length,
                       "l2": "flushed between timed steps (256 MiB write, outside the timed events)",
                       "rmse_u_vs_exact": rmse, "error_spread": error_spread, "paths_per_point_total": n_paths_total,
                       "parallelism": f"replicas x{world}, points x independent path streams",
                       "autotune": {"chosen_config": tuned[0], "ms_per_config": tuned[1]},
                       "line_grid": {"bins": scene.info()["line_grid_bins"], "cells": scene.info()["line_grid_cells"]}},
            "roofline": {"bound": "l2_gather", "achieved": achieved, "peak": gather["peak_gbs"], "unit": "GB/s",
                         "frac": achieved / gather["peak_gbs"],
                         "peak_source": "measured in this run: guide-entry + 64-byte record gathers over tables of "
                                        "this scene's sizes at full occupancy (wob_measure_gather_peak, "
                                        f"{gather['samples_per_s']:.4g} samples/s), in the same algorithmic bytes "
                                        "per sample (76 + 8) as achieved",
                         "hbm": {"peak": peak, "frac": achieved / peak,
                                 "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured copy bandwidth)" if peaks
                                 else "fallback 6.8 TB/s",
                                 "note": "the scene is L2-resident: the algorithmic bytes are L1/L2 gathers, not "
                                         "DRAM traffic, so this fraction does not bound the kernel"},
                         "traffic": None,
                         "traffic_note": "not measured in this run (no profiler in the timed run); the ncu capture "
                                         "of this launch read " + str(TRAFFIC_BYTES_PER_LAUNCH) + " B of DRAM "
                                         "(profiles/launches_robin3d_default_bench.md)",
                         "algorithmic_bytes_per_bounce": bytes_per_bounce} if bytes_per_bounce else
                        fp32_roofline(bounces_per_launch / (avg_ms / 1e3), clk),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": n_pts * D * 4,
                    "d2h_bytes_per_step": n_pts * (D + 1) * 8 * 2 + 8 + 4, "steps": e2e_steps},
            "clocks": clk,
            "gpu_launches": args.steps,
            "kernel_ms": kernel_ms,
        }
        if not args.no_cpu_baseline and args.workload == "robin3d":
            from oracle import oracle_py as O
            O.build()
            sample_pts = cpu_sample(sc, args.cpu_points)
            dt, b, threads = time_cpu(sc, sample_pts, args.cpu_paths)
            out["cpu_baseline"] = {"value": b / dt, "unit": UNIT, "cores": threads, "nproc": os.cpu_count(), "kind": "port",
                                   "sample": f"{len(sample_pts)} inside slice points x {args.cpu_paths} paths x "
                                             f"{PATH_LENGTH} bounces ({dt:.1f} s)"}
        elif not args.no_cpu_baseline and args.workload == "dl2d":
            # the full 2D workload on the host cores: 7,960 points x 1024 paths x 8 bounces, line
            # queries through the oracle's binary BVH (the reference's algorithm, same results)
            from oracle import oracle_py as O
            O.build()
            el = O.Elements(sc["verts"], sc["normals"], sc["bvals"], sc["types"], sc["alphas"])
            t0 = time.perf_counter()
            _, _, b, _ = O.solve_domain(el, p, sc["points"], accel=True)
            dt = time.perf_counter() - t0
            out["cpu_baseline"] = {"value": b / dt, "unit": UNIT, "cores": O.max_threads(), "nproc": os.cpu_count(),
                                   "kind": "port",
                                   "sample": f"the full workload: {len(sc['points'])} points x {p.num_sample_paths} "
                                             f"paths x {p.path_length} bounces ({dt:.1f} s)"}
    scene.close()
    if rank == 0 and args.workload == "robin3d" and not args.small and not args.no_time_to_rmse:
        # the metric's second half: time to RMSE 1e-3 against the analytic solution, plain vs the
        # learned residual control variate, on the exterior Neumann workload (327,680 triangles)
        ttr = cv_time_to_rmse(dev, plain_budget=12.0, cv_budget=4.0)
        ttr["cv_curve"] = ttr["cv_curve"][::max(1, len(ttr["cv_curve"]) // 8)]
        out["time_to_rmse"] = ttr
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_batch(args):
    """Batched workload: 256 seeded 2D scenes (lobes U{3..9}, amplitude U[0.1, 0.35], segments
    log-uniform in [64, 16384], points U[1k, 64k]; interior / exterior x Neumann / Robin, Gaussian
    sources in the interior scenes) in one persistent launch per walk variant (three here: backward
    single layer, forward single-layer Neumann, the general walk for the scenes with sources), against
    the same 256 solves launched one after another (eagerly and replayed from a captured CUDA graph)."""
    import torch
    import wobtoolbox_gb300 as wob
    from wobtoolbox_gb300 import workloads as W
    rank, world, local = dist_init(args)
    wob.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    paths = args.batch_paths
    specs = W.batch_scenes(256, seed=SEED, paths=paths, path_length=8,
                           point_range=(args.batch_points_min, args.batch_points_max))
    scenes, plist = [], []
    for sc in specs:
        s = wob.SceneHost(sc["verts"], sc["normals"], sc["bvals"], sc["types"], sc["alphas"])
        if sc["volume"] is not None:
            s.set_volume_cache(*sc["volume"])
        scenes.append(s)
        plist.append(wob.EstimatorParams(seed=SEED, **sc["params"]))
    n_pts = [len(sc["points"]) for sc in specs]
    pts = torch.from_numpy(np.concatenate([sc["points"] for sc in specs])).to(dev)
    total = len(pts)
    batch = wob.SceneBatch(scenes, plist, n_pts)
    off = batch.offsets
    d_sum = torch.zeros(total, 3, dtype=torch.float64, device=dev)
    d_sq = torch.zeros_like(d_sum)
    d_b = torch.zeros(1, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def sequential(k):
        for i, (s, p) in enumerate(zip(scenes, plist)):
            q = dataclasses.replace(p, path_offset=k * paths)
            s.solve_domain(q, pts[off[i]:off[i + 1]], n_pts[i], d_sum[off[i]:off[i + 1]], d_sq[off[i]:off[i + 1]],
                           d_b, stream)

    def batched(k):
        batch.solve(pts, d_sum, d_sq, d_b, k * paths, stream)

    def timed(fn, steps, base):
        ms = []
        for k in range(steps):
            flush.fill_(float(k))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn(base + k)
            e1.record(stream)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        return ms

    for w in range(args.warmup):
        batched(w)
        sequential(w)
    torch.cuda.synchronize()
    d_b.zero_()
    with ClockSampler(local) as clocks:
        b_ms = timed(batched, args.steps, 100)
        torch.cuda.synchronize()
        bounces_batched = int(d_b.item())
        s_ms = timed(sequential, args.steps, 200)
        # the sequential solves replayed from a captured graph (no launch overhead)
        g = torch.cuda.CUDAGraph()
        gs = torch.cuda.Stream()
        gs.wait_stream(stream)
        with torch.cuda.stream(gs):
            with torch.cuda.graph(g, stream=gs):
                for i, (s, p) in enumerate(zip(scenes, plist)):
                    s.solve_domain(p, pts[off[i]:off[i + 1]], n_pts[i], d_sum[off[i]:off[i + 1]],
                                   d_sq[off[i]:off[i + 1]], d_b, gs)
        stream.wait_stream(gs)
        g_ms = timed(lambda k: g.replay(), args.steps, 300)
    clk = clocks.summary()
    value = bounces_batched / (sum(b_ms) / 1e3)
    out = {
        "metric": "batched plain WoB: speedup of persistent batched launches (one per walk variant) over 256 "
                  "sequential launches",
        "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": sum(b_ms) / len(b_ms), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": "256 2D star scenes (lobes U{3..9}, amplitude U[0.1,0.35], segments log-uniform "
                               "[64,16384], points U[1k,64k]); interior/exterior x Neumann (SL forward) / Robin (SL "
                               "backward, RIS 64); 4 Gaussian sources in interior scenes",
                   "points": total, "points_per_scene": [args.batch_points_min, args.batch_points_max],
                   "paths_per_point": paths, "path_length": 8,
                   "batched_ms": sum(b_ms) / len(b_ms), "sequential_ms": sum(s_ms) / len(s_ms),
                   "graph_sequential_ms": sum(g_ms) / len(g_ms),
                   "speedup_vs_sequential": (sum(s_ms) / sum(b_ms)),
                   "speedup_vs_graph_sequential": (sum(g_ms) / sum(b_ms)),
                   "l2": "flushed between timed steps (256 MiB write, outside the timed events)"},
        "clocks": clk, "gpu_launches": args.steps,
    }
    if rank == 0:
        print(json.dumps(out), flush=True)
    batch.close()
    for s in scenes:
        s.close()


def exterior_neumann_case(dev, subdiv=7, seed=SEED):
    """The exterior Neumann workload (data/config_general_3d_exterior_Neumann.json at the mesh
    size of the learned-CV configuration): displaced icosphere (0.15 sum c_lm Y_lm, l <= 4)
    subdivided `subdiv` times (7: 327,680 triangles), Neumann data of u = sum_{k<3} q_k / (4 pi
    |x - s_k|) with s_k inside at radius <= 0.5 and q_k ~ U[-1, 1]; the points of the 256^2 z = 0
    slice over [-2, 2]^2 outside the surface (half-line parity on the GPU). Returns (scene, points,
    exact u at the points, faces)."""
    import torch
    import wobtoolbox_gb300 as wob
    from wobtoolbox_gb300 import workloads as W
    rng = np.random.default_rng(seed)
    V, F, _ = W.displaced_icosphere(subdiv, 0.15, 4, seed)
    verts, normals = W.mesh_elements(V, F)
    dirs = rng.standard_normal((3, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    src = dirs * rng.uniform(0, 0.5, (3, 1))
    q = rng.uniform(-1, 1, 3)
    uv = W.point_sources(verts.reshape(-1, 3), src, q).reshape(len(F), 3, 4)
    g = (uv[..., 1:] * normals[:, None, :].astype(np.float64)).sum(-1).astype(np.float32)
    scene = wob.SceneHost(verts, normals, g, np.ones(len(F), np.int32))
    cand = W.slice_points_z0(256, 4.0)
    d_c = torch.from_numpy(cand).to(dev)
    d_dir = torch.from_numpy(probe_dirs(len(cand))).to(dev)
    counts = torch.zeros(len(cand), dtype=torch.int32, device=dev)
    hits = torch.zeros(len(cand), 64, dtype=torch.int32, device=dev)
    hp = torch.zeros(len(cand), 64, 3, dtype=torch.float32, device=dev)
    scene.line_query(d_c, d_dir, len(cand), counts, hits, hp)
    valid = torch.arange(64, device=dev)[None, :] < torch.clamp(counts, max=64)[:, None]
    t = ((hp - d_c[:, None, :]) * d_dir[:, None, :]).sum(-1)
    outside = (((t > 0) & valid).sum(1) % 2 == 0).cpu().numpy()
    del hits, hp
    pts = np.ascontiguousarray(cand[outside])
    exact_u = W.point_sources(pts, src, q)[:, 0]
    return scene, pts, exact_u, F


def run_fwd3d(args):
    """The plain walk of the learned-CV workload alone (exterior_neumann_case: forward single
    layer, line-intersection sampling, 4 bounces, 327,680 triangles, 54,025 slice points): bounces
    per second over `--steps` solves of `--fwd-paths` paths per point, L2 flushed between steps,
    the kernel configuration autotuned (or pinned with --fwd-config), with the lockstep kernel's
    rate (configuration 0) measured beside it. --small: the first 4096 points, 128 paths (the
    profiling case)."""
    import ctypes as C
    import torch
    import wobtoolbox_gb300 as wob
    rank, world, local = dist_init(args)
    lib = wob.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    scene, pts, _, F = exterior_neumann_case(dev, args.cv_subdiv, SEED)
    paths = args.fwd_paths
    if args.small:
        pts, paths = np.ascontiguousarray(pts[:4096]), 128
    n = len(pts)
    d = torch.from_numpy(pts).to(dev)
    L = 4
    p = wob.EstimatorParams(bie_model=wob.IndirectSingleLayer, domain=wob.ExteriorDomain,
                            estimator=wob.ForwardEstimator, problem=wob.NeumannProblem, path_length=L, seed=SEED,
                            num_sample_paths=paths)
    var = C.c_int32(-1)
    wob.check(lib.wob_tunable_variant(scene.handle, C.byref(p.to_c()), C.byref(var)))
    saved = C.c_int32(0)
    wob.check(lib.wob_get_domain_config(var.value, C.byref(saved)))
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    s_ = torch.zeros(n, 4, dtype=torch.float64, device=dev)
    b_ = torch.zeros(1, dtype=torch.int64, device=dev)

    def timed(steps, base):
        ms = []
        for k in range(steps):
            flush.fill_(float(k))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            scene.solve_domain(dataclasses.replace(p, path_offset=(base + k) * paths), d, n, s_, None, b_, stream)
            e1.record(stream)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        return ms

    try:
        if args.fwd_config >= 0:
            wob.check(lib.wob_set_domain_config(var.value, args.fwd_config))
            tuned = None
        else:
            tuned = scene.autotune_domain(p, d, n, stream)
        cfg = C.c_int32(0)
        wob.check(lib.wob_get_domain_config(var.value, C.byref(cfg)))
        timed(args.warmup, 0)
        b_.zero_()
        with ClockSampler(local) as clocks:
            ms = timed(args.steps, 100)
        bounces = int(b_.item())
        clk = clocks.summary()
        lock_ms = None
        if not args.small and cfg.value != 0:
            wob.check(lib.wob_set_domain_config(var.value, 0))
            timed(1, 200)
            lock_ms = min(timed(max(1, args.steps // 2), 300))
    finally:
        lib.wob_set_domain_config(var.value, saved.value)
    value = bounces / (sum(ms) / 1e3)
    wave = cfg.value % 4 != 0
    chunk = [1 << 22, 1 << 21, 1 << 20, 1 << 19][cfg.value // 4]
    chunks = -(-n // max(1, chunk // paths))
    out = {
        "metric": "bounces/s, 3D forward single-layer walk (line-intersection sampling)", "value": value,
        "unit": "bounces/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": sum(ms) / len(ms), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"exterior Neumann, forward single layer, {L} bounces, displaced icosphere "
                               f"{len(F)} triangles, {n} slice points outside the surface, {paths} paths per point "
                               "per step",
                   "kernel_config": cfg.value,
                   "kernel": (f"split-phase wavefront, trace shape {cfg.value % 4}"
                              f"{' (compressed nodes)' if cfg.value % 4 == 3 else ''}, {chunk} paths per chunk"
                              if wave else "lockstep walk"),
                   "autotune": None if tuned is None else {"chosen_config": tuned[0], "ms_per_config": tuned[1]},
                   "l2": "flushed between timed steps (256 MiB write, outside the timed events)"},
        "lockstep_ms_per_step": lock_ms,
        "speedup_vs_lockstep": (lock_ms / (sum(ms) / len(ms))) if lock_ms else None,
        "clocks": clk,
        "gpu_launches": args.steps * (chunks * (2 + 2 * (L - 1)) if wave else 1),
    }
    if rank == 0:
        print(json.dumps(out), flush=True)
    scene.close()


def cv_time_to_rmse(dev, subdiv=7, target=1e-3, plain_paths=256, cv_paths=32, plain_budget=20.0, cv_budget=5.0,
                    train_steps=2000, near_factor=3.0, theta=0.3, seed=SEED):
    """Time to RMSE `target` against the analytic solution, plain forward WoB vs the learned
    residual control variate, on the exterior Neumann workload: displaced icosphere (0.15 sum
    c_lm Y_lm, l <= 4) subdivided `subdiv` times (7: 327,680 triangles), Neumann data of
    u = sum_{k<3} q_k / (4 pi |x - s_k|) with s_k inside at radius <= 0.5 and q_k ~ U[-1, 1];
    forward single-layer estimator (data/config_general_3d_exterior_Neumann.json), 4 bounces;
    evaluation at the 256^2 points of the z = 0 slice over [-2, 2]^2 outside the surface.

    Both estimators run progressive iterations (plain_paths / cv_paths new paths per point each) and
    the RMSE of the running estimate is taken after each; times are wall-clock on a synchronised
    device, excluding only the RMSE evaluation. The control variate's clock starts before its
    training labels: labels (65,536 boundary points x 256-path walk estimates of the density,
    clamped to the 0.999 quantile of their magnitude), 2000 device Adam steps of the 32-frequency 4 x 64 SiLU network, the network at every
    triangle's centroid, the residual Neumann data, the residual scene, the control variate's
    potential at the points, then the residual walks. Returns a dict."""
    import torch
    import wobtoolbox_gb300 as wob
    from wobtoolbox_gb300 import cv
    scene, pts, exact_u, F = exterior_neumann_case(dev, subdiv, seed)
    n_pts = len(pts)
    d_pts = torch.from_numpy(pts).to(dev)
    base = wob.EstimatorParams(bie_model=wob.IndirectSingleLayer, domain=wob.ExteriorDomain,
                               estimator=wob.ForwardEstimator, problem=wob.NeumannProblem, path_length=4, seed=seed)

    def clock():
        torch.cuda.synchronize()
        return time.perf_counter()

    def progressive(sc, paths, budget_s, t_start, offset_u=None):
        s_ = torch.zeros(n_pts, 4, dtype=torch.float64, device=dev)
        b_ = torch.zeros(1, dtype=torch.int64, device=dev)
        curve, k, elapsed = [], 0, 0.0
        t_hit = None
        while elapsed < budget_s and k < 100000:
            t0 = clock()
            sc.solve_domain(dataclasses.replace(base, num_sample_paths=paths, path_offset=k * paths), d_pts, n_pts,
                            s_, None, b_)
            elapsed += clock() - t0
            k += 1
            u = s_[:, 0].cpu().numpy() / (k * paths)
            if offset_u is not None:
                u = u + offset_u
            r = float(np.sqrt(np.mean((u - exact_u) ** 2)))
            curve.append((t_start + elapsed, r, k * paths))
            if r <= target:
                t_hit = t_start + elapsed
                break
        return curve, t_hit, int(b_.item())

    # one-time calibration and warm-up (not timed): the forward walk's kernel shape is autotuned
    # (it serves the plain and the residual walks alike), then the training graph is warmed up
    tuned = scene.autotune_domain(dataclasses.replace(base, num_sample_paths=plain_paths), d_pts, n_pts)
    tmp = torch.zeros(n_pts, 4, dtype=torch.float64, device=dev)
    scene.solve_domain(dataclasses.replace(base, num_sample_paths=32), d_pts, n_pts, tmp)
    warm, _ = cv.train_density_cv(scene, base, n_train=8192, train_paths=16, steps=20, batch=8192, lr=2e-3, seed=99)
    warm.close()
    torch.cuda.synchronize()

    plain_curve, t_plain, plain_b = progressive(scene, plain_paths, plain_budget, 0.0)
    t0 = clock()
    mlp, info = cv.train_density_cv(scene, base, n_train=65536, train_paths=256, steps=train_steps, batch=8192,
                                    lr=2e-3, freq_sigma=1.0, seed=seed)
    t1 = clock()
    rscene, sigma = cv.residual_control_variate(scene, mlp, wob.ExteriorDomain, near_factor=near_factor, theta=theta)
    t2 = clock()
    pot = cv.control_variate_potential(scene, sigma, d_pts, n_pts, near_factor=near_factor, theta=theta)
    u_cv = pot[:, 0].double().cpu().numpy()
    t3 = clock()
    setup = t3 - t0
    cv_curve, t_cv, cv_b = progressive(rscene, cv_paths, cv_budget, setup, offset_u=u_cv)
    rate = plain_b / max(plain_curve[-1][0], 1e-9)
    out = {
        "target_rmse": target, "plain_s": t_plain, "cv_s": t_cv,
        "plain_over_cv": (t_plain / t_cv) if (t_plain and t_cv) else None,
        "cv_setup_s": {"labels": info["t_labels_s"], "training_2000_adam_steps": info["t_train_s"],
                       "labels_and_training": t1 - t0, "residual_data_and_scene": t2 - t1, "potential": t3 - t2,
                       "total": setup},
        "cv_walk_s": (t_cv - setup) if t_cv else None,
        "paths_per_point": {"plain": plain_curve[-1][2], "cv": cv_curve[-1][2]},
        "final_rmse": {"plain": plain_curve[-1][1], "cv": cv_curve[-1][1]},
        "triangles": int(len(F)), "points": n_pts, "plain_bounces_per_s": rate,
        "forward_walk_autotune": {"chosen_config": tuned[0], "ms_per_config": tuned[1]},
        "train_loss_first_last": [info["history"][0][1], info["history"][-1][1]],
        "label_clip": {"quantile": info["clip_quantile"], "threshold": info["clip_threshold"]},
        "cv_tables": {"near_factor": near_factor, "cluster_theta": theta},
        "plain_curve": plain_curve[::max(1, len(plain_curve) // 8)], "cv_curve": cv_curve,
        "clock": "wall time on a synchronised device; RMSE evaluation excluded; CV time includes its setup",
    }
    mlp.close()
    rscene.close()
    scene.close()
    return out


def run_cv(args):
    """Learned control variate vs plain WoB, time to RMSE 1e-3 against the analytic solution on
    the exterior Neumann workload (cv_time_to_rmse)."""
    import torch
    import wobtoolbox_gb300 as wob
    rank, world, local = dist_init(args)
    wob.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    res = cv_time_to_rmse(dev, subdiv=args.cv_subdiv, plain_paths=args.cv_paths, plain_budget=args.cv_budget,
                          cv_budget=args.cv_budget, near_factor=args.cv_near,
                          theta=args.cv_theta)
    out = {
        "metric": "time to RMSE 1e-3 vs analytic, plain vs learned-CV WoB (3D exterior Neumann)",
        "value": res["plain_over_cv"], "unit": "x (plain time / CV time including its setup)", "n_gpus": world,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "exterior Neumann, forward single layer, 4 bounces, displaced icosphere; residual "
                               "control variate: 32 Fourier features, 4x64 SiLU, 2000 Adam steps on 65,536 x "
                               "256-path density estimates"},
        "time_to_rmse": res,
    }
    if rank == 0:
        print(json.dumps(out), flush=True)


def mixed_rhs_scene(subdiv, n_rhs, seed=SEED, dev=None):
    """Interior mixed problem of the multi-RHS workload: displaced icosphere (as the Robin workload),
    Dirichlet on faces whose centroid has z > 0, Neumann elsewhere; RHS r is the exact solution of
    three exterior point sources (radius U[2, 4], strengths U[-1, 1]). Returns the element arrays, the
    RHS table [n, 3, n_rhs] (per element vertex: u on Dirichlet faces, du/dn on Neumann faces) and
    the sources [n_rhs, 3, 3] / strengths [n_rhs, 3]."""
    from wobtoolbox_gb300 import workloads as W
    V, F, _ = W.displaced_icosphere(subdiv, 0.15, 4, seed)
    verts, normals = W.mesh_elements(V, F)
    cz = V[F][:, :, 2].astype(np.float64).mean(1)
    types = np.where(cz > 0, 0, 1).astype(np.int32)
    rng = np.random.default_rng(seed + 1)
    dirs = rng.standard_normal((n_rhs, 3, 3))
    dirs /= np.linalg.norm(dirs, axis=2, keepdims=True)
    src = dirs * rng.uniform(2.0, 4.0, (n_rhs, 3, 1))
    q = rng.uniform(-1.0, 1.0, (n_rhs, 3))
    if dev is None:
        table = np.empty((len(F), 3, n_rhs), np.float32)
        nrm = normals.astype(np.float64)
        dirichlet = (types == 0)[:, None]
        for r in range(n_rhs):
            ug = W.point_sources(V, src[r], q[r])                   # [n_vertices, 4]: u, grad u
            uf = ug[F]                                              # [n, 3, 4]
            dudn = (uf[..., 1:] * nrm[:, None, :]).sum(-1)
            table[:, :, r] = np.where(dirichlet, uf[..., 0], dudn)
    else:  # the same formulas in float64 on the device
        import torch
        Vt = torch.from_numpy(V.astype(np.float64)).to(dev)
        Ft = torch.from_numpy(F.astype(np.int64)).to(dev)
        nt = torch.from_numpy(normals.astype(np.float64)).to(dev)
        dt = torch.from_numpy(types == 0).to(dev)[:, None]
        tt = torch.empty((len(F), 3, n_rhs), dtype=torch.float32, device=dev)
        for r in range(n_rhs):
            u = torch.zeros(len(V), dtype=torch.float64, device=dev)
            gr = torch.zeros(len(V), 3, dtype=torch.float64, device=dev)
            for k in range(3):
                d = Vt - torch.from_numpy(src[r, k]).to(dev)[None, :]
                rr = torch.linalg.norm(d, dim=1)
                u += q[r, k] / (4.0 * np.pi * rr)
                gr += (-q[r, k] / (4.0 * np.pi)) * d / (rr ** 3)[:, None]
            dudn = (gr[Ft] * nt[:, None, :]).sum(-1)
            tt[:, :, r] = torch.where(dt, u[Ft], dudn).float()
        table = tt.cpu().numpy()
    return dict(V=V, F=F, verts=verts, normals=normals, types=types, table=table, src=src, q=q)


def inside_points(scene, n, lo, hi, seed, dev):
    """n points uniform in the box [lo, hi]^3 and inside the surface (half-line crossing parity)."""
    import torch
    rng = np.random.default_rng(seed)
    out, have = [], 0
    while have < n:
        m = int((n - have) * 2.2) + 1024
        cand = rng.uniform(lo, hi, (m, 3)).astype(np.float32)
        d_c = torch.from_numpy(cand).to(dev)
        d_dir = torch.from_numpy(probe_dirs(m)).to(dev)
        counts = torch.zeros(m, dtype=torch.int32, device=dev)
        hits = torch.zeros(m, 64, dtype=torch.int32, device=dev)
        hp = torch.zeros(m, 64, 3, dtype=torch.float32, device=dev)
        scene.line_query(d_c, d_dir, m, counts, hits, hp)
        valid = torch.arange(64, device=dev)[None, :] < torch.clamp(counts, max=64)[:, None]
        t = ((hp - d_c[:, None, :]) * d_dir[:, None, :]).sum(-1)
        inside = (((t > 0) & valid).sum(1) % 2 == 1).cpu().numpy()
        out.append(cand[inside])
        have += int(inside.sum())
    return np.ascontiguousarray(np.concatenate(out)[:n])


def run_multi_rhs(args):
    """Multi-RHS workload: 3D interior mixed problem (Dirichlet on faces with centroid z > 0, Neumann
    elsewhere) on a displaced icosphere with 1,310,720 triangles; 64 RHS, each the exact solution of
    three exterior point sources (radius 2-4, strengths U[-1, 1]), share one set of walks. Estimator:
    the reference's interior Mixed configuration (data/config_general_3d_interior_Mixed.json: single
    layer, backward, 4 bounces, 64 RIS candidates, eps 1e-5, first-kind scaling 2). Evaluation: 10^6
    random interior points. Progressive iterations of --mrhs-paths paths per point; after each, the
    mean over the 64 RHS of the RMSE against the exact solutions is recorded against cumulative GPU
    time. The same iteration is also timed as one scalar walk (one RHS) to give the cost of 64
    separate solves."""
    import torch
    import wobtoolbox_gb300 as wob
    rank, world, local = dist_init(args)
    wob.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    R = args.mrhs_rhs
    t0 = time.perf_counter()
    sc = mixed_rhs_scene(args.mrhs_subdiv, R, dev=dev)
    t_data = time.perf_counter() - t0
    t0 = time.perf_counter()
    scene = wob.SceneHost(sc["verts"], sc["normals"], sc["table"][:, :, 0], sc["types"])
    t_build = time.perf_counter() - t0
    t0 = time.perf_counter()
    scene.set_rhs(sc["table"])
    t_rhs = time.perf_counter() - t0
    lo, hi = float(sc["V"].min()), float(sc["V"].max())
    pts = inside_points(scene, args.mrhs_points, lo, hi, SEED + 2, dev)
    n_pts = len(pts)
    d_pts = torch.from_numpy(pts).to(dev)
    # exact solutions [n_pts, R] (float64, on the device)
    src = torch.from_numpy(sc["src"]).to(dev)
    qq = torch.from_numpy(sc["q"]).to(dev)
    xp = d_pts.double()
    exact = torch.zeros(n_pts, R, dtype=torch.float64, device=dev)
    for k in range(3):
        dist = torch.linalg.norm(xp[:, None, :] - src[None, :, k, :], dim=2)
        exact += qq[None, :, k] / (4.0 * np.pi * dist)
    if args.mrhs_bie == "direct":  # direct BIE, two uniform samples per bounce (estimator.cuh:335-347)
        base = wob.EstimatorParams(bie_model=wob.Direct, domain=wob.InteriorDomain, estimator=wob.BackwardEstimator,
                                   problem=wob.MixedProblem, path_length=args.mrhs_path_length or 4,
                                   first_kind_equation_scaling_constant=2.0, seed=SEED)
    else:
        base = wob.EstimatorParams(bie_model=wob.IndirectSingleLayer, domain=wob.InteriorDomain,
                                   estimator=wob.BackwardEstimator, problem=wob.MixedProblem,
                                   path_length=args.mrhs_path_length or 4, num_resampling_candidates=64, eps=1e-5,
                                   first_kind_equation_scaling_constant=2.0, seed=SEED)
    paths = args.mrhs_paths
    stream = torch.cuda.current_stream()
    s = torch.zeros(n_pts, R, dtype=torch.float64, device=dev)
    b = torch.zeros(1, dtype=torch.int64, device=dev)
    # warm-up of both kernels (small path offsets beyond any timed one are not reused)
    warm = dataclasses.replace(base, num_sample_paths=1, path_offset=1 << 40)
    for _ in range(args.warmup):
        scene.solve_domain_multi(warm, d_pts, n_pts, s, None, None, None, stream)
    s1 = torch.zeros(n_pts, 4, dtype=torch.float64, device=dev)
    for _ in range(args.warmup):
        scene.solve_domain(warm, d_pts, n_pts, s1, None, None, stream)
    # one scalar walk iteration (RHS 0 only), timed
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s1.zero_()
    e0.record(stream)
    scene.solve_domain(dataclasses.replace(base, num_sample_paths=paths), d_pts, n_pts, s1, None, None, stream)
    e1.record(stream)
    torch.cuda.synchronize()
    t_scalar = e0.elapsed_time(e1) / 1e3
    sampler = ClockSampler(torch.cuda.current_device())
    sampler.__enter__()

    def progressive(solve, budget_s):
        s.zero_()
        b.zero_()
        curve, total, k = [], 0.0, 0
        while (total < budget_s and k < args.steps * 1000) or k < args.steps:
            p = dataclasses.replace(base, num_sample_paths=paths, path_offset=k * paths)
            e0.record(stream)
            solve(p)
            e1.record(stream)
            torch.cuda.synchronize()
            total += e0.elapsed_time(e1) / 1e3
            k += 1
            u = s / (k * paths)
            rmse = torch.sqrt(((u - exact) ** 2).mean(0))
            curve.append((total, float(rmse.mean().item()), k * paths))
        # time to mean RMSE 1e-3, extrapolated from the last point with RMSE ~ 1/sqrt(paths)
        t_last, r_last, _ = curve[-1]
        return curve, int(b.item()), t_last * (r_last / 1e-3) ** 2

    plain_curve, bounces, plain_target = progressive(
        lambda p: scene.solve_domain_multi(p, d_pts, n_pts, s, None, b, None, stream), args.mrhs_budget)
    sampler.__exit__(None, None, None)
    clocks = sampler.summary()
    # how the error is spread over the points (diagnostic): per-point RMS error over the RHS, its
    # median and the RMSE of the 99 % / 99.9 % of points with the smallest error
    err_pt = torch.sqrt(((s / plain_curve[-1][2] - exact) ** 2).mean(1))
    srt = torch.sort(err_pt).values
    spread = {"median_point_error": float(srt[len(srt) // 2].item()),
              "rmse_best_99pct_points": float(torch.sqrt((srt[:int(0.99 * len(srt))] ** 2).mean()).item()),
              "rmse_best_99.9pct_points": float(torch.sqrt((srt[:int(0.999 * len(srt))] ** 2).mean()).item()),
              "rmse_all_points": float(torch.sqrt((srt ** 2).mean()).item())}
    total = plain_curve[-1][0]
    t_iter = total / len(plain_curve)
    if args.mrhs_plain_only:
        if rank == 0:
            print(json.dumps({"metric": "multi-RHS WoB (plain leg only)", "value": bounces / total,
                              "unit": "bounces/s (each bounce serves every RHS)", "n_gpus": world,
                              "config": {"triangles": int(len(sc["F"])), "points": n_pts, "rhs": R,
                                         "iteration_ms": t_iter * 1e3, "scalar_iteration_ms": t_scalar * 1e3,
                                         "estimator": args.mrhs_bie, "path_length": base.path_length,
                                         "error_spread": spread,
                                         "mean_rmse_over_rhs": plain_curve[-1][1], "paths_per_point": plain_curve[-1][2],
                                         "curve": plain_curve[::max(1, len(plain_curve) // 10)]},
                              "clocks": clocks}), flush=True)
        scene.close()
        return
    # learned control variate: one MLP with an R-wide head trained on shared-walk density labels
    from wobtoolbox_gb300 import cv
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    mlp, info = cv.train_density_cv_multi(scene, sc["table"], base, n_train=131072, train_paths=128, steps=2000,
                                          batch=8192, lr=2e-3, seed=SEED)
    scene.set_rhs_control_variate(cv.element_cv_table(mlp, scene))
    torch.cuda.synchronize()
    t_setup = time.perf_counter() - t0
    for _ in range(args.warmup):
        scene.solve_domain_multi_cv(warm, args.mrhs_npot, d_pts, n_pts, s, None, None, None, stream)
    cv_curve, _, cv_target = progressive(
        lambda p: scene.solve_domain_multi_cv(p, args.mrhs_npot, d_pts, n_pts, s, None, b, None, stream),
        args.mrhs_budget)
    mlp.close()
    out = {
        "metric": "multi-RHS WoB: 64 RHS sharing walks, 3D interior mixed problem, 1,310,720 triangles",
        "value": bounces / total, "unit": "bounces/s (each bounce serves every RHS)",
        "n_gpus": world, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "interior mixed (Dirichlet z>0, Neumann elsewhere), "
                               + ("single layer, backward, 64 RIS candidates" if args.mrhs_bie == "sl" else
                                  "direct BIE, backward, uniform sampling")
                               + f", {base.path_length} bounces; 64 RHS of 3 exterior point sources each; "
                                 "10^6 interior points",
                   "triangles": int(len(sc["F"])), "points": n_pts, "rhs": R, "paths_per_iteration": paths,
                   "iterations": len(plain_curve), "gpu_time_s": total, "bounces": bounces,
                   "rhs_bounces_per_s": bounces * R / total,
                   "iteration_ms": {"shared_walk_64_rhs": t_iter * 1e3, "scalar_walk_1_rhs": t_scalar * 1e3},
                   "speedup_vs_separate_scalar_solves": R * t_scalar / t_iter,
                   "plain": {"mean_rmse_over_rhs": plain_curve[-1][1], "paths_per_point": plain_curve[-1][2],
                             "error_spread": spread,
                             "time_to_mean_rmse_1e-3_s (variance-only extrapolation, RMSE ~ 1/sqrt(paths); ignores the bias of the truncated series)": plain_target,
                             "curve": plain_curve[::max(1, len(plain_curve) // 10)]},
                   "learned_cv": {"potential_samples": args.mrhs_npot, "setup_s (labels + training + table)": t_setup,
                                  "train_info": info, "mean_rmse_over_rhs": cv_curve[-1][1],
                                  "paths_per_point": cv_curve[-1][2],
                                  "time_to_mean_rmse_1e-3_s (variance-only extrapolation, RMSE ~ 1/sqrt(paths); ignores the bias of the truncated series)": cv_target,
                                  "curve": cv_curve[::max(1, len(cv_curve) // 10)]},
                   "plain_over_cv_time_to_target": plain_target / (cv_target + t_setup),
                   "setup_s": {"rhs_data": t_data, "scene_build": t_build, "rhs_upload": t_rhs}},
        "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(out), flush=True)
    scene.close()


def run_build(args):
    """Scene construction: host build (wob_scene_create) vs GPU build (wob_scene_create_device) of
    the displaced icosphere with 4^subdiv * 20 triangles, and the line-intersection walk rate on
    both scenes (their BVHs differ: median-split on the host, radix tree collapsed to 4-wide on the
    GPU), measured with the 3D double-layer Dirichlet estimator on interior points."""
    import torch
    import wobtoolbox_gb300 as wob
    from wobtoolbox_gb300 import workloads as W
    rank, world, local = dist_init(args)
    wob.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    V, F, _ = W.displaced_icosphere(args.build_subdiv, 0.15, 4, SEED)
    verts, nrm = W.mesh_elements(V, F)
    n = len(F)
    bv = W.point_sources(verts.reshape(-1, 3), np.array([[3.0, 0.5, 0.0]]), np.array([1.0]))[:, 0]
    bv = bv.reshape(n, 3).astype(np.float32)
    ty = np.zeros(n, np.int32)
    t_host = []
    for _ in range(2):
        t0 = time.perf_counter()
        hs = wob.SceneHost(verts, nrm, bv, ty)
        t_host.append(time.perf_counter() - t0)
        if len(t_host) < 2:
            hs.close()
    tv, tn, tb = (torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (verts, nrm, bv))
    tt = torch.from_numpy(ty).to(dev)
    t_dev = []
    for _ in range(max(3, args.warmup)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ds = wob.SceneHost.build_on_device(tv, tn, tb, tt)
        torch.cuda.synchronize()
        t_dev.append(time.perf_counter() - t0)
        if len(t_dev) < max(3, args.warmup):
            ds.close()
    pts = inside_points(hs, 4096, -0.6, 0.6, SEED + 3, dev)
    d_pts = torch.from_numpy(pts).to(dev)
    p = wob.EstimatorParams(bie_model=wob.IndirectDoubleLayer, path_length=4, num_sample_paths=256, seed=SEED)
    rates = {}
    for name, sc in (("host_bvh", hs), ("device_bvh", ds)):
        s = torch.zeros(len(pts), 4, dtype=torch.float64, device=dev)
        b = torch.zeros(1, dtype=torch.int64, device=dev)
        sc.solve_domain(p, d_pts, len(pts), s)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        sc.solve_domain(dataclasses.replace(p, path_offset=256), d_pts, len(pts), s, None, b)
        e1.record()
        torch.cuda.synchronize()
        rates[name] = {"bounces_per_s": int(b.item()) / (e0.elapsed_time(e1) / 1e3),
                       "nodes": sc.info()["n_nodes"], "depth": sc.info()["bvh_depth"]}
    out = {"metric": "scene build time, host vs GPU", "value": min(t_host) / min(t_dev),
           "unit": "x (host build time / GPU build time)", "n_gpus": world, "higher_is_better": True,
           "config": {"workload": f"displaced icosphere, {n} triangles", "host_build_s": min(t_host),
                      "device_build_s": min(t_dev), "device_build_all_s": t_dev,
                      "line_intersection_walk (3D double layer, 4096 interior points x 256 paths x 4 bounces)": rates}}
    if rank == 0:
        print(json.dumps(out), flush=True)
    hs.close()
    ds.close()


VPL_FLOPS_PER_PAIR_2D = 60  # FP32 operations of one (point, VPL) pair: G, dG/dx, three products and sums


def run_fmad(args):
    """What the bit-exact build costs: the hot workloads with FMA contraction on. The contraction-
    enabled variant of the library (wobtoolbox_gb300/_lib/fma/, every CUDA unit with -fmad=true,
    built here on demand) runs in the same process beside the default build; each workload is timed
    on both (CUDA events, L2 flushed between steps) and the two builds' per-point estimates, drawn
    with different seeds, are compared by z-scores (the fast build is not path-for-path identical
    to the oracle, so it is validated statistically against the exact one):
      robin3d -- the headline step (timing only: the alpha = 2 series diverges);
      dl2d    -- the 2D double-layer star at 1024 paths x 8 bounces;
      fwd3d   -- the 327,680-triangle forward walk, 256 paths;
      vpl2d   -- the VPL aggregation over the same VPLs (deterministic: relative difference)."""
    import ctypes as C
    import torch
    import wobtoolbox_gb300 as wob
    from wobtoolbox_gb300 import _capi
    from wobtoolbox_gb300 import build as B
    from wobtoolbox_gb300 import workloads as W
    rank, world, local = dist_init(args)
    exact = wob.load()
    fma = _capi.load_library(B.build(fma=True))
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def make(lib, verts, normals, bvals, types, alphas=None):
        f = lambda a: None if a is None else np.ascontiguousarray(a, np.float32)
        v, n_, b_, a_ = f(verts), f(normals), f(bvals), f(alphas)
        t = np.ascontiguousarray(types, np.int32)
        h = C.c_void_p()
        st = lib.wob_scene_create(v.shape[1], len(v), v.ctypes.data, n_.ctypes.data, b_.ctypes.data,
                                  None if a_ is None else a_.ctypes.data, t.ctypes.data, C.byref(h))
        if st != 0:
            raise RuntimeError(lib.wob_last_error().decode())
        return h

    def solve(lib, h, p, d, n, s_, q_, steps, base_offset, tune):
        pc = p.to_c()
        if tune:
            chosen, nc = C.c_int32(-1), C.c_int32(0)
            ms = (C.c_float * 64)()
            lib.wob_autotune_domain(h, C.byref(pc), d.data_ptr(), n, C.byref(chosen), ms, C.byref(nc),
                                    C.c_void_p(stream.cuda_stream))
        times = []
        for k in range(steps + 1):  # launch 0 warms up; its sums are discarded
            if k == 1:
                s_.zero_()
                q_.zero_()
            flush.fill_(float(k))
            pk = dataclasses.replace(p, path_offset=base_offset + k * p.num_sample_paths).to_c()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            st = lib.wob_solve_domain(h, C.byref(pk), d.data_ptr(), n, s_.data_ptr(), q_.data_ptr(), None,
                                      C.c_void_p(stream.cuda_stream))
            e1.record(stream)
            torch.cuda.synchronize()
            if st != 0:
                raise RuntimeError(lib.wob_last_error().decode())
            if k:
                times.append(e0.elapsed_time(e1))
        return min(times)

    def compare(name, arrays, p, pts, steps, tune, z_test=True):
        d = torch.from_numpy(np.ascontiguousarray(pts)).to(dev)
        n = len(pts)
        D = pts.shape[1]
        res = {}
        stats_ = {}
        for label, lib, seed in (("exact", exact, SEED), ("fma", fma, SEED + 1)):
            h = make(lib, *arrays)
            s_ = torch.zeros(n, D + 1, dtype=torch.float64, device=dev)
            q_ = torch.zeros_like(s_)
            res[label] = solve(lib, h, dataclasses.replace(p, seed=seed), d, n, s_, q_, steps, 0, tune)
            stats_[label] = (s_[:, 0].cpu().numpy(), q_[:, 0].cpu().numpy())
            lib.wob_scene_destroy(h)
        out = {"exact_ms": res["exact"], "fma_ms": res["fma"], "speedup": res["exact"] / res["fma"]}
        if z_test:
            N = steps * p.num_sample_paths
            (sa, qa), (sb, qb) = stats_["exact"], stats_["fma"]
            ma, mb = sa / N, sb / N
            va, vb = np.maximum(qa / N - ma ** 2, 0), np.maximum(qb / N - mb ** 2, 0)
            z = (ma - mb) / np.sqrt(np.maximum(va / N + vb / N, 1e-300))
            from scipy import stats as sst
            out.update({"points": n, "paths_per_point": N, "max_abs_z": float(np.abs(z).max()),
                        "bonferroni_bound": float(sst.norm.isf(1e-3 / (2 * n))), "mean_z": float(z.mean())})
        return out

    results = {}
    sc = build_scene_arrays()
    cand = W.slice_points_z0(GRID, EXTENT)
    tmp = wob.SceneHost(sc["verts"], sc["normals"], sc["bvals"], sc["types"], sc["alphas"])
    pts = np.ascontiguousarray(cand[slice_inside(tmp, cand, dev)])
    tmp.close()
    results["robin3d"] = compare("robin3d", (sc["verts"], sc["normals"], sc["bvals"], sc["types"], sc["alphas"]),
                                 dataclasses.replace(params(), num_sample_paths=PATHS), pts, 2, True, z_test=False)
    c0 = W.star_dirichlet_scene()
    p0 = wob.EstimatorParams(bie_model=wob.IndirectDoubleLayer, domain=wob.InteriorDomain,
                             estimator=wob.BackwardEstimator, problem=wob.DirichletProblem, path_length=8,
                             num_sample_paths=1024, seed=SEED)
    results["dl2d"] = compare("dl2d", (c0["verts"], c0["normals"], c0["bvals"], c0["types"], None), p0,
                              c0["points"], 2, True)
    scene3, pts3, _, _ = exterior_neumann_case(dev, args.cv_subdiv, SEED)
    v3, n3, b3, t3, _ = scene3.stored_arrays()
    scene3.close()
    p3 = wob.EstimatorParams(bie_model=wob.IndirectSingleLayer, domain=wob.ExteriorDomain,
                             estimator=wob.ForwardEstimator, problem=wob.NeumannProblem, path_length=4, seed=SEED,
                             num_sample_paths=256)
    results["fwd3d"] = compare("fwd3d", (v3, n3, b3, t3, None), p3, pts3, 4, False)
    # VPL aggregation over one set of VPLs (from the exact build's walks), both builds
    verts, nrm, data, ty, circles = W.vpl_flow_scene()
    g, keep = W.vpl_flow_points(256, circles)
    vpts = torch.from_numpy(np.ascontiguousarray(g[keep])).to(dev)
    M = 100000
    pv = wob.EstimatorParams(bie_model=wob.IndirectSingleLayer, domain=wob.InteriorDomain,
                             estimator=wob.BackwardEstimator, problem=wob.NeumannProblem, path_length=4,
                             num_resampling_candidates=1024, eps=1e-4, seed=SEED)
    vp = torch.zeros(M, 2, dtype=torch.float32, device=dev)
    vm = torch.zeros(M, dtype=torch.float32, device=dev)
    h = make(exact, verts, nrm, data, ty)
    exact.wob_vpl_paths(h, C.byref(pv.to_c()), M, vp.data_ptr(), vm.data_ptr(), None, C.c_void_p(stream.cuda_stream))
    agg = {}
    for label, lib in (("exact", exact), ("fma", fma)):
        hh = h if lib is exact else make(fma, verts, nrm, data, ty)
        ms = []
        for k in range(4):
            sv = torch.zeros(len(vpts), 3, dtype=torch.float64, device=dev)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            lib.wob_vpl_aggregate(hh, 1e-4, vp.data_ptr(), vm.data_ptr(), M, vpts.data_ptr(), len(vpts), sv.data_ptr(),
                                  C.c_void_p(stream.cuda_stream))
            e1.record(stream)
            torch.cuda.synchronize()
            if k:
                ms.append(e0.elapsed_time(e1))
        agg[label] = (min(ms), sv[:, 0].cpu().numpy())
        if lib is fma:
            fma.wob_scene_destroy(hh)
    exact.wob_scene_destroy(h)
    rel = np.abs(agg["exact"][1] - agg["fma"][1]).max() / np.abs(agg["exact"][1]).max()
    results["vpl2d_aggregation"] = {"exact_ms": agg["exact"][0], "fma_ms": agg["fma"][0],
                                    "speedup": agg["exact"][0] / agg["fma"][0], "max_rel_diff": float(rel)}
    out = {"metric": "time per step, bit-exact build (-fmad=false) vs contraction-enabled build (-fmad=true)",
           "value": results["robin3d"]["speedup"], "unit": "x (exact time / contracted time, headline step)",
           "n_gpus": world, "higher_is_better": True, "dtype": "f32", "data": "synthetic",
           "config": {"workload": "headline robin3d, dl2d (2D double-layer star), fwd3d (327,680-triangle forward walk), "
                                  "VPL aggregation",
                      "note": "per-point estimates of the two builds drawn with different seeds; z = difference / "
                              "combined standard error"},
           "results": results}
    if rank == 0:
        print(json.dumps(out), flush=True)


def run_vpl(args):
    """VPL potential flow (apps/potential_flow_with_vpl.cu with data/config_potential_flow_with_vpl.json:
    100,000 paths per iteration, 4 bounces, 1024 RIS candidates, eps 1e-4, 256^2 grid minus the four
    obstacles): per iteration the VPL walks and the dense aggregation over every (point, VPL) pair,
    each timed with CUDA events. The aggregation is FP32-issue bound; its roofline is the FP32 FMA
    rate 2 x 152 SMs x 128 lanes x SM clock (the bit-exact build keeps every product and sum
    separately rounded, so half of that is its ceiling; --workload fmad measures the difference)."""
    import torch
    import wobtoolbox_gb300 as wob
    from wobtoolbox_gb300 import workloads as W
    rank, world, local = dist_init(args)
    wob.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    verts, nrm, data, ty, circles = W.vpl_flow_scene()
    scene = wob.SceneHost(verts, nrm, data, ty)
    g, keep = W.vpl_flow_points(256, circles)
    pts = np.ascontiguousarray(g[keep])
    n_pts = len(pts)
    d_pts = torch.from_numpy(pts).to(dev)
    M = args.vpl_paths
    base = wob.EstimatorParams(bie_model=wob.IndirectSingleLayer, domain=wob.InteriorDomain,
                               estimator=wob.BackwardEstimator, problem=wob.NeumannProblem, path_length=4,
                               num_resampling_candidates=1024, eps=1e-4, seed=SEED)
    vp = torch.zeros(M, 2, dtype=torch.float32, device=dev)
    vm = torch.zeros(M, dtype=torch.float32, device=dev)
    s = torch.zeros(n_pts, 3, dtype=torch.float64, device=dev)
    b = torch.zeros(1, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    t_paths, t_agg = [], []
    sampler = ClockSampler(torch.cuda.current_device())
    for it in range(args.warmup + args.steps):
        if it == args.warmup:
            torch.cuda.synchronize()
            s.zero_()
            b.zero_()
            sampler.__enter__()
        p = dataclasses.replace(base, path_offset=it * M)
        ev[0].record(stream)
        scene.vpl_paths(p, M, vp, vm, b, stream)
        ev[1].record(stream)
        scene.vpl_aggregate(base.eps, vp, vm, M, d_pts, n_pts, s, stream)
        ev[2].record(stream)
        torch.cuda.synchronize()
        if it >= args.warmup:
            t_paths.append(ev[0].elapsed_time(ev[1]) / 1e3)
            t_agg.append(ev[1].elapsed_time(ev[2]) / 1e3)
    sampler.__exit__(None, None, None)
    clocks = sampler.summary()
    pairs = float(n_pts) * M
    agg = sum(t_agg) / len(t_agg)
    pth = sum(t_paths) / len(t_paths)
    mhz = clocks.get("sm_mhz") or 2070.0
    peak = 2 * 152 * 128 * mhz * 1e6 / 1e12  # FP32 with FMA counted as two operations
    achieved = pairs * VPL_FLOPS_PER_PAIR_2D / agg / 1e12
    u = (s[:, 0] / (args.steps * M)).cpu().numpy()
    gx = (s[:, 1] / (args.steps * M)).cpu().numpy()
    out = {"metric": "VPL potential flow: (point, VPL) pairs per second of the aggregation",
           "value": pairs / agg, "unit": "pairs/s", "n_gpus": world, "higher_is_better": True, "dtype": "f32",
           "data": "synthetic",
           "config": {"workload": "box with 4 circular obstacles, 814 segments, SL backward Neumann, 4 bounces, "
                                  "1024 RIS candidates; 256^2 grid outside the obstacles",
                      "points": n_pts, "vpl_per_iteration": M, "iterations": args.steps,
                      "iteration_ms": {"vpl_walks": pth * 1e3, "aggregation": agg * 1e3},
                      "walk_bounces_per_s": int(b.item()) / sum(t_paths),
                      "mean_grad_x_far_field": float(np.mean(gx[np.abs(pts[:, 1]) > 0.45]))},
           "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s (FP32)",
                        "frac": achieved / peak, "flops_per_pair": VPL_FLOPS_PER_PAIR_2D,
                        "peak_source": "152 SMs x 128 FP32 lanes x 2 (FMA) x median SM clock during the run; "
                                       "the bit-exact build issues no FMA, so half of this is its ceiling"},
           "clocks": clocks}
    if rank == 0:
        print(json.dumps(out), flush=True)
    scene.close()


def run_wos(args):
    """WoB vs walk on spheres (apps/simple_wob_and_wos.cu) on the 2D star workload (1024 segments,
    g = e^x cos y, 7,960 interior points): the double-layer WoB of the headline 2D workload (8
    bounces) and WoS with eps 1e-4, each run as progressive iterations for --wos-budget GPU seconds;
    RMSE against the exact solution is recorded against cumulative GPU time."""
    import torch
    import wobtoolbox_gb300 as wob
    from wobtoolbox_gb300 import workloads as W
    rank, world, local = dist_init(args)
    wob.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    sc = W.star_dirichlet_scene()
    scene = wob.SceneHost(sc["verts"], sc["normals"], sc["bvals"], sc["types"], sc["alphas"])
    pts = sc["points"]
    n_pts = len(pts)
    exact = W.exp_cos(pts)[:, 0]
    d_pts = torch.from_numpy(pts).to(dev)
    stream = torch.cuda.current_stream()
    wob_p = wob.EstimatorParams(bie_model=wob.IndirectDoubleLayer, path_length=8, num_sample_paths=256, seed=SEED)
    wos_p = wob.EstimatorParams(num_sample_paths=256, eps=1e-4, seed=SEED)

    def progressive(solve, params, width):
        s = torch.zeros(n_pts, width, dtype=torch.float64, device=dev)
        q = torch.zeros(1, dtype=torch.int64, device=dev)
        for _ in range(args.warmup):
            solve(dataclasses.replace(params, path_offset=1 << 40), s, q)
        torch.cuda.synchronize()
        s.zero_()
        q.zero_()
        curve, total, k = [], 0.0, 0
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        while total < args.wos_budget and k < 100000:
            e0.record(stream)
            solve(dataclasses.replace(params, path_offset=k * params.num_sample_paths), s, q)
            e1.record(stream)
            torch.cuda.synchronize()
            total += e0.elapsed_time(e1) / 1e3
            k += 1
            u = (s[:, 0] / (k * params.num_sample_paths)).cpu().numpy()
            curve.append((total, float(np.sqrt(np.mean((u - exact) ** 2))), k * params.num_sample_paths))
        return curve, int(q.item())

    wob_curve, wob_b = progressive(lambda p, s, q: scene.solve_domain(p, d_pts, n_pts, s, None, q, stream), wob_p, 3)
    wos_curve, wos_q = progressive(lambda p, s, q: scene.solve_wos(p, d_pts, n_pts, s, None, q, None, stream), wos_p, 1)
    target = max(wob_curve[-1][1], wos_curve[-1][1]) * 1.0001

    def time_to(curve):
        for t_s, r, _ in curve:
            if r <= target:
                return t_s
        return None

    tw, ts = time_to(wob_curve), time_to(wos_curve)
    out = {"metric": "WoB vs walk on spheres, time to a common RMSE (2D star, 1024 segments)",
           "value": (ts / tw) if (tw and ts) else None, "unit": "x (WoS time / WoB time to the common RMSE)",
           "n_gpus": world, "higher_is_better": True, "dtype": "f32", "data": "synthetic",
           "config": {"workload": "2D interior Dirichlet star r = 1 + 0.3 cos 5t, g = e^x cos y, 7960 points",
                      "rmse_target": target, "wob_time_s": tw, "wos_time_s": ts,
                      "wob": {"paths_per_s": wob_curve[-1][2] * n_pts / wob_curve[-1][0],
                              "bounces_per_s": wob_b / wob_curve[-1][0], "final": wob_curve[-1]},
                      "wos": {"paths_per_s": wos_curve[-1][2] * n_pts / wos_curve[-1][0],
                              "closest_point_queries_per_s": wos_q / wos_curve[-1][0],
                              "queries_per_path": wos_q / (wos_curve[-1][2] * n_pts), "final": wos_curve[-1]},
                      "wob_curve": wob_curve[::max(1, len(wob_curve) // 8)],
                      "wos_curve": wos_curve[::max(1, len(wos_curve) // 8)]}}
    if rank == 0:
        print(json.dumps(out), flush=True)
    scene.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-points", type=int, default=8192, help="CPU baseline sample (inside points)")
    ap.add_argument("--cpu-paths", type=int, default=PATHS)
    ap.add_argument("--ref-points", type=int, default=768, help="points per step of --impl reference")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--small", action="store_true", help="profiling case: 1/16 of the points, 512 paths")
    ap.add_argument("--workload", choices=["robin3d", "dl2d", "batch2d", "cv3d", "fwd3d", "mrhs3d", "build3d",
                                           "vpl2d", "wos2d", "fmad"],
                    default="robin3d",
                    help="robin3d: the headline 3D Robin icosphere workload; dl2d: 2D double-layer star; "
                         "batch2d: 256 batched 2D scenes vs sequential launches")
    ap.add_argument("--batch-paths", type=int, default=32, help="paths per point of --workload batch2d")
    ap.add_argument("--batch-points-min", type=int, default=1000)
    ap.add_argument("--batch-points-max", type=int, default=64000)
    ap.add_argument("--cv-subdiv", type=int, default=7, help="icosphere subdivision of --workload cv3d")
    ap.add_argument("--cv-paths", type=int, default=256, help="plain paths per point per iteration of --workload cv3d")
    ap.add_argument("--cv-budget", type=float, default=20.0, help="seconds per estimator of --workload cv3d")
    ap.add_argument("--cv-near", type=float, default=3.0, help="near-field factor of the control-variate tables")
    ap.add_argument("--cv-theta", type=float, default=0.3,
                    help="cluster acceptance of the control-variate tables' far field (0: every triangle)")
    ap.add_argument("--fwd-paths", type=int, default=256, help="paths per point per step of --workload fwd3d")
    ap.add_argument("--fwd-config", type=int, default=-1,
                    help="--workload fwd3d: kernel configuration (0 lockstep; 1-3 + 4k wavefront; -1 autotune)")
    ap.add_argument("--no-time-to-rmse", action="store_true",
                    help="skip the plain vs learned-CV time-to-RMSE leg of the default workload")
    ap.add_argument("--mrhs-subdiv", type=int, default=8, help="icosphere subdivision of --workload mrhs3d")
    ap.add_argument("--mrhs-rhs", type=int, default=64)
    ap.add_argument("--mrhs-points", type=int, default=1000000)
    ap.add_argument("--mrhs-paths", type=int, default=32, help="paths per point per iteration of --workload mrhs3d "
                                                                "(a warp runs 32 paths of one point)")
    ap.add_argument("--mrhs-budget", type=float, default=20.0, help="GPU seconds per estimator of --workload mrhs3d")
    ap.add_argument("--mrhs-npot", type=int, default=4, help="potential samples of the learned CV (mrhs3d)")
    ap.add_argument("--mrhs-plain-only", action="store_true", help="mrhs3d without the learned-CV leg (profiling)")
    ap.add_argument("--mrhs-bie", choices=["sl", "direct"], default="sl",
                    help="mrhs3d estimator: single layer + RIS 64 (the reference's Mixed config) or direct, uniform")
    ap.add_argument("--mrhs-path-length", type=int, default=0, help="mrhs3d bounces (0: 4)")
    ap.add_argument("--build-subdiv", type=int, default=8, help="icosphere subdivision of --workload build3d")
    ap.add_argument("--vpl-paths", type=int, default=100000, help="VPL walks per iteration of --workload vpl2d")
    ap.add_argument("--wos-budget", type=float, default=5.0, help="GPU seconds per method of --workload wos2d")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch2d":
        run_batch(args)
    elif args.workload == "cv3d":
        run_cv(args)
    elif args.workload == "fwd3d":
        run_fwd3d(args)
    elif args.workload == "mrhs3d":
        run_multi_rhs(args)
    elif args.workload == "build3d":
        run_build(args)
    elif args.workload == "vpl2d":
        run_vpl(args)
    elif args.workload == "wos2d":
        run_wos(args)
    elif args.workload == "fmad":
        run_fmad(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
