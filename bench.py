#!/usr/bin/env python
"""Benchmark of the GB300 PO engine.

Headline workload (default; one step = one full solve): the synthetic fiber
segment -- elliptical cross-section 25 x 20 um, 60 um long, cuticle sawtooth
(5 um scales, 0.4 um step, 3 degree tilt) and seeded Gaussian height noise
(sigma 0.05 um, correlation 1 um), sampled at 0.05 um (3.40M points) by the
GPU height-field sampler; index 1.55+0.1i, 25 wavelengths 400 + 12 i nm
(i = 0..24, the reference's even spacing, compareMie/sphere.cu:489), 64
incidences (theta sweep at phi = 0, fibersim/treePO.cu:559-564), TM, octree
depth 7 with the reference's level grids (fibersim/treePO.cu:353-373),
output 180 x 360; split hi+lo BF16 tensor-core leaf products with FP32
accumulation and FP64 phase arguments, double-cover theta interpolation.
The same line carries the plain FP64 direct sum on the same GPU (timed on
the full point set for one pattern, scaled by the pattern count), the
end-to-end time through po_solve with host buffers, the roofline of the
dominant kernel class and the FP64 oracle on the host cores.

Other workloads (--workload): ellipsoid (8 x 5 x 5 um, 400k points, 25
wavelengths, depth 5), cylinder-grad (the gradient of ||I(h) - I_t||^2 with
respect to a displacement field), batch (256 independent solves in one CUDA
graph).

Metric: Gpoint-dirs/s = N * 180*360 * L * I * P / time / 1e9 (the equivalent
depth-0 count), plus patterns/s; accuracy is the rel-L2 of intensity against
the FP64 direct sum.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--workload W]

`--impl reference` times the reference path's CPU implementation: the
reference ships CUDA only, so this is the FP64 direct-sum restatement of its
algorithm (oracle/) on all host cores, on a bounded direction sample of the
same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

RADII = (8e-6, 5e-6, 5e-6)
N_POINTS = 400_000
N_THETA, N_PHI = 180, 360
DEPTH = 5
LAMBDAS = [(400.0 + 12.0 * i) * 1e-9 for i in range(25)]
ETA = 1.55 + 0.1j
SIGMA = 1e-2
WORKLOAD = "ellipsoid 8x5x5um, 400k points, depth 5, 25 wavelengths x 1 incidence x TM, 180x360 grid"


PRECISIONS = {"fp32": 0, "split_bf16": 2}
INTERP = {"fft": 0, "tensor": 1}
THETA_MODES = {"double_cover": 0, "reference": 1}


def make_workload(precision: str = "fp32", interp: str = "tensor", tile: int = 0, n_lambda: int = 25,
                  n_inc: int = 1, theta_mode: str = "double_cover"):
    from wavefiber3d_gb300 import api, geometry
    cloud = geometry.ellipsoid(RADII, N_POINTS)
    bmin = [-1.1 * r for r in RADII]
    bmax = [1.1 * r for r in RADII]
    cfg = api.Config.reference_rule(DEPTH, N_THETA, N_PHI, bmin, bmax, 16e-6, 16e-6, 1.3,
                                    precision=PRECISIONS[precision], interp_method=INTERP[interp],
                                    interp_tile=tile, theta_mode=THETA_MODES[theta_mode])
    # one incidence along +x (the workload); more for profiling runs: a theta sweep at phi = 0.3
    th = [0.0] if n_inc == 1 else list(np.linspace(-1.0, 1.0, n_inc))
    ph = [0.0] if n_inc == 1 else [0.3] * n_inc
    illum = api.Illumination(LAMBDAS[:n_lambda], th, ph, api.PO_POL_TM, ETA, SIGMA)
    return cloud, cfg, illum


def point_dirs_per_step(illum) -> float:
    return float(N_POINTS) * N_THETA * N_PHI * illum.n_patterns


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(v: float, world: int) -> float:
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sample_directions(k: int, seed: int = 20231203) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(N_THETA * N_PHI, size=k, replace=False)).astype(np.int64)


def cpu_direct_sample(cloud, lam, dirs, theta_i=0.0, phi_i=0.0):
    """FP64 oracle direct sum (all host cores) on the sampled directions; returns
    (intensity, seconds, threads)."""
    import oracle
    il = oracle.make_illum(lam, theta_i, phi_i, "M", ETA, SIGMA)
    t0 = time.perf_counter()
    cur = oracle.currents(cloud, il)
    f = oracle.far_field_sampled(cloud, cur, 2 * math.pi / lam, [0.0, 0.0, 0.0], N_THETA, N_PHI, dirs)
    inten = oracle.intensity_sampled(f, N_THETA, N_PHI, dirs)
    return inten, time.perf_counter() - t0, oracle.num_threads()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during a
    timed region: the sampler is live (first line written) before the region
    starts and only lines written after that count; a region shorter than the
    period gets one immediate sample when it ends."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.path = Path(tempfile.mkstemp(prefix="clocks_", suffix=".csv")[1])
        self.gpu_index = gpu_index
        self.proc = None
        self.skip = 0
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={gpu_index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        if self.proc is not None:
            t0 = time.perf_counter()
            while time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
                if self.path.stat().st_size > 0:
                    break
                time.sleep(0.02)
            self.skip = len(self.path.read_text().splitlines())

    @staticmethod
    def parse(lines):
        """(sm MHz list, max MHz list, active slowdown reasons) of nvidia-smi CSV lines."""
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return sm, mx, reasons

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        lines = self.path.read_text().splitlines()[self.skip:]
        if not self.parse(lines)[0]:
            try:
                r = subprocess.run(["nvidia-smi", f"--id={self.gpu_index}", f"--query-gpu={self.Q}",
                                    "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=20)
                lines = r.stdout.splitlines()
            except (FileNotFoundError, OSError, subprocess.TimeoutExpired):
                lines = []
        sm, mx, reasons = self.parse(lines)
        self.path.unlink(missing_ok=True)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def run_engine(args, world, rank, local):
    import torch

    from wavefiber3d_gb300 import api
    import __graft_entry__
    __graft_entry__.build()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    bf16_peak = peaks.get("bf16_tflops", 1900.0)
    peak_src = "measured" if peaks else "fallback"

    cloud, cfg, illum = make_workload(args.precision, args.interp, args.interp_tile, args.lambdas, args.incidences,
                                      args.theta_mode)
    pd_step = point_dirs_per_step(illum)
    st = torch.cuda.current_stream()
    g_dev = torch.from_numpy(cloud.soa()).to(dev)
    geom_dev = tuple(g_dev[k] for k in range(7))
    g_host = torch.from_numpy(cloud.soa()).pin_memory()
    geom_host = tuple(g_host[k] for k in range(7))
    solver = api.Solver(cfg)
    shape = solver.out_shape(illum)
    out_dev = torch.empty(shape, dtype=torch.float32, device=dev)
    out_host = torch.empty(shape, dtype=torch.float32).pin_memory()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # 256 MiB > 129 MB L2

    for _ in range(args.warmup):
        solver.solve(geom_dev, illum, out=out_dev)
    torch.cuda.synchronize()

    # ---- device-resident timed region
    reps = []
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    barrier(world)
    torch.cuda.synchronize()
    t_wall0 = time.perf_counter()
    for i in range(args.steps):
        flush.zero_()
        evs[i][0].record(st)
        # no report inside the timed steps: a report makes the call wait for the solve, and host
        # scheduling between its end and the next event would land inside the step
        solver.solve(geom_dev, illum, out=out_dev, report=False)
        evs[i][1].record(st)
    torch.cuda.synchronize()
    barrier(world)
    t_wall = time.perf_counter() - t_wall0
    clk = clocks.stop()
    # per-kernel-class breakdown: the same solve with its report (events inside the solve), untimed
    for _ in range(3):
        flush.zero_()
        solver.solve(geom_dev, illum, out=out_dev)
        reps.append(dict(solver.last_report))
    ms_steps = [a.elapsed_time(b) for a, b in evs]
    ms_step = sum(ms_steps) / args.steps
    ms_step_max = max_over_ranks(ms_step, world)

    # ---- end to end through the C ABI with host buffers (H2D + D2H inside)
    e2e_ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier(world)
    torch.cuda.synchronize()
    for i in range(args.steps):
        flush.zero_()
        e2e_ev[i][0].record(st)
        solver.solve(geom_host, illum, out=out_host)
        e2e_ev[i][1].record(st)
    torch.cuda.synchronize()
    barrier(world)
    e2e_ms = max_over_ranks(sum(a.elapsed_time(b) for a, b in e2e_ev) / args.steps, world)

    # ---- roofline of the dominant kernel class (CUDA events inside the solve)
    r = reps[-1]
    classes = {
        "leaf far-field sums": (statistics.mean(x["ms_leaf_kernel"] for x in reps), r["n_leaf_launches"]),
        "row (phi) interpolation": (statistics.mean(x["ms_rows"] for x in reps), r["n_row_launches"]),
        "column (theta) interpolation + translation + child sum":
            (statistics.mean(x["ms_cols"] for x in reps), r["n_col_launches"]),
    }
    dom = max(classes, key=lambda k: classes[k][0])
    ms_dom, n_dom = classes[dom]
    if dom.startswith("leaf"):
        flops = r["leaf_point_dirs"] * (8 * 6 + 5)
        achieved = flops / n_dom / (ms_dom / n_dom * 1e-3) / 1e12
        roof = {"bound": "tensor", "kernel": dom, "achieved": achieved, "peak": bf16_peak, "unit": "TFLOP/s",
                "frac": achieved / bf16_peak, "traffic": None,
                "note": f"FP32 CUDA-core kernel; algorithmic flops = point-dirs x 53; peak = {peak_src} bf16 dense"}
    else:
        key = "rows_bytes" if dom.startswith("row") else "cols_bytes"
        achieved = r[key] / (ms_dom * 1e-3) / 1e9
        roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak, "traffic": None,
                "note": f"algorithmic bytes = child patterns read + parent patterns written; peak = {peak_src} copy"}

    # ---- accuracy and the CPU baseline (rank 0 only)
    result = None
    if rank == 0:
        dirs = sample_directions(args.cpu_dirs)
        cpu_inten, cpu_s, threads = cpu_direct_sample(cloud, LAMBDAS[0], dirs, illum.theta_i[0], illum.phi_i[0])
        gpu_inten = out_dev[0, 0, 0].reshape(-1).cpu().numpy()[dirs].astype(np.float64)
        acc = float(np.linalg.norm(gpu_inten - cpu_inten) / np.linalg.norm(cpu_inten))
        cpu_value = N_POINTS * dirs.size / cpu_s / 1e9
        value = pd_step * world / (ms_step_max * 1e-3) / 1e9
        result = {
            "metric": "Gpoint-dirs/s (equivalent depth-0 point x direction terms) at rel-L2<=1e-3 vs FP64 direct sum",
            "value": value,
            "unit": "Gpoint-dirs/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": ms_step_max,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32 (f64 phase arguments)" if args.precision == "fp32" else
                     "split bf16 hi+lo leaf products, f32 accumulation (f64 phase arguments)",
            "data": "synthetic (seeded ellipsoid, analytic normals)",
            "config": {"workload": WORKLOAD, "points": N_POINTS, "directions": N_THETA * N_PHI,
                       "wavelengths": len(illum.wavelengths_m), "incidences": len(illum.theta_i), "polarisations": 1,
                       "depth": DEPTH,
                       "level_grids": [list(cfg.n_theta), list(cfg.n_phi)],
                       "theta_mode": args.theta_mode.replace("_", " "),
                       "precision": args.precision, "theta_interpolation": args.interp,
                       "theta_tile": args.interp_tile,
                       "l2": "flushed between steps (256 MiB write, outside the timed events)",
                       "parallelism": f"replicas x{world}"},
            "patterns_per_s": illum.n_patterns * world / (ms_step_max * 1e-3),
            "rel_l2_vs_fp64": acc,
            "accuracy_sample": f"{dirs.size} seeded directions of lambda={LAMBDAS[0] * 1e9:.0f} nm",
            "e2e": {"value": pd_step * world / (e2e_ms * 1e-3) / 1e9, "unit": "Gpoint-dirs/s",
                    "ms_per_step": e2e_ms, "h2d_bytes_per_step": int(g_host.numel() * 4),
                    "d2h_bytes_per_step": int(out_host.numel() * 4)},
            "roofline": roof,
            "kernel_ms_per_step": {k: v[0] for k, v in classes.items()},
            "cpu_baseline": {"value": cpu_value, "unit": "Gpoint-dirs/s", "cores": threads, "kind": "port",
                             "sample": f"FP64 direct sum, {N_POINTS} points x {dirs.size} directions, 1 wavelength",
                             "seconds": cpu_s},
            "gpu_launches": int(args.steps * r["kernel_launches"]),  # launches per solve are fixed
            "clocks": clk,
            "wall_s_timed_region": t_wall,
            "report": r,
        }
    solver.close()
    return result


# ---------------------------------------------------------------- fiber workload
FIBER_RADII = (25e-6, 20e-6)
FIBER_LENGTH = 60e-6
FIBER_DEPTH = 7
FIBER_SIGMA = 10e-6          # Gaussian beam width of the reference's fiber presets 0/1 (treePO.cu:47)
FIBER_INC = 64               # theta sweep at phi_i = 0: theta_i = -pi/2 + 1e-10 + pi/180 * idx, idx = 58..121
FIBER_SEED = 11
FIBER_WORKLOAD = ("fiber segment 25x20um x 60um, cuticle 5um/0.4um/3deg + Gaussian noise 0.05um/1um, "
                  "0.05um spacing (3.40M points), depth 7, 25 wavelengths x 64 incidences x TM, 180x360 grid")
FIBER_BOX_MIN = [-1.1 * FIBER_RADII[0], -1.1 * FIBER_RADII[1], -0.55 * FIBER_LENGTH]  # treePO.cu:96-98
FIBER_BOX_MAX = [-v for v in FIBER_BOX_MIN]
# DRAM bytes per algorithmic byte of the aggregation passes, from the ncu capture summarised in
# profiles/aggregation_traffic_fiber_8inc.md (dram__bytes_read.sum + dram__bytes_write.sum of every phi
# and theta launch of one 8-incidence solve of this workload, 165.45 GB, over the per-level
# algorithmic bytes of the same solve, 49.42 GB)
FIBER_AGG_TRAFFIC_RATIO = 154.19 / 49.25


def fiber_incidences(n: int = FIBER_INC):
    idx = np.arange(58, 58 + n)
    return list(-math.pi / 2 + 1e-10 + math.pi / 180 * idx), [0.0] * n


def fiber_config(precision: str, interp: str = "tensor", workspace_gb: float = 0.0):
    from wavefiber3d_gb300 import api
    return api.Config.reference_rule(FIBER_DEPTH, N_THETA, N_PHI, FIBER_BOX_MIN, FIBER_BOX_MAX, FIBER_LENGTH,
                                     2 * max(FIBER_RADII), 1.2, precision=PRECISIONS[precision],
                                     interp_method=INTERP[interp],
                                     max_workspace_bytes=int(workspace_gb * 1e9))  # treePO.cu:353-359


def run_fiber(args, world, rank, local):
    """Config 3, the headline: the split-precision hierarchical solve of the
    3.4M-point fiber segment over 25 wavelengths x 64 incidences per step,
    against the plain FP64 direct sum on the same GPU (B1, timed on the full
    point set for one (wavelength, incidence) pair and scaled by the pattern
    count) and the FP64 oracle on the host cores."""
    import torch

    from wavefiber3d_gb300 import api, geometry
    import __graft_entry__
    __graft_entry__.build()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    st = torch.cuda.current_stream()
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    bf16_peak = peaks.get("bf16_tflops_sustained", 1700.0)
    peak_src = "measured" if peaks else "fallback"
    hf = geometry.fiber_height_field(FIBER_RADII, FIBER_LENGTH, seed=FIBER_SEED)
    t0 = time.perf_counter()
    g_dev = api.height_field_points(hf)  # the GPU height-field sampler (util/geometry.h:76-179)
    torch.cuda.synchronize()
    t_geom = time.perf_counter() - t0
    n = g_dev.shape[1]
    geom_dev = tuple(g_dev[k] for k in range(7))
    g_host = g_dev.cpu().pin_memory()
    geom_host = tuple(g_host[k] for k in range(7))
    lams = LAMBDAS[: args.fiber_lambdas]
    n_inc = max(1, min(FIBER_INC, args.fiber_incidences))
    th, ph = fiber_incidences(n_inc)
    illum = api.Illumination(lams, th, ph, api.PO_POL_TM, ETA, FIBER_SIGMA)
    cfg = fiber_config(args.precision, args.interp, args.workspace_gb)
    solver = api.Solver(cfg)
    out = torch.empty(solver.out_shape(illum), dtype=torch.float32, device=dev)
    out_host = torch.empty(solver.out_shape(illum), dtype=torch.float32).pin_memory()
    pd_step = float(n) * N_THETA * N_PHI * illum.n_patterns

    for _ in range(args.warmup):
        solver.solve(geom_dev, illum, out=out, report=False)
    torch.cuda.synchronize()

    # ---- device-resident timed region (inputs, tree and level buffers are far larger than L2)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    barrier(world)
    torch.cuda.synchronize()
    t_wall0 = time.perf_counter()
    for i in range(args.steps):
        evs[i][0].record(st)
        solver.solve(geom_dev, illum, out=out, report=False)
        evs[i][1].record(st)
    torch.cuda.synchronize()
    barrier(world)
    t_wall = time.perf_counter() - t_wall0
    clk = clocks.stop()
    ms_step = statistics.mean(a.elapsed_time(b) for a, b in evs)
    ms_step_max = max_over_ranks(ms_step, world)

    # ---- per-kernel-class breakdown: one more solve with its report (events inside the solve), untimed
    solver.solve(geom_dev, illum, out=out)
    r = dict(solver.last_report)

    # ---- end to end through the C ABI with host buffers (geometry H2D and intensity D2H inside)
    n_e2e = max(1, min(args.steps, args.e2e_steps))
    e2e_ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n_e2e)]
    barrier(world)
    torch.cuda.synchronize()
    for i in range(n_e2e):
        e2e_ev[i][0].record(st)
        solver.solve(geom_host, illum, out=out_host, report=False)
        e2e_ev[i][1].record(st)
    torch.cuda.synchronize()
    barrier(world)
    e2e_ms = max_over_ranks(statistics.mean(a.elapsed_time(b) for a, b in e2e_ev), world)
    e2e_same = bool(torch.equal(out_host, out.cpu()))
    solver.close()
    result = None
    if rank != 0:
        return None

    # ---- plain FP64 direct sum on the same GPU (B1): full point set, one (wavelength, incidence) pair
    cfg64 = api.Config(0, [N_THETA], [N_PHI], FIBER_BOX_MIN, FIBER_BOX_MAX, precision=api.PO_PREC_FP64)
    il64 = api.Illumination(lams[:1], th[:1], ph[:1], api.PO_POL_TM, ETA, FIBER_SIGMA)
    with api.Solver(cfg64) as s64:
        o64 = torch.empty(s64.out_shape(il64), dtype=torch.float32, device=dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        s64.solve(geom_dev, il64, out=o64, report=False)
        e1.record(st)
        torch.cuda.synchronize()
        ms64_pair = e0.elapsed_time(e1)
    ms64_full = ms64_pair * illum.n_patterns  # linear in the pattern count (one sum per pattern)
    ref64 = o64[0, 0, 0].double()
    rel_full_grid = float((out[0, 0, 0].double() - ref64).norm() / ref64.norm())

    # ---- accuracy against the FP64 oracle on the host (two incidences, sampled directions)
    import oracle
    cloud = geometry.PointCloud.from_soa(g_host.numpy())
    dirs = sample_directions(args.fiber_dirs)
    errs = []
    ctr = [0.5 * (a + b) for a, b in zip(np.float32(FIBER_BOX_MIN), np.float32(FIBER_BOX_MAX))]
    for ii in sorted({0, n_inc - 1}):
        il = oracle.make_illum(lams[0], th[ii], ph[ii], "M", ETA, FIBER_SIGMA)
        cur = oracle.currents(cloud, il)
        f = oracle.far_field_sampled(cloud, cur, 2 * math.pi / lams[0], ctr, N_THETA, N_PHI, dirs)
        ref = oracle.intensity_sampled(f, N_THETA, N_PHI, dirs)
        got = out[0, ii, 0].reshape(-1).cpu().numpy()[dirs].astype(np.float64)
        errs.append(float(np.linalg.norm(got - ref) / np.linalg.norm(ref)))

    # ---- CPU baseline: the FP64 oracle direct sum on all host cores, bounded direction sample
    cdirs = sample_directions(args.cpu_dirs, seed=5)
    il = oracle.make_illum(lams[0], th[0], ph[0], "M", ETA, FIBER_SIGMA)
    t0 = time.perf_counter()
    cur = oracle.currents(cloud, il)
    f = oracle.far_field_sampled(cloud, cur, 2 * math.pi / lams[0], ctr, N_THETA, N_PHI, cdirs)
    oracle.intensity_sampled(f, N_THETA, N_PHI, cdirs)
    cpu_s = time.perf_counter() - t0
    cpu_value = float(n) * cdirs.size / cpu_s / 1e9

    # ---- roofline of the dominant kernel class (CUDA events inside the solve)
    agg_ms = r["ms_rows"] + r["ms_cols"]
    classes = {"leaf far-field contraction": r["ms_leaf_kernel"],
               "aggregation (phi + theta passes, translation, child sums)": agg_ms}
    dom = max(classes, key=classes.get)
    if dom.startswith("leaf"):
        flops = r["leaf_point_dirs"] * (8 * 6 + 5)
        achieved = flops / (r["ms_leaf_kernel"] * 1e-3) / 1e12
        roof = {"bound": "tensor", "kernel": dom, "achieved": achieved, "peak": bf16_peak, "unit": "TFLOP/s",
                "frac": achieved / bf16_peak, "traffic": None,
                "note": f"algorithmic flops = leaf point-directions x (8 x 6 + 5); peak = {peak_src} sustained bf16 "
                        "dense (the hi/lo split products are not counted as work)"}
    else:
        achieved = r["agg_bytes"] / (agg_ms * 1e-3) / 1e9
        traffic = None if FIBER_AGG_TRAFFIC_RATIO is None else FIBER_AGG_TRAFFIC_RATIO * r["agg_bytes"]
        roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak, "traffic": traffic,
                "note": "algorithmic bytes = per level, the child patterns read at the child grid + the parent "
                        f"patterns written (8 B per complex sample); peak = {peak_src} copy bandwidth; traffic = "
                        "ncu DRAM bytes per algorithmic byte of an 8-incidence capture of the same kernels "
                        "(profiles/aggregation_traffic_fiber_8inc.md) times this step's algorithmic bytes"}
    result = {
        "metric": "Gpoint-dirs/s (equivalent depth-0 point x direction terms) at rel-L2<=1e-3 vs FP64 direct sum",
        "value": pd_step * world / (ms_step_max * 1e-3) / 1e9,
        "unit": "Gpoint-dirs/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_step_max, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "split bf16 hi+lo tensor-core products, f32 accumulation (f64 phase arguments)"
                 if args.precision == "split_bf16" else "f32 (f64 phase arguments)",
        "data": "synthetic (seeded fiber height field, sampled on the GPU)",
        "config": {"workload": FIBER_WORKLOAD, "points": n, "numel": hf.numel, "numelvert": hf.numelvert,
                   "wavelengths": len(lams), "incidences": n_inc, "polarisations": 1, "depth": FIBER_DEPTH,
                   "directions": N_THETA * N_PHI, "level_grids": [list(cfg.n_theta), list(cfg.n_phi)],
                   "precision": args.precision, "theta_mode": "double cover", "theta_interpolation": args.interp,
                   "beam_sigma_m": FIBER_SIGMA,
                   "workspace_cap_gb": args.workspace_gb if args.workspace_gb > 0 else "half the device",
                   "l2": "no flush: inputs (95 MB), tree and level buffers (>100 GB) are far larger than L2",
                   "parallelism": f"replicas x{world}"},
        "patterns_per_s": illum.n_patterns * world / (ms_step_max * 1e-3),
        "e2e": {"value": pd_step * world / (e2e_ms * 1e-3) / 1e9, "unit": "Gpoint-dirs/s", "ms_per_step": e2e_ms,
                "steps": n_e2e, "h2d_bytes_per_step": int(g_host.numel() * 4),
                "d2h_bytes_per_step": int(out_host.numel() * 4), "equals_device_output": e2e_same,
                "path": "po_solve with host geometry and host intensity (copies inside the call)"},
        "plain_fp64_gpu": {"ms_per_pattern_measured": ms64_pair, "ms_per_step_scaled": ms64_full,
                           "value": pd_step / (ms64_full * 1e-3) / 1e9,
                           "note": f"FP64 depth-0 sum (k_direct_f64) over all {n} points and 64800 directions for "
                                   f"lambda={lams[0] * 1e9:.0f} nm, incidence 0; scaled by the "
                                   f"{illum.n_patterns} patterns of a step"},
        "speedup_vs_plain_fp64_gpu": ms64_full / ms_step_max,
        "rel_l2_vs_fp64": max(errs + [rel_full_grid]),
        "rel_l2_vs_fp64_gpu_full_grid": rel_full_grid,
        "rel_l2_vs_fp64_oracle_per_incidence": errs,
        "accuracy_sample": f"all 64800 directions of lambda={lams[0] * 1e9:.0f} nm, incidence 0 against the FP64 GPU "
                           f"sum; {dirs.size} seeded directions of incidences 0 and {n_inc - 1} against the "
                           "FP64 oracle on the host",
        "roofline": roof,
        "kernel_ms_per_step": {"leaf": r["ms_leaf_kernel"], "phi passes": r["ms_rows"], "theta passes": r["ms_cols"],
                               "phi by level": r["ms_rows_level"][:FIBER_DEPTH],
                               "theta by level": r["ms_cols_level"][:FIBER_DEPTH]},
        "cpu_baseline": {"value": cpu_value, "unit": "Gpoint-dirs/s", "cores": oracle.num_threads(), "kind": "port",
                         "sample": f"FP64 direct sum (oracle/po_oracle.c) of all {n} points x {cdirs.size} seeded "
                                   f"directions, lambda={lams[0] * 1e9:.0f} nm, incidence 0",
                         "seconds": cpu_s},
        "geometry_build_ms": t_geom * 1e3,
        "gpu_launches": int(args.steps * r["kernel_launches"]),  # launches per solve are fixed
        "clocks": clk,
        "wall_s_timed_region": t_wall,
        "report": r,
    }
    return result


# ---------------------------------------------------- differentiation workload
CYL_R, CYL_L, CYL_N, CYL_DEPTH, CYL_INC, CYL_EXTENT = 10e-6, 20e-6, 1_000_000, 6, 8, 26e-6
CYL_WORKLOAD = ("rough cylinder r=10um L=20um (1.0M points), normal displacement h ~ Gaussian(0.02um, 0.5um), "
                "25 wavelengths x 8 incidences x TM, depth 6, loss ||I(h) - I(h_target)||^2, gradient dL/dh")


def run_cylinder_grad(args, world, rank, local):
    """Forward + adjoint of the loss ||I(h) - I_t||^2 over the displacement
    field h of a rough cylinder, through torch.autograd; the gradient is
    checked against the FP64 reference gradient and central differences."""
    import torch

    from wavefiber3d_gb300 import api, autograd, geometry
    import __graft_entry__
    __graft_entry__.build()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    st = torch.cuda.current_stream()
    hf, h = geometry.cylinder_height_field(CYL_R, CYL_L, CYL_N, seed=1)
    _, h_t = geometry.cylinder_height_field(CYL_R, CYL_L, CYL_N, seed=2)
    numel, numelvert = hf.numel, hf.numelvert
    phi = torch.arange(numel, dtype=torch.float64, device=dev) * (2 * math.pi / numel)
    cs, sn = torch.cos(phi)[:, None], torch.sin(phi)[:, None]

    def xy_of(hh):
        r = CYL_R + hh
        return torch.stack([r * cs, r * sn]).float()

    box = [-1.1 * CYL_R, -1.1 * CYL_R, -0.55 * CYL_L]
    bmax = [-v for v in box]
    # level grids by the reference rule (ratio 1.2) on a 26 um extent: the rule's 20 um (the cylinder
    # length) leaves the level-1 cells of the 22 um box (19 um diagonals) under-resolved (forward
    # rel-L2 7e-4, gradient 5%); 26 um gives 4e-6 and 1e-4 for 1.4x the time
    cfg = api.Config.reference_rule(CYL_DEPTH, N_THETA, N_PHI, box, bmax, CYL_EXTENT, CYL_EXTENT, 1.2,
                                    precision=PRECISIONS[args.precision])
    th = [0.05 * i for i in range(CYL_INC)]  # theta sweep from normal incidence on the axis-normal plane
    ph = [0.0] * CYL_INC
    lams = LAMBDAS[: args.cyl_lambdas]
    illum = api.Illumination(lams, th, ph, api.PO_POL_TM, ETA, 1.0)
    solver = api.Solver(cfg)
    h_dev = torch.from_numpy(h).to(dev)
    with torch.no_grad():
        s_t = api.height_field_points_tensor(xy_of(torch.from_numpy(h_t).to(dev)), hf.period, hf.unitz, 0, numel - 1)
        target = solver.solve(tuple(s_t[k] for k in range(7)), illum)

    def step():
        hh = h_dev.clone().requires_grad_(True)
        samples = autograd.height_field_samples(xy_of(hh), hf.period, hf.unitz)
        inten = autograd.far_field_intensity(solver, illum, samples)
        loss = ((inten - target) ** 2).sum()
        loss.backward()
        return loss, hh.grad

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    evs = []
    clocks = ClockSampler(local)
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        loss, g_h = step()
        e1.record(st)
        evs.append((e0, e1))
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms_step = statistics.mean(a.elapsed_time(b) for a, b in evs)
    # forward alone, for the adjoint/forward ratio
    with torch.no_grad():
        s0 = api.height_field_points_tensor(xy_of(h_dev), hf.period, hf.unitz, 0, numel - 1)
        out = torch.empty(solver.out_shape(illum), dtype=torch.float32, device=dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        solver.solve(tuple(s0[k] for k in range(7)), illum, out=out)
        e1.record(st)
        torch.cuda.synchronize()
        ms_fwd = e0.elapsed_time(e1)
        w_full = 2 * (out - target)
        e0.record(st)
        solver.grad(s0, illum, w_full)
        e1.record(st)
        torch.cuda.synchronize()
        ms_grad = e0.elapsed_time(e1)
    grad_report = dict(solver.last_report)
    solver.close()

    # ---- checks on one pattern (400 nm, first incidence), all points
    import oracle
    il1 = api.Illumination(lams[:1], th[:1], ph[:1], api.PO_POL_TM, ETA, 1.0)
    cfg64 = api.Config(0, [N_THETA], [N_PHI], box, bmax, precision=api.PO_PREC_FP64)
    with api.Solver(cfg) as s_tree, api.Solver(cfg64) as s64, torch.no_grad():
        t1 = s64.solve(tuple(s_t[k] for k in range(7)), il1)
        i64 = s64.solve(tuple(s0[k] for k in range(7)), il1)
        w1 = 2 * (i64 - t1)
        t0 = time.perf_counter()
        g64 = s64.grad(s0, il1, w1).double()
        torch.cuda.synchronize()
        s_fp64 = time.perf_counter() - t0
        g_tree = s_tree.grad(s0, il1, w1).double()
        ref_err = {grp: float((g_tree[r] - g64[r]).norm() / g64[r].norm())
                   for grp, r in (("positions", slice(0, 3)), ("normals", slice(3, 6)), ("areas", slice(6, 7)))}
        gh_tree = api.height_field_adjoint(xy_of(h_dev), hf.period, hf.unitz, 0, numel - 1, g_tree.float())
        gh_64 = api.height_field_adjoint(xy_of(h_dev), hf.period, hf.unitz, 0, numel - 1, g64.float())
        dh_tree = (gh_tree[0].double() * cs + gh_tree[1].double() * sn)
        dh_64 = (gh_64[0].double() * cs + gh_64[1].double() * sn)
        ref_err_h = float((dh_tree - dh_64).norm() / dh_64.norm())
        # central differences of the FP64 oracle (host, sampled directions) under a perturbation of
        # 64 random samples, against the gradients of the same sampled loss
        rng = np.random.default_rng(64)
        dirs = np.sort(rng.choice(N_THETA * N_PHI, args.cyl_fd_dirs, replace=False))
        wv = np.zeros(N_THETA * N_PHI)
        wv[dirs] = rng.standard_normal(dirs.size)
        wt = torch.from_numpy(wv.reshape(1, 1, 1, N_THETA, N_PHI)).float().to(dev)
        gs64 = s64.grad(s0, il1, wt).double().cpu().numpy()
        gst = s_tree.grad(s0, il1, wt).double().cpu().numpy()
        sn0 = s0.double().cpu().numpy()
        pick = rng.choice(sn0.shape[1], 64, replace=False)
        v = np.zeros_like(sn0)
        v[:3, pick] = rng.choice([-1.0, 1.0], (3, 64)) * 1e-10
        v[3:6, pick] = rng.choice([-1.0, 1.0], (3, 64)) * 1e-6
        v[6, pick] = sn0[6, pick] * 1e-6
        il_o = oracle.make_illum(lams[0], th[0], ph[0], "M", ETA, 1.0)
        t0 = time.perf_counter()
        fd = float(wv[dirs] @ (oracle.solve_sampled_f64(sn0 + v, il_o, N_THETA, N_PHI, dirs) -
                               oracle.solve_sampled_f64(sn0 - v, il_o, N_THETA, N_PHI, dirs)))
        s_fd = time.perf_counter() - t0
        ad64 = float((gs64 * 2 * v).sum())
        adtree = float((gst * 2 * v).sum())
    n = numel * numelvert
    pd = float(n) * N_THETA * N_PHI * illum.n_patterns
    return {
        "metric": "gradient evaluations/s of ||I(h) - I_target||^2 w.r.t. the displacement field h (forward + adjoint)",
        "value": 1000.0 / ms_step, "unit": "gradients/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "split bf16 hi+lo products, f32 accumulation (f64 phase arguments); f64 currents Jacobian"
                 if args.precision == "split_bf16" else "f32 (f64 phase arguments); f64 currents Jacobian",
        "data": "synthetic (seeded displacement fields, target from a second seed)",
        "config": {"workload": CYL_WORKLOAD, "points": n, "numel": numel, "numelvert": numelvert,
                   "wavelengths": len(lams), "incidences": CYL_INC, "depth": CYL_DEPTH,
                   "level_grids": [list(cfg.n_theta), list(cfg.n_phi)], "precision": args.precision},
        "ms_forward": ms_fwd, "ms_po_grad": ms_grad, "grad_over_forward": ms_grad / ms_fwd,
        "equivalent_gpoint_dirs_per_s_forward": pd / (ms_fwd * 1e-3) / 1e9,
        "gradient_check": {
            "pattern": f"lambda={lams[0] * 1e9:.0f} nm, incidence 0, all {n} points, loss ||I - I_t||^2",
            "rel_l2_vs_fp64_reference_gradient": ref_err,
            "rel_l2_vs_fp64_reference_gradient_dL_dh": ref_err_h,
            "fd_64_samples": {"loss": f"sum of seeded weights x FP64 oracle intensity on {dirs.size} directions",
                              "steps": "1e-10 m positions, 1e-6 normals, 1e-6 relative areas, random signs",
                              "central_difference": fd, "adjoint_fp64": ad64, "adjoint_tree": adtree,
                              "rel_err_fp64": abs(ad64 - fd) / abs(fd), "rel_err_tree": abs(adtree - fd) / abs(fd),
                              "oracle_s": s_fd},
            "fp64_reference_gradient_s": s_fp64},
        "loss": float(loss.detach()), "grad_h_norm": float(g_h.norm()),
        "gpu_launches": int(grad_report.get("kernel_launches", 0)),
        "clocks": clk,
        "report_grad": grad_report,
    }


# ------------------------------------------------------------ batch workload
BATCH_WORKLOAD = ("256 independent solves: spheres and ellipsoids r = 1-10 um, 5k-500k points (log-uniform), "
                  "random wavelength 400-700 nm and incidence, TM, 180x360, depth / leaf precision / tile by "
                  "the autotuner, one CUDA graph")


def make_batch_items(n_items: int, seed: int = 4):
    from wavefiber3d_gb300 import geometry
    rng = np.random.default_rng(seed)
    items = []
    for i in range(n_items):
        r = float(rng.uniform(1e-6, 10e-6))
        n = int(round(math.exp(rng.uniform(math.log(5e3), math.log(5e5)))))
        if rng.random() < 0.5:
            radii = (r, r, r)
            cloud = geometry.fibonacci_sphere(r, n)
        else:
            radii = (r, r * float(rng.uniform(0.5, 1.0)), r * float(rng.uniform(0.5, 1.0)))
            cloud = geometry.ellipsoid(radii, n)
        lam = float(rng.uniform(400e-9, 700e-9))
        th = float(rng.uniform(-math.pi / 2 + 0.05, math.pi / 2 - 0.05))
        ph = float(rng.uniform(0, 2 * math.pi))
        items.append((cloud, radii, lam, th, ph))
    return items


def run_batch(args, world, rank, local):
    """Config 4: many independent solves in one captured CUDA graph."""
    import torch

    import oracle
    from wavefiber3d_gb300 import api, autotune
    import __graft_entry__
    __graft_entry__.build()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    st = torch.cuda.current_stream()
    items = make_batch_items(args.batch_items)
    tuner = autotune.Autotuner(cache_path=args.tune_cache, reps=2)
    configs, samples, illums, choices = [], [], [], []
    t0 = time.perf_counter()
    for cloud, radii, lam, th, ph in items:
        r = max(radii)
        box = [-1.1 * a for a in radii], [1.1 * a for a in radii]
        g = torch.from_numpy(cloud.soa()).to(dev)
        il = api.Illumination([lam], [th], [ph], api.PO_POL_TM, ETA, 1.0)

        def make(depth, prec, box=box, r=r):
            return api.Config.reference_rule(depth, N_THETA, N_PHI, box[0], box[1], 2 * r, 2 * r, 1.3,
                                             precision=prec)
        ch = tuner.choose(g, il, make, 2 * r)
        configs.append(autotune.apply(make(ch["depth"], ch["precision"]), ch))
        samples.append(g)
        illums.append(il)
        choices.append(ch)
    tune_s = time.perf_counter() - t0
    tuner.save()
    batch = api.Batch(configs, n_streams=args.batch_streams)
    t0 = time.perf_counter()
    batch.prepare(samples, illums)
    torch.cuda.synchronize()
    prepare_s = time.perf_counter() - t0
    for _ in range(args.warmup):
        batch.launch()
    torch.cuda.synchronize()
    evs = []
    clocks = ClockSampler(local)
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        batch.launch()
        e1.record(st)
        evs.append((e0, e1))
    torch.cuda.synchronize()
    clk = clocks.stop()
    batch.check(st)  # raises if an item's kernels gave up a bounded device wait
    ms_graph = statistics.mean(a.elapsed_time(b) for a, b in evs)
    info = batch.info()
    # the same solves one by one (po_solve, no graph)
    solvers = [api.Solver(c) for c in configs]
    outs = [torch.empty(s.out_shape(il), dtype=torch.float32, device=dev) for s, il in zip(solvers, illums)]
    for s, g, il, o in zip(solvers, samples, illums, outs):
        s.solve(tuple(g[k] for k in range(7)), il, out=o)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for s, g, il, o in zip(solvers, samples, illums, outs):
        s.solve(tuple(g[k] for k in range(7)), il, out=o)
    e1.record(st)
    torch.cuda.synchronize()
    ms_serial = e0.elapsed_time(e1)
    same = all(torch.equal(a, b) for a, b in zip(outs, batch.outputs))
    for s in solvers:
        s.close()
    # per-solve error against the FP64 oracle on sampled directions
    rng = np.random.default_rng(7)
    errs = []
    t0 = time.perf_counter()
    for (cloud, radii, lam, th, ph), o in zip(items, batch.outputs):
        dirs = np.sort(rng.choice(N_THETA * N_PHI, args.batch_dirs, replace=False))
        il_o = oracle.make_illum(lam, th, ph, "M", ETA, 1.0)
        ref = oracle.solve_sampled_f64(cloud.soa().astype(np.float64), il_o, N_THETA, N_PHI, dirs)
        got = o.reshape(-1).cpu().numpy()[dirs].astype(np.float64)
        errs.append(float(np.linalg.norm(got - ref) / np.linalg.norm(ref)))
    oracle_s = time.perf_counter() - t0
    batch.close()
    npts = sum(int(g.shape[1]) for g in samples)
    pd = float(npts) * N_THETA * N_PHI
    # baselines on the first solves of the batch, scaled to the whole batch by
    # point-direction terms: the plain FP64 direct sum on this GPU (B1, full
    # grid) and the FP64 oracle on the host cores (B0, seeded directions)
    k = min(args.batch_baseline_items, len(items))
    b1_ms, b1_pd, b0_s, b0_pd = 0.0, 0.0, 0.0, 0.0
    dirs = sample_directions(args.cpu_dirs)
    for (cloud, radii, lam, th, ph), g in zip(items[:k], samples[:k]):
        il = api.Illumination([lam], [th], [ph], api.PO_POL_TM, ETA, 1.0)
        cfg = api.Config(0, [N_THETA], [N_PHI], [-1.1 * a for a in radii], [1.1 * a for a in radii],
                         precision=api.PO_PREC_FP64)
        with api.Solver(cfg) as s64:
            out = torch.empty(s64.out_shape(il), dtype=torch.float32, device=dev)
            s64.solve(tuple(g[q] for q in range(7)), il, out=out)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            s64.solve(tuple(g[q] for q in range(7)), il, out=out, report=False)
            e1.record(st)
            torch.cuda.synchronize()
        b1_ms += e0.elapsed_time(e1)
        b1_pd += float(g.shape[1]) * N_THETA * N_PHI
        il_o = oracle.make_illum(lam, th, ph, "M", ETA, 1.0)
        t0 = time.perf_counter()
        oracle.solve_sampled_f64(cloud.soa().astype(np.float64), il_o, N_THETA, N_PHI, dirs)
        b0_s += time.perf_counter() - t0
        b0_pd += float(g.shape[1]) * dirs.size
    b1_rate, b0_rate = b1_pd / (b1_ms * 1e-3) / 1e9, b0_pd / b0_s / 1e9
    depth_hist = {d: sum(1 for c in choices if c["depth"] == d) for d in range(7)}
    return {
        "metric": "Gpoint-dirs/s (equivalent depth-0 terms) of a batch of independent solves in one CUDA graph",
        "value": pd / (ms_graph * 1e-3) / 1e9, "unit": "Gpoint-dirs/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_graph, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 / split bf16 per solve (autotuned), f64 phase arguments",
        "data": "synthetic (seeded spheres and ellipsoids)",
        "config": {"workload": BATCH_WORKLOAD, "solves": len(items), "points_total": npts,
                   "streams": args.batch_streams, "depths": depth_hist,
                   "split_bf16_solves": sum(1 for c in choices if c["precision"] == api.PO_PREC_SPLIT_BF16),
                   "tiles": {t: sum(1 for c in choices if c["tile"] == t) for t in (0, 8, 16)},
                   "leaf_kernels": {k: sum(1 for c in choices if c.get("leaf_kernel", 0) == v)
                                    for k, v in (("auto", 0), ("warp", 1), ("tcgen05", 2))}},
        "solves_per_s": len(items) / (ms_graph * 1e-3),
        "ms_same_solves_one_by_one": ms_serial, "graph_speedup": ms_serial / ms_graph,
        "graph_equals_one_by_one": same,
        "graph_nodes": info["graph_nodes"], "workspace_bytes": info["workspace_bytes"],
        "prepare_s": prepare_s, "tuning_s": tune_s, "tuning_trials": tuner.trials, "tuned_classes": len(tuner.cache),
        "per_solve_rel_l2_vs_fp64": {"max": max(errs), "median": float(np.median(errs)),
                                     "sample": f"{args.batch_dirs} seeded directions per solve, FP64 oracle"},
        "oracle_s": oracle_s,
        "plain_fp64_gpu": {"value": b1_rate, "unit": "Gpoint-dirs/s", "ms_per_step_scaled": pd / b1_rate / 1e6,
                           "sample": f"FP64 depth-0 sum (k_direct_f64) of the first {k} solves on the full grid, "
                                     "scaled by point-direction terms"},
        "speedup_vs_plain_fp64_gpu": (pd / b1_rate / 1e6) / ms_graph,
        "cpu_baseline": {"value": b0_rate, "unit": "Gpoint-dirs/s", "cores": oracle.num_threads(), "kind": "port",
                         "ms_per_step_scaled": pd / b0_rate / 1e6,
                         "sample": f"FP64 oracle direct sum of the first {k} solves on {dirs.size} seeded directions"},
        "clocks": clk,
    }


def run_reference_cuda(args, world, rank, local):
    """The reference's own CUDA path timed on this GPU (baseline B2): the
    unmodified util/*.h driven in the order of compareMie/sphere.cu:212-936 by
    oracle/ref_harness.cu, on the plain-method sphere (config 1, in full) and
    on one (wavelength, incidence) pair of the ellipsoid (config 2: the leaf
    loop on a subset of its directions and each level on a subset of its
    children, extrapolated linearly by the counts, which the reference's
    per-direction and per-child launches make exact up to launch jitter).
    The fiber (config 3) is not run: its depth-7 CDP octree issues 299,593
    device launches (util/tree.h:710-712) against the pending-launch limit of
    32,768 that the reference sets."""
    if rank != 0:
        return None
    import torch

    from wavefiber3d_gb300 import api, geometry
    import __graft_entry__
    __graft_entry__.build()
    harness = ROOT / "oracle" / "_ref" / "ref_harness"
    if not harness.exists():
        return {"impl": "reference-cuda", "unavailable": "oracle/_ref/ref_harness not built (no staged headers)"}
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    tmp = Path(tempfile.mkdtemp(prefix="refcuda_"))

    def run(cloud, box, depth, nth, nph, lam, th, ph, eta, sigma, caps):
        gpath, opath = tmp / "geom.bin", tmp / "out.bin"
        cloud.soa().astype(np.float32).tofile(gpath)
        cmd = [str(harness), "time", str(gpath), str(cloud.n), *[repr(float(v)) for v in box], str(depth)]
        for a, b in zip(nth, nph):
            cmd += [str(a), str(b)]
        cmd += [repr(lam), repr(th), repr(ph), "M", repr(eta.real), repr(eta.imag), repr(sigma), str(opath),
                *[str(c) for c in caps]]
        t0 = time.perf_counter()
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=1200)
        wall = time.perf_counter() - t0
        if r.returncode != 0:
            raise RuntimeError(f"ref_harness failed ({r.returncode}): {r.stderr[-2000:]}")
        line = [x for x in r.stdout.splitlines() if x.startswith("{")][-1]
        t = json.loads(line)
        leaf = t["leaf_ms"] * t["leaf_dirs"] / max(1, t["leaf_dirs_done"])
        levels = sum(v["ms"] * v["children"] / max(1, v["children_done"]) for v in t["levels"] if v["children_done"])
        total = t["tree_ms"] + t["setup_ms"] + leaf + levels + t["intensity_ms"]
        out = np.fromfile(opath, dtype=np.float32) if opath.exists() else None
        return t, total, wall, out

    # ---- config 1: 20,000-point sphere, depth 0, 180 x 360, one pattern, complete
    sph = geometry.fibonacci_sphere(2e-6, 20000)
    box1 = [-2.2e-6] * 3 + [2.2e-6] * 3
    t1, ms1, wall1, out1 = run(sph, box1, 0, [N_THETA], [N_PHI], 500e-9, math.pi / 2, math.pi, 1.55 + 0j, 1e-2,
                               (0, 0, 0))
    cfg1 = api.Config(0, [N_THETA], [N_PHI], box1[:3], box1[3:], precision=api.PO_PREC_FP32)
    il1 = api.Illumination([500e-9], [math.pi / 2], [math.pi], api.PO_POL_TM, 1.55 + 0j, 1e-2)
    with api.Solver(cfg1) as s:
        eng1 = s.solve(sph, il1).reshape(-1).astype(np.float64)
    agree1 = float(np.linalg.norm(out1 - eng1) / np.linalg.norm(eng1))

    # the engine (B1 FP64, B3 FP32) and the host FP64 oracle (B0) on the same configs
    st = torch.cuda.current_stream()
    g1 = torch.from_numpy(sph.soa()).to(dev)

    def engine_ms(cfg, g, il, reps=5):
        with api.Solver(cfg) as s:
            out = torch.empty(s.out_shape(il), dtype=torch.float32, device=dev)
            geom = tuple(g[k] for k in range(7))
            for _ in range(2):
                s.solve(geom, il, out=out, report=False)
            ts = []
            for _ in range(reps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(st)
                s.solve(geom, il, out=out, report=False)
                e1.record(st)
                torch.cuda.synchronize()
                ts.append(e0.elapsed_time(e1))
            return statistics.median(ts)
    import oracle
    eng = {"sphere_20k_depth0": {
        "b1_fp64_gpu_ms": engine_ms(api.Config(0, [N_THETA], [N_PHI], box1[:3], box1[3:], precision=api.PO_PREC_FP64),
                                    g1, il1),
        "b3_fp32_gpu_ms": engine_ms(cfg1, g1, il1)}}
    t0 = time.perf_counter()
    oracle.solve_direct(sph, oracle.make_illum(500e-9, math.pi / 2, math.pi, "M", 1.55, 1e-2), N_THETA, N_PHI)
    eng["sphere_20k_depth0"]["b0_fp64_host_ms"] = (time.perf_counter() - t0) * 1e3
    # plain vs tensor-core at depth 0: the split-BF16 tcgen05 direct sum (one leaf of all points), for the
    # config's one pattern and per pattern at 64 incidences (where one phase tile serves 64 slots)
    cfg1t = api.Config(0, [N_THETA], [N_PHI], box1[:3], box1[3:], precision=api.PO_PREC_SPLIT_BF16)
    e1 = eng["sphere_20k_depth0"]
    e1["b3_tensor_core_gpu_ms"] = engine_ms(cfg1t, g1, il1)
    with api.Solver(cfg1t) as s, api.Solver(api.Config(0, [N_THETA], [N_PHI], box1[:3], box1[3:],
                                                      precision=api.PO_PREC_FP64)) as s64:
        ot = s.solve(sph, il1).reshape(-1).astype(np.float64)
        o64 = s64.solve(sph, il1).reshape(-1).astype(np.float64)
    e1["tensor_core_rel_l2_vs_fp64"] = float(np.linalg.norm(ot - o64) / np.linalg.norm(o64))
    th64, ph64 = fiber_incidences(64)
    il64 = api.Illumination([500e-9], th64, ph64, api.PO_POL_TM, 1.55 + 0j, 1e-2)
    e1["per_pattern_ms_at_64_incidences"] = {"fp32": engine_ms(cfg1, g1, il64, reps=3) / 64,
                                             "tensor_core": engine_ms(cfg1t, g1, il64, reps=3) / 64}
    eng["sphere_20k_depth0"]["b0_cores"] = oracle.num_threads()

    # ---- config 2: 400k-point ellipsoid, depth 5, one (wavelength, incidence) pair, capped loops
    ell = geometry.ellipsoid(RADII, N_POINTS)
    box2 = [-1.1 * r for r in RADII] + [1.1 * r for r in RADII]
    cfg2 = api.Config.reference_rule(DEPTH, N_THETA, N_PHI, box2[:3], box2[3:], 16e-6, 16e-6, 1.3)
    caps2 = (args.ref_leaf_dirs, args.ref_children, 1)
    t2, ms2, wall2, _ = run(ell, box2, DEPTH, cfg2.n_theta, cfg2.n_phi, LAMBDAS[0], 0.0, 0.0, ETA, SIGMA, caps2)
    g2 = torch.from_numpy(ell.soa()).to(dev)
    il2 = api.Illumination(LAMBDAS[:1], [0.0], [0.0], api.PO_POL_TM, ETA, SIGMA)
    eng["ellipsoid_400k_depth5"] = {
        "b1_fp64_gpu_ms_per_pattern": engine_ms(
            api.Config(0, [N_THETA], [N_PHI], box2[:3], box2[3:], precision=api.PO_PREC_FP64), g2, il2, reps=2)}
    return {
        "impl": "reference-cuda",
        "metric": "ms per pattern of the reference's own CUDA build (baseline B2)",
        "unit": "ms", "higher_is_better": False, "n_gpus": 1,
        "data": "synthetic (seeded sphere and ellipsoid)",
        "plain_sphere_20k_depth0": {
            "ms_per_pattern": ms1, "wall_s": wall1, "phases": t1,
            "gpoint_dirs_per_s": sph.n * N_THETA * N_PHI / (ms1 * 1e-3) / 1e9,
            "rel_l2_vs_engine_fp32": agree1,
            "note": "complete run: CDP octree of depth 0, 64,800 x (transform + thrust::reduce + fill), intensity"},
        "ellipsoid_400k_depth5": {
            "ms_per_pattern_extrapolated": ms2, "ms_per_step_extrapolated": ms2 * len(LAMBDAS),
            "wall_s": wall2, "phases": t2,
            "gpoint_dirs_per_s": N_POINTS * N_THETA * N_PHI / (ms2 * 1e-3) / 1e9,
            "note": f"lambda={LAMBDAS[0] * 1e9:.0f} nm, incidence +x: leaf loop timed on {t2['leaf_dirs_done']} of "
                    f"{t2['leaf_dirs']} directions, levels 4..1 on up to {args.ref_children} children each, "
                    "extrapolated by the counts; the root level (197 -> 180 theta samples, a downsampling the "
                    "reference's interpolation cannot do) and the intensity are left out, so this is a lower "
                    f"bound; the step figure scales by the {len(LAMBDAS)} wavelengths"},
        "engine_and_host_same_configs": eng,
        "fiber_3p4m_depth7": {"unavailable": "the reference's depth-7 CDP octree issues 299,593 device-side "
                                             "launches (util/tree.h:710-712) against its pending-launch limit of "
                                             "32,768; not run on this pool"},
    }


def run_reference(args, world, rank):
    """CPU implementation of the path on all host cores: the reference ships
    CUDA only, so this is the FP64 direct-sum restatement of its algorithm
    (oracle/), on a bounded direction sample of the workload's geometry."""
    if rank != 0:
        return None
    import oracle
    from wavefiber3d_gb300 import geometry
    if args.workload == "ellipsoid":
        cloud = geometry.ellipsoid(RADII, N_POINTS)
        wl, lam_list, incs, sigma, ctr = WORKLOAD, LAMBDAS, [(0.0, 0.0)], SIGMA, [0.0, 0.0, 0.0]
        data = "synthetic (seeded ellipsoid, analytic normals)"
    else:
        hf = geometry.fiber_height_field(FIBER_RADII, FIBER_LENGTH, seed=FIBER_SEED)
        soa, bad = oracle.height_field(hf)  # util/geometry.h:76-179 on the host (bit-exact with the GPU sampler)
        assert not bad
        cloud = geometry.PointCloud.from_soa(soa)
        th, ph = fiber_incidences()
        wl, lam_list, incs, sigma = FIBER_WORKLOAD, LAMBDAS, list(zip(th, ph)), FIBER_SIGMA
        ctr = [0.5 * (a + b) for a, b in zip(np.float32(FIBER_BOX_MIN), np.float32(FIBER_BOX_MAX))]
        data = "synthetic (seeded fiber height field, sampled on the host)"
    dirs = sample_directions(args.ref_dirs)

    def one(i, d):
        lam = lam_list[i % len(lam_list)]
        t, p = incs[(i // len(lam_list)) % len(incs)]
        il = oracle.make_illum(lam, t, p, "M", ETA, sigma)
        t0 = time.perf_counter()
        cur = oracle.currents(cloud, il)
        f = oracle.far_field_sampled(cloud, cur, 2 * math.pi / lam, ctr, N_THETA, N_PHI, d)
        oracle.intensity_sampled(f, N_THETA, N_PHI, d)
        return time.perf_counter() - t0

    for _ in range(max(0, min(args.warmup, 1))):
        one(0, dirs[:64])
    secs = [one(i, dirs) for i in range(args.steps)]
    per = sum(secs) / len(secs)
    value = cloud.n * dirs.size / per / 1e9
    return {
        "impl": "reference",
        "metric": "Gpoint-dirs/s (equivalent depth-0 point x direction terms) at rel-L2<=1e-3 vs FP64 direct sum",
        "value": value, "unit": "Gpoint-dirs/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": per * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": data,
        "config": {"workload": wl, "points": cloud.n, "directions": N_THETA * N_PHI,
                   "step": f"bounded sample: {dirs.size} directions x 1 (wavelength, incidence) per step, cycling "
                           "through the workload's wavelengths and incidences"},
        "cpu_baseline": {"value": value, "unit": "Gpoint-dirs/s", "cores": oracle.num_threads(), "kind": "port",
                         "sample": f"FP64 direct sum (oracle/po_oracle.c), {cloud.n} points x {dirs.size} "
                                   "directions per step; the reference ships no CPU path and its CUDA build "
                                   "needs a GPU"},
        "e2e": {"value": value, "unit": "Gpoint-dirs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["engine", "reference"], default="engine")
    ap.add_argument("--cpu-dirs", type=int, default=1024, help="directions of the FP64 CPU baseline sample")
    ap.add_argument("--precision", choices=sorted(PRECISIONS), default=None,
                    help="leaf precision (default: split_bf16 for the ellipsoid and the fiber -- the faster one at "
                         "the same accuracy on GB300 -- and fp32 for the cylinder gradient)")
    ap.add_argument("--interp", choices=sorted(INTERP), default="tensor")
    ap.add_argument("--interp-tile", type=int, choices=[0, 8, 16], default=0,
                    help="complex columns per CTA of the tensor-core theta pass (0: automatic)")
    ap.add_argument("--theta-mode", choices=sorted(THETA_MODES), default="double_cover",
                    help="ellipsoid workload: the engine's double-cover theta sampling, or the reference's "
                         "pi-periodic theta interpolation (its drop-in mode)")
    ap.add_argument("--lambdas", type=int, default=25,
                    help="wavelengths of the ellipsoid workload (25 = the workload; fewer for profiling runs)")
    ap.add_argument("--incidences", type=int, default=1,
                    help="incidences of the ellipsoid workload (1 = the workload; more for profiling runs)")
    ap.add_argument("--fiber-incidences", type=int, default=64,
                    help="incidences per fiber step (64 = the workload; fewer for profiling runs)")
    ap.add_argument("--workload", choices=["fiber", "ellipsoid", "cylinder-grad", "batch", "reference-cuda"],
                    default="fiber",
                    help="fiber: the headline, the 3.4M-point fiber segment, 25 wavelengths x 64 incidences, depth 7 "
                         "(split precision vs plain FP64 on the same GPU); ellipsoid: 400k points, 25 wavelengths, "
                         "depth 5; cylinder-grad: the gradient workload; batch: 256 independent solves; "
                         "reference-cuda: the reference's own CUDA build on configs 1 and 2 (baseline B2)")
    ap.add_argument("--ref-leaf-dirs", type=int, default=24, help="reference-cuda: leaf directions timed")
    ap.add_argument("--ref-children", type=int, default=48, help="reference-cuda: children timed per level")
    ap.add_argument("--fiber-lambdas", type=int, default=25, help="wavelengths per fiber step (25 = the workload)")
    ap.add_argument("--workspace-gb", type=float, default=0.0,
                    help="fiber: the solver's workspace cap in GB, which sets how many patterns go through the tree "
                         "at once (0: the library default, half the device)")
    ap.add_argument("--e2e-steps", type=int, default=2, help="steps of the end-to-end (host buffers) timing")
    ap.add_argument("--ref-dirs", type=int, default=256, help="directions per step of the --impl reference arm")
    ap.add_argument("--fiber-dirs", type=int, default=512, help="directions of the fiber accuracy sample")
    ap.add_argument("--cyl-lambdas", type=int, default=25, help="wavelengths of the cylinder gradient step")
    ap.add_argument("--cyl-fd-dirs", type=int, default=256, help="directions of the cylinder FD check")
    ap.add_argument("--batch-items", type=int, default=256, help="independent solves of the batch workload")
    ap.add_argument("--batch-streams", type=int, default=16, help="concurrent graph branches of the batch")
    ap.add_argument("--batch-dirs", type=int, default=64, help="FP64 check directions per batch solve")
    ap.add_argument("--batch-baseline-items", type=int, default=4,
                    help="solves of the batch timed for its FP64 GPU and host baselines")
    ap.add_argument("--tune-cache", default=None, help="JSON file of the autotuner's choices (read and written)")
    args = ap.parse_args()
    if args.precision is None:
        args.precision = "fp32" if args.workload == "cylinder-grad" else "split_bf16"
    if args.warmup < 3 and args.impl == "engine":
        args.warmup = 3
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        res = run_reference(args, world, rank)
    elif args.workload == "fiber":
        res = run_fiber(args, world, rank, local)
    elif args.workload == "cylinder-grad":
        res = run_cylinder_grad(args, world, rank, local) if rank == 0 else None
    elif args.workload == "batch":
        res = run_batch(args, world, rank, local) if rank == 0 else None
    elif args.workload == "reference-cuda":
        res = run_reference_cuda(args, world, rank, local)
    else:
        res = run_engine(args, world, rank, local)
    if rank == 0 and res is not None:
        print(json.dumps(res), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
