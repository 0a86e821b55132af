"""Autotuner of the per-solve schedule.

For a geometry class (point count, electrical size and patterns per
wavelength, bucketed on a log2 scale) it times candidate schedules and keeps
the fastest, one knob after the other:

1. octree depth and leaf arithmetic: the heuristic depth (about 48 points
   per leaf) and its two neighbours, 0..6, each with FP32 CUDA-core leaf
   sums and (depth >= 1) split hi+lo BF16 tensor-core leaf sums;
2. leaf-batch schedule, for a split-BF16 tree winner: the warp-level
   mma.sync leaf kernel (4 patterns per CTA) or the tcgen05 leaf kernel with
   16, 32 or 64 patterns of a wavelength per pass (each pass regenerates the
   phase operands of every leaf; fewer patterns per pass need less operand
   scratch);
3. theta-pass tile of the warp-level tensor-core kernel: 8 or 16 complex
   columns per CTA (tree winners).

Every candidate computes the same double-cover patterns; their accuracy
differences are far below the 1e-3 bar, so the choice is by time alone
(`tests/test_gpu_configs.py::test_batch_items_vs_fp64_oracle` checks solves
under every kernel choice against the FP64 oracle, and
`tests/test_gpu_batch.py::test_autotuned_batch_vs_fp64_oracle` the tuner's own
choices).  Results are cached per class, in memory and optionally in a JSON
file, so a batch of many solves tunes each class once.

The timer is a parameter: the default times `api.Solver.solve` with CUDA
events on the current stream; tests pass a model of the timings instead.
"""
from __future__ import annotations

import dataclasses
import json
import math
from pathlib import Path
from typing import Callable, Optional

import numpy as np

from . import api

MAX_DEPTH = 6
LEAF_SLOTS = (16, 32, 64)


def heuristic_depth(n_points: int) -> int:
    return int(min(MAX_DEPTH, max(0, round(math.log(max(n_points, 1) / 48.0, 8)))))


def class_key(n_points: int, size_m: float, wavelength_m: float, patterns_per_lambda: int = 1) -> str:
    return (f"n{round(math.log2(max(n_points, 1)))}_s{round(math.log2(max(size_m / wavelength_m, 1e-3)))}"
            f"_g{round(math.log2(max(patterns_per_lambda, 1)))}")


def patterns_per_lambda(illum: api.Illumination) -> int:
    return illum.n_patterns // max(len(illum.wavelengths_m), 1)


def leaf_schedules(g: int) -> list:
    """(leaf_kernel, leaf_slots) candidates for g patterns per wavelength: the
    warp-level kernel, and the tcgen05 kernel with every pass size below g
    plus the one pass that holds all g (rounded up to 8, at most 64)."""
    whole = min(64, 8 * ((g + 7) // 8))
    slots = sorted({s for s in LEAF_SLOTS if s < whole} | {whole})
    return [(api.PO_LEAF_WARP, 0)] + [(api.PO_LEAF_TCGEN05, s) for s in slots]


def apply(cfg: api.Config, choice: dict) -> api.Config:
    """The config of `choice` (depth and precision already in cfg)."""
    return dataclasses.replace(cfg, interp_tile=choice.get("tile", 0),
                               leaf_kernel=choice.get("leaf_kernel", api.PO_LEAF_AUTO),
                               leaf_slots=choice.get("leaf_slots", 0))


def time_solve(cfg: api.Config, samples, illum: api.Illumination, reps: int = 2) -> float:
    """Median device time (ms) of `reps` solves after one untimed solve."""
    import torch
    geo = tuple(samples[k] for k in range(7))
    st = torch.cuda.current_stream()
    with api.Solver(cfg) as s:
        out = torch.empty(s.out_shape(illum), dtype=torch.float32, device=samples.device)
        s.solve(geo, illum, out=out)
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            s.solve(geo, illum, out=out)
            e1.record(st)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
    return float(np.median(ts))


class Autotuner:
    def __init__(self, cache_path=None, reps: int = 2,
                 timer: Optional[Callable[[api.Config, object, api.Illumination], float]] = None):
        self.cache_path = Path(cache_path) if cache_path else None
        self.reps = reps
        self.timer = timer or (lambda cfg, samples, illum: time_solve(cfg, samples, illum, self.reps))
        self.cache: dict = {}
        self.trials = 0
        if self.cache_path and self.cache_path.exists():
            self.cache = json.loads(self.cache_path.read_text())

    def save(self):
        if self.cache_path:
            self.cache_path.write_text(json.dumps(self.cache, indent=1, sort_keys=True))

    def _time(self, cfg, samples, illum) -> float:
        self.trials += 1
        return float(self.timer(cfg, samples, illum))

    def choose(self, samples, illum, make_config, size_m: float) -> dict:
        """samples: (7, n) tensor; make_config(depth, precision) -> api.Config.
        Returns {"depth", "precision", "tile", "leaf_kernel", "leaf_slots", "ms"}
        for this geometry's class; `apply(make_config(depth, precision), choice)`
        is the chosen config."""
        n = int(samples.shape[1])
        g = patterns_per_lambda(illum)
        key = class_key(n, size_m, min(illum.wavelengths_m), g)
        if key in self.cache:
            return self.cache[key]
        d0 = heuristic_depth(n)
        best = None
        for depth in sorted({max(0, d0 - 1), d0, min(MAX_DEPTH, d0 + 1)}):
            for prec in [api.PO_PREC_FP32] + ([api.PO_PREC_SPLIT_BF16] if depth >= 1 else []):
                ms = self._time(make_config(depth, prec), samples, illum)
                if best is None or ms < best["ms"]:
                    best = {"depth": depth, "precision": prec, "tile": 0, "leaf_kernel": api.PO_LEAF_AUTO,
                            "leaf_slots": 0, "ms": ms}
        base = make_config(best["depth"], best["precision"])
        if best["depth"] >= 1 and best["precision"] == api.PO_PREC_SPLIT_BF16:
            for kern, slots in leaf_schedules(g):
                cand = dict(best, leaf_kernel=kern, leaf_slots=slots)
                ms = self._time(apply(base, cand), samples, illum)
                if ms < best["ms"]:
                    best = dict(cand, ms=ms)
        if best["depth"] >= 1:
            for tile in (8, 16):
                cand = dict(best, tile=tile)
                ms = self._time(apply(base, cand), samples, illum)
                if ms < best["ms"]:
                    best = dict(cand, ms=ms)
        self.cache[key] = best
        return best
