"""Autotuner of the per-solve schedule.

For a geometry class (point count and electrical size, bucketed on a log2
scale) it times the candidate schedules on the GPU and keeps the fastest:

* octree depth: the heuristic depth (about 48 points per leaf) and its two
  neighbours, 0..6;
* leaf contraction: FP32 CUDA cores or split hi+lo BF16 tensor cores
  (depth >= 1);
* theta-pass tile: 8 or 16 complex columns per CTA (after the two choices
  above).

Every candidate computes the same double-cover patterns (their accuracy
differences are far below the 1e-3 bar; `tests/test_gpu_batch.py` checks
every item of a batch built from the chosen schedules against the FP64
oracle), so the choice is by time alone.  Results are cached per class, in memory and optionally in a JSON
file, so a batch of many solves tunes each class once.
"""
from __future__ import annotations

import json
import math
from pathlib import Path

import numpy as np

from . import api

MAX_DEPTH = 6


def heuristic_depth(n_points: int) -> int:
    return int(min(MAX_DEPTH, max(0, round(math.log(max(n_points, 1) / 48.0, 8)))))


def class_key(n_points: int, size_m: float, wavelength_m: float) -> str:
    return f"n{round(math.log2(max(n_points, 1)))}_s{round(math.log2(max(size_m / wavelength_m, 1e-3)))}"


class Autotuner:
    def __init__(self, cache_path=None, reps: int = 2):
        self.cache_path = Path(cache_path) if cache_path else None
        self.reps = reps
        self.cache: dict = {}
        self.trials = 0
        if self.cache_path and self.cache_path.exists():
            self.cache = json.loads(self.cache_path.read_text())

    def save(self):
        if self.cache_path:
            self.cache_path.write_text(json.dumps(self.cache, indent=1, sort_keys=True))

    def _time(self, cfg, samples, illum) -> float:
        import torch
        geo = tuple(samples[k] for k in range(7))
        with api.Solver(cfg) as s:
            out = torch.empty(s.out_shape(illum), dtype=torch.float32, device="cuda")
            s.solve(geo, illum, out=out)
            ts = []
            for _ in range(self.reps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                s.solve(geo, illum, out=out)
                e1.record()
                torch.cuda.synchronize()
                ts.append(e0.elapsed_time(e1))
        self.trials += 1 + self.reps
        return float(np.median(ts))

    def choose(self, samples, illum, make_config, size_m: float) -> dict:
        """samples: (7, n) CUDA tensor; make_config(depth, precision, tile) -> api.Config.
        Returns {"depth", "precision", "tile", "ms"} for this geometry's class."""
        n = int(samples.shape[1])
        key = class_key(n, size_m, min(illum.wavelengths_m))
        if key in self.cache:
            return self.cache[key]
        d0 = heuristic_depth(n)
        best = None
        for depth in sorted({max(0, d0 - 1), d0, min(MAX_DEPTH, d0 + 1)}):
            precs = [api.PO_PREC_FP32] + ([api.PO_PREC_SPLIT_BF16] if depth >= 1 else [])
            for prec in precs:
                ms = self._time(make_config(depth, prec, 0), samples, illum)
                if best is None or ms < best["ms"]:
                    best = {"depth": depth, "precision": prec, "tile": 0, "ms": ms}
        if best["depth"] >= 1:
            for tile in (8, 16):
                ms = self._time(make_config(best["depth"], best["precision"], tile), samples, illum)
                if ms < best["ms"]:
                    best = dict(best, tile=tile, ms=ms)
        self.cache[key] = best
        return best
