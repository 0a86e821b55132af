"""Replica sharding of independent PO work units over processes / GPUs.

The PO path has no exchange step: every (wavelength, incidence,
polarisation) pattern is independent (the reference shards the same way by
command-line ranges, compareMie/sphere.cu:23-24, fibersim/treePO.cu:27-30).
Multi-GPU runs are therefore replicas: each rank solves its own slice of the
wavelength list and the patterns are gathered on the host.  No collective
touches the data path except the final host gather.
"""
from __future__ import annotations

import dataclasses

import numpy as np


def shard_range(n: int, rank: int, world: int) -> range:
    """Contiguous block of [0, n) owned by `rank` (sizes differ by at most one)."""
    if world <= 0 or not (0 <= rank < world):
        raise ValueError("rank must be in [0, world)")
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def shard_illumination(illum, rank: int, world: int):
    """The Illumination restricted to this rank's wavelengths."""
    idx = shard_range(len(illum.wavelengths_m), rank, world)
    return dataclasses.replace(illum, wavelengths_m=[illum.wavelengths_m[i] for i in idx]), idx


def gather_patterns(local: np.ndarray, n_lambda: int, rank: int, world: int, group=None):
    """Gathers per-rank [L_r][...] pattern blocks into [n_lambda][...] on every
    rank (host memory, torch.distributed all_gather_object; works on gloo)."""
    if world == 1:
        return local
    import torch.distributed as dist
    parts = [None] * world
    dist.all_gather_object(parts, (rank, np.asarray(local)), group=group)
    out = None
    for r, arr in sorted(parts, key=lambda t: t[0]):
        idx = shard_range(n_lambda, r, world)
        if out is None:
            out = np.zeros((n_lambda,) + arr.shape[1:], dtype=arr.dtype)
        if len(idx):
            out[idx.start:idx.stop] = arr
    return out
