"""Angular grids of the hierarchical PO solve.

* Direction grid (compareMie/sphere.cu:370-384): theta is the elevation
  theta_j = -pi/2 + 1e-10 + j*pi/n_theta, phi_k = 2*pi*k/n_phi, and
  s = (cos th cos ph, cos th sin ph, sin th), stored row-major [theta][phi].
* Per-level sample counts (compareMie/sphere.cu:345-352, fibersim/treePO.cu:353-359):
  n(i) = ceil(k_min d_i + beta (k_min d_i)^(1/3)), d_i = 0.5^i * extent * ratio,
  k_min = 2 pi / 0.4 um, beta = 6; level 0 is the output grid.
"""
from __future__ import annotations

import math

import numpy as np

THETA_OFFSET = 1e-10


def directions(n_theta: int, n_phi: int) -> np.ndarray:
    """(n_theta*n_phi, 3) float64 unit vectors in [theta][phi] order."""
    th = -math.pi / 2 + THETA_OFFSET + math.pi / n_theta * np.arange(n_theta)
    ph = 2 * math.pi / n_phi * np.arange(n_phi)
    ct, st = np.cos(th)[:, None], np.sin(th)[:, None]
    s = np.empty((n_theta, n_phi, 3))
    s[..., 0] = ct * np.cos(ph)[None, :]
    s[..., 1] = ct * np.sin(ph)[None, :]
    s[..., 2] = st
    return s.reshape(-1, 3)


def reference_level_count(extent: float, ratio: float, level: int, beta: float = 6.0,
                          lambda_min: float = 0.4e-6) -> int:
    """Sample count of one angular axis at tree level `level` >= 1.  The size
    d is formed in float32 as the reference does (sphere.cu:346)."""
    d = float(np.float32(0.5 ** level * float(np.float32(np.float32(extent) * np.float32(ratio)))))
    kd = 2 * math.pi / lambda_min * d
    return int(math.ceil(kd + beta * kd ** (1.0 / 3.0)))


def level_grids(n_theta_out: int, n_phi_out: int, depth: int, theta_extent: float,
                phi_extent: float, ratio: float, beta: float = 6.0, lambda_min: float = 0.4e-6):
    """Lists (n_theta[l], n_phi[l]) for l = 0..depth; level 0 = output grid."""
    nth = [int(n_theta_out)]
    nph = [int(n_phi_out)]
    for i in range(1, depth + 1):
        nth.append(reference_level_count(theta_extent, ratio, i, beta, lambda_min))
        nph.append(reference_level_count(phi_extent, ratio, i, beta, lambda_min))
    return nth, nph


def smooth_at_least(n: int, primes=(2, 3, 5, 7)) -> int:
    """Smallest integer >= n whose prime factors are all in `primes`."""
    m = max(int(n), 1)
    while True:
        k = m
        for p in primes:
            while k % p == 0:
                k //= p
        if k == 1:
            return m
        m += 1
