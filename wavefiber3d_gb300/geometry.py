"""Surface point clouds for the PO far-field engine.

The reference consumes a point cloud with one normal and one area per point
(README.md:96-98), either read from SoA float32 ``.binary`` files
(compareMie/sphere.cu:94-125) or built from a fiber height field
(util/geometry.h:3-72).  This module produces the same arrays:

* ``PointCloud`` -- float32 x, y, z, nx, ny, nz, area (metres, unit normals, m^2);
* readers/writers for the reference's SoA ``*_float.binary`` mesh files;
* seeded synthetic generators used by the tests and the benchmark
  (Fibonacci-lattice sphere, analytic ellipsoid).

Everything here runs on the host and only prepares inputs.
"""
from __future__ import annotations

import dataclasses
import math
from pathlib import Path

import numpy as np

_FIELDS = ("x", "y", "z", "nx", "ny", "nz", "area")


@dataclasses.dataclass
class PointCloud:
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    nx: np.ndarray
    ny: np.ndarray
    nz: np.ndarray
    area: np.ndarray

    def __post_init__(self):
        for f in _FIELDS:
            setattr(self, f, np.ascontiguousarray(getattr(self, f), dtype=np.float32))
        n = self.x.shape[0]
        for f in _FIELDS:
            if getattr(self, f).shape != (n,):
                raise ValueError(f"{f} must have shape ({n},)")

    @property
    def n(self) -> int:
        return int(self.x.shape[0])

    def soa(self) -> np.ndarray:
        """(7, n) float32 array in the order x, y, z, nx, ny, nz, area."""
        return np.stack([getattr(self, f) for f in _FIELDS])

    @classmethod
    def from_soa(cls, a: np.ndarray) -> "PointCloud":
        a = np.asarray(a, dtype=np.float32)
        return cls(*[a[i] for i in range(7)])

    def subset(self, idx) -> "PointCloud":
        return PointCloud(*[getattr(self, f)[idx] for f in _FIELDS])

    def save(self, path) -> None:
        """Single-file SoA float32 dump: x[n] y[n] z[n] nx[n] ny[n] nz[n] area[n]."""
        self.soa().tofile(str(path))

    @classmethod
    def load(cls, path, n: int | None = None) -> "PointCloud":
        a = np.fromfile(str(path), dtype=np.float32)
        if n is None:
            if a.size % 7:
                raise ValueError("file size is not a multiple of 7 float32 arrays")
            n = a.size // 7
        return cls.from_soa(a[: 7 * n].reshape(7, n))

    def bbox(self):
        lo = np.array([self.x.min(), self.y.min(), self.z.min()], dtype=np.float64)
        hi = np.array([self.x.max(), self.y.max(), self.z.max()], dtype=np.float64)
        return lo, hi


def read_reference_mesh(points_path, area_path, normal_path, n: int) -> PointCloud:
    """Reads the reference's SoA mesh files (compareMie/sphere.cu:94-125):
    ``points`` = [x0..x_{n-1}, y.., z..], ``area`` = [a..], ``normal`` = [nx.., ny.., nz..]."""
    p = np.fromfile(str(points_path), dtype=np.float32, count=3 * n).reshape(3, n)
    a = np.fromfile(str(area_path), dtype=np.float32, count=n)
    q = np.fromfile(str(normal_path), dtype=np.float32, count=3 * n).reshape(3, n)
    return PointCloud(p[0], p[1], p[2], q[0], q[1], q[2], a)


def write_reference_mesh(cloud: PointCloud, prefix) -> tuple[Path, Path, Path]:
    """Writes ``{prefix}_float.binary``, ``{prefix}_area_float.binary`` and
    ``{prefix}_normal_float.binary`` in the reference's layout."""
    prefix = str(prefix)
    pp, ap, np_ = Path(prefix + "_float.binary"), Path(prefix + "_area_float.binary"), Path(prefix + "_normal_float.binary")
    np.stack([cloud.x, cloud.y, cloud.z]).tofile(pp)
    cloud.area.tofile(ap)
    np.stack([cloud.nx, cloud.ny, cloud.nz]).tofile(np_)
    return pp, ap, np_


def _fibonacci_unit(n: int) -> np.ndarray:
    """Unit vectors of the spherical Fibonacci lattice (golden-angle spiral), float64 (n, 3)."""
    i = np.arange(n, dtype=np.float64)
    zc = 1.0 - (2.0 * i + 1.0) / n
    r = np.sqrt(np.maximum(0.0, 1.0 - zc * zc))
    golden = math.pi * (3.0 - math.sqrt(5.0))
    ph = golden * i
    return np.stack([r * np.cos(ph), r * np.sin(ph), zc], axis=1)


def fibonacci_sphere(radius: float, n: int, center=(0.0, 0.0, 0.0)) -> PointCloud:
    """Sphere sampled with n Fibonacci-lattice points, outward normals and equal
    areas 4 pi R^2 / n."""
    u = _fibonacci_unit(n)
    p = u * radius + np.asarray(center, dtype=np.float64)
    a = np.full(n, 4.0 * math.pi * radius * radius / n)
    return PointCloud(p[:, 0], p[:, 1], p[:, 2], u[:, 0], u[:, 1], u[:, 2], a)


def ellipsoid(radii, n: int, center=(0.0, 0.0, 0.0)) -> PointCloud:
    """Ellipsoid x^2/a^2 + y^2/b^2 + z^2/c^2 = 1 sampled by mapping the
    Fibonacci lattice; each point carries the area of its cell (area-weighted
    points) and the analytic normal grad(x^2/a^2 + ...) / |.|.

    The map (u,v,w) -> (a u, b v, c w) scales a unit-sphere area element by
    sqrt((b c u)^2 + (a c v)^2 + (a b w)^2); every lattice cell has area 4 pi / n."""
    a, b, c = (float(r) for r in radii)
    u = _fibonacci_unit(n)
    p = u * np.array([a, b, c])
    g = u / np.array([a, b, c])
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    scale = np.sqrt((b * c * u[:, 0]) ** 2 + (a * c * u[:, 1]) ** 2 + (a * b * u[:, 2]) ** 2)
    area = 4.0 * math.pi / n * scale
    p = p + np.asarray(center, dtype=np.float64)
    return PointCloud(p[:, 0], p[:, 1], p[:, 2], g[:, 0], g[:, 1], g[:, 2], area)
