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


# --------------------------------------------------------------------------
# Fiber height fields (util/geometry.h, fibersim/treePO.cu:83-86)
# --------------------------------------------------------------------------

@dataclasses.dataclass
class HeightField:
    """A fiber surface as a quad grid of vertices, in the reference's layout.

    ``xy`` is float32 [2][numel][numelvert]: plane 0 holds x, plane 1 holds y of
    vertex (j, i), j around the ring and i along the axis; vertex row i sits at
    z_i = i*unitz - period/2 (util/geometry.h:89-90).  The reference reads
    this array from ``mesh/fiber<k>.binary`` (fibersim/treePO.cu:81-86)."""
    xy: np.ndarray
    period: float
    unitz: float

    def __post_init__(self):
        self.xy = np.ascontiguousarray(self.xy, dtype=np.float32)
        if self.xy.ndim != 3 or self.xy.shape[0] != 2:
            raise ValueError("xy must have shape (2, numel, numelvert)")

    @property
    def numel(self) -> int:
        return int(self.xy.shape[1])

    @property
    def numelvert(self) -> int:
        return int(self.xy.shape[2])

    def n_points(self, ring_begin: int = 0, ring_end: int | None = None) -> int:
        ring_end = self.numel - 1 if ring_end is None else ring_end
        return (ring_end - ring_begin + 1) * self.numelvert

    def save(self, path) -> None:
        """Raw float32 [2][numel][numelvert] (the reference's fiber file)."""
        self.xy.tofile(str(path))

    @classmethod
    def load(cls, path, numel: int, numelvert: int, period: float) -> "HeightField":
        a = np.fromfile(str(path), dtype=np.float32, count=2 * numel * numelvert)
        if a.size != 2 * numel * numelvert:
            raise ValueError(f"{path}: expected {2 * numel * numelvert} float32 values, got {a.size}")
        return cls(a.reshape(2, numel, numelvert), float(period), float(np.float32(period) / np.float32(numelvert)))


def gaussian_random_field(shape, spacing, sigma: float, corr_len: float, seed: int) -> np.ndarray:
    """Seeded stationary Gaussian field on a periodic grid, float64.

    White noise filtered in Fourier space so that the covariance is
    sigma^2 exp(-r^2 / corr_len^2) (spectral density proportional to
    exp(-k^2 corr_len^2 / 4)), then rescaled to a sample standard deviation of
    exactly sigma.  Both axes wrap around (the ring closes; the axial wrap only
    correlates the two ends of the segment)."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal(shape)
    k0 = 2 * np.pi * np.fft.fftfreq(shape[0], d=spacing[0])
    k1 = 2 * np.pi * np.fft.rfftfreq(shape[1], d=spacing[1])
    k2 = k0[:, None] ** 2 + k1[None, :] ** 2
    f = np.fft.irfft2(np.fft.rfft2(w) * np.exp(-k2 * corr_len * corr_len / 8.0), s=shape)
    f -= f.mean()
    sd = f.std()
    return f * (sigma / sd) if sd > 0 else f


def _ellipse_arclength_angles(a: float, b: float, numel: int) -> np.ndarray:
    """Parameter angles t_j of numel points equally spaced in arc length on
    (a cos t, b sin t), starting at t = 0."""
    m = 64 * numel
    t = np.linspace(0.0, 2 * np.pi, m + 1)
    ds = np.hypot(a * np.sin(t), b * np.cos(t))
    s = np.concatenate([[0.0], np.cumsum(0.5 * (ds[1:] + ds[:-1]) * (t[1] - t[0]))])
    target = np.arange(numel) * (s[-1] / numel)
    return np.interp(target, s, t)


def ellipse_perimeter(a: float, b: float) -> float:
    """Ramanujan's second approximation."""
    h = ((a - b) / (a + b)) ** 2
    return math.pi * (a + b) * (1 + 3 * h / (10 + math.sqrt(4 - 3 * h)))


def fiber_height_field(radii=(25e-6, 20e-6), length=60e-6, spacing=0.05e-6, scale_spacing=5e-6,
                       scale_step=0.4e-6, scale_tilt_deg=3.0, noise_sigma=0.05e-6, noise_corr=1e-6,
                       seed: int = 0) -> HeightField:
    """Synthetic fiber segment: elliptical cross-section, cuticle sawtooth and
    Gaussian height noise, sampled at ``spacing`` in arc length and along z.

    Vertex (j, i) = e(t_j) + (c(j, i) + g(j, i)) n(t_j), with e the ellipse
    (a cos t, b sin t) at arc-length-uniform t_j, n its outward unit normal,
    g a seeded Gaussian field (``gaussian_random_field``) and c the cuticle
    sawtooth c = step * frac(u), u = (z_i + period/2 + tan(tilt) (x_j + a)) /
    scale_spacing: a ramp rising by ``scale_step`` over each scale, whose
    edges lie in planes tilted by ``scale_tilt_deg`` about the y axis."""
    a, b = float(radii[0]), float(radii[1])
    numel = int(round(ellipse_perimeter(a, b) / spacing))
    numelvert = int(round(length / spacing))
    t = _ellipse_arclength_angles(a, b, numel)
    ex, ey = a * np.cos(t), b * np.sin(t)
    gx, gy = np.cos(t) / a, np.sin(t) / b
    gn = np.hypot(gx, gy)
    nx, ny = gx / gn, gy / gn
    unitz = float(np.float32(length) / np.float32(numelvert))
    z = np.arange(numelvert) * unitz
    u = (z[None, :] + math.tan(math.radians(scale_tilt_deg)) * (ex[:, None] + a)) / scale_spacing
    cut = scale_step * (u - np.floor(u))
    noise = gaussian_random_field((numel, numelvert), (spacing, unitz), noise_sigma, noise_corr, seed)
    d = cut + noise
    xy = np.stack([ex[:, None] + d * nx[:, None], ey[:, None] + d * ny[:, None]])
    return HeightField(xy, float(length), unitz)


def cylinder_height_field(radius=10e-6, length=20e-6, n_points=1_000_000, h=None, h_sigma=0.02e-6,
                          h_corr=0.5e-6, seed: int = 0):
    """Rough circular cylinder with a normal (radial) displacement field h.

    The spacing is chosen so that numel * numelvert ~ n_points; vertex (j, i) =
    (radius + h[j, i]) (cos phi_j, sin phi_j), phi_j = 2 pi j / numel.  Returns
    (HeightField, h) with h float64 [numel][numelvert] (seeded Gaussian field
    unless given)."""
    spacing = math.sqrt(2 * math.pi * radius * length / n_points)
    numel = int(round(2 * math.pi * radius / spacing))
    numelvert = int(round(length / spacing))
    unitz = float(np.float32(length) / np.float32(numelvert))
    if h is None:
        h = gaussian_random_field((numel, numelvert), (2 * math.pi * radius / numel, unitz), h_sigma, h_corr, seed)
    h = np.asarray(h, dtype=np.float64)
    if h.shape != (numel, numelvert):
        raise ValueError(f"h must have shape ({numel}, {numelvert})")
    phi = 2 * np.pi * np.arange(numel) / numel
    r = radius + h
    xy = np.stack([r * np.cos(phi)[:, None], r * np.sin(phi)[:, None]])
    return HeightField(xy, float(length), unitz), h
