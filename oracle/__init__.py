"""ctypes front-end of the FP64 CPU oracle (oracle/po_oracle*.c).

TEST INFRASTRUCTURE ONLY.  Imported by tests/, by __graft_entry__.smoke() and
by bench.py's CPU-baseline leg, where it is the checker, never the thing
measured for the GPU arm and never shipped in the product path.
"""
from __future__ import annotations

import ctypes
import math
import subprocess
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
_LIB_PATH = _HERE / "_build" / "libpo_oracle.so"
_lib = None

f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")


class Illum(ctypes.Structure):
    """Mirror of po_oracle_illum: one (wavelength, incidence, polarisation)."""
    _fields_ = [("lambda_m", ctypes.c_double), ("theta_i", ctypes.c_double), ("phi_i", ctypes.c_double),
                ("eta_re", ctypes.c_double), ("eta_im", ctypes.c_double), ("sigma", ctypes.c_double),
                ("dis", ctypes.c_double), ("mode_te", ctypes.c_int)]


def make_illum(lambda_m, theta_i, phi_i, mode="M", eta=1.55 + 0j, sigma=1e-2, dis=1.0) -> Illum:
    return Illum(float(lambda_m), float(theta_i), float(phi_i), float(np.real(eta)), float(np.imag(eta)),
                 float(sigma), float(dis), 1 if mode in ("E", "TE", 1) else 0)


def build() -> Path:
    """Compiles the oracle with the Makefile beside this file (gcc + OpenMP)."""
    subprocess.run(["make", "-s", "-C", str(_HERE), "lib"], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not _LIB_PATH.exists():
            build()
        L = ctypes.CDLL(str(_LIB_PATH))
        L.po_oracle_currents.argtypes = [ctypes.c_int64] + [f32p] * 7 + [ctypes.POINTER(Illum), ctypes.c_int, f64p]
        L.po_oracle_far_field.argtypes = [ctypes.c_int64, f32p, f32p, f32p, f64p, ctypes.c_double, f64p,
                                          ctypes.c_int, ctypes.c_int, f64p]
        L.po_oracle_far_field_sampled.argtypes = [ctypes.c_int64, f32p, f32p, f32p, f64p, ctypes.c_double, f64p,
                                                  ctypes.c_int, ctypes.c_int, ctypes.c_int64, i64p, f64p]
        L.po_oracle_intensity.argtypes = [ctypes.c_int, ctypes.c_int, f64p, f64p]
        L.po_oracle_intensity_sampled.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int64, i64p, f64p, f64p]
        L.po_oracle_solve_direct.argtypes = [ctypes.c_int64] + [f32p] * 7 + [ctypes.POINTER(Illum), f64p,
                                                                            ctypes.c_int, ctypes.c_int, f64p]
        L.po_oracle_octree.argtypes = [ctypes.c_int, f32p, f32p, f32p, f32p, f32p, ctypes.c_int, i32p, i32p, f32p]
        L.po_oracle_octree.restype = ctypes.c_int
        L.po_oracle_interp.argtypes = [ctypes.c_int] * 5 + [f64p, f64p]
        L.po_oracle_interp.restype = ctypes.c_int
        L.po_oracle_solve_tree.argtypes = [ctypes.c_int] + [f32p] * 7 + [ctypes.POINTER(Illum), f32p, f32p,
                                                                          ctypes.c_int, i32p, i32p, ctypes.c_int, f64p]
        L.po_oracle_solve_tree.restype = ctypes.c_int
        L.po_oracle_fresnel.argtypes = [ctypes.c_double] * 5 + [f64p, f64p]
        L.po_oracle_height_field.argtypes = [f32p, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                             ctypes.c_int, ctypes.c_int] + [f32p] * 7
        L.po_oracle_height_field.restype = ctypes.c_int
        L.po_oracle_solve_sampled_d.argtypes = [ctypes.c_int64] + [f64p] * 7 + [ctypes.POINTER(Illum), ctypes.c_int,
                                                                               ctypes.c_int, ctypes.c_int64, i64p, f64p]
        L.po_oracle_solve_direct_d.argtypes = [ctypes.c_int64] + [f64p] * 7 + [ctypes.POINTER(Illum), f64p,
                                                                              ctypes.c_int, ctypes.c_int, f64p]
        L.po_oracle_fields_sampled_d.argtypes = [ctypes.c_int64] + [f64p] * 7 + [
            ctypes.POINTER(Illum), ctypes.c_int, ctypes.c_int, ctypes.c_int64, i64p, ctypes.c_int, f64p]
        L.po_oracle_project_sampled.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int64, i64p, f64p, f64p]
        L.po_oracle_average.argtypes = [f32p, ctypes.c_int, ctypes.c_int, f32p, ctypes.c_int, ctypes.c_int]
        L.po_oracle_z0.restype = ctypes.c_double
        L.po_oracle_num_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _g(cloud):
    return [cloud.x, cloud.y, cloud.z, cloud.nx, cloud.ny, cloud.nz, cloud.area]


def z0() -> float:
    return lib().po_oracle_z0()


def num_threads() -> int:
    return lib().po_oracle_num_threads()


def currents(cloud, il: Illum, scale: bool = True) -> np.ndarray:
    """(n, 6) complex128 [Jx,Jy,Jz,Mx,My,Mz]; scaled by area and E/H prefactors if `scale`."""
    out = np.zeros((cloud.n, 12))
    lib().po_oracle_currents(cloud.n, *_g(cloud), ctypes.byref(il), 1 if scale else 0, out)
    return out.view(np.complex128)


def far_field(cloud, cur: np.ndarray, k0: float, center, n_theta: int, n_phi: int) -> np.ndarray:
    """(n_theta*n_phi, 6) complex128 far field of scaled currents about `center`."""
    c12 = np.ascontiguousarray(cur, dtype=np.complex128).view(np.float64).reshape(-1)
    out = np.zeros((n_theta * n_phi, 12))
    lib().po_oracle_far_field(cloud.n, cloud.x, cloud.y, cloud.z, c12, k0,
                              np.asarray(center, dtype=np.float64), n_theta, n_phi, out)
    return out.view(np.complex128)


def far_field_sampled(cloud, cur, k0, center, n_theta, n_phi, dirs) -> np.ndarray:
    dirs = np.ascontiguousarray(dirs, dtype=np.int64)
    c12 = np.ascontiguousarray(cur, dtype=np.complex128).view(np.float64).reshape(-1)
    out = np.zeros((dirs.size, 12))
    lib().po_oracle_far_field_sampled(cloud.n, cloud.x, cloud.y, cloud.z, c12, k0,
                                      np.asarray(center, dtype=np.float64), n_theta, n_phi, dirs.size, dirs, out)
    return out.view(np.complex128)


def intensity(fields: np.ndarray, n_theta: int, n_phi: int) -> np.ndarray:
    f = np.ascontiguousarray(fields, dtype=np.complex128).view(np.float64).reshape(-1)
    out = np.zeros(n_theta * n_phi)
    lib().po_oracle_intensity(n_theta, n_phi, f, out)
    return out.reshape(n_theta, n_phi)


def intensity_sampled(fields, n_theta, n_phi, dirs) -> np.ndarray:
    dirs = np.ascontiguousarray(dirs, dtype=np.int64)
    f = np.ascontiguousarray(fields, dtype=np.complex128).view(np.float64).reshape(-1)
    out = np.zeros(dirs.size)
    lib().po_oracle_intensity_sampled(n_theta, n_phi, dirs.size, dirs, f, out)
    return out


def solve_direct(cloud, il: Illum, n_theta: int, n_phi: int, center=(0.0, 0.0, 0.0)) -> np.ndarray:
    """Plain FP64 depth-0 solve: intensity (n_theta, n_phi) float64."""
    out = np.zeros(n_theta * n_phi)
    lib().po_oracle_solve_direct(cloud.n, *_g(cloud), ctypes.byref(il),
                                 np.asarray(center, dtype=np.float64), n_theta, n_phi, out)
    return out.reshape(n_theta, n_phi)


def octree(cloud, box_min, box_max, depth: int):
    """Reference octree (util/tree.h:289-715): (perm, node_range[(8^(d+1)-1)/7, 2], node_box[.., 6])."""
    nn = (8 ** (depth + 1) - 1) // 7
    perm = np.zeros(cloud.n, dtype=np.int32)
    rng = np.zeros(2 * nn, dtype=np.int32)
    box = np.zeros(6 * nn, dtype=np.float32)
    rc = lib().po_oracle_octree(cloud.n, cloud.x, cloud.y, cloud.z, np.asarray(box_min, dtype=np.float32),
                                np.asarray(box_max, dtype=np.float32), depth, perm, rng, box)
    if rc:
        raise ValueError("unsupported octree depth")
    return perm, rng.reshape(nn, 2), box.reshape(nn, 6)


def interp(pattern: np.ndarray, th_p: int, ph_p: int, nyquist_quirk: bool = True) -> np.ndarray:
    """interpFFT restated (util/interpolation.h:11-80): (th_c, ph_c) complex -> (th_p, ph_p)."""
    th_c, ph_c = pattern.shape
    src = np.ascontiguousarray(pattern, dtype=np.complex128).view(np.float64).reshape(-1)
    out = np.zeros(2 * th_p * ph_p)
    rc = lib().po_oracle_interp(th_c, ph_c, th_p, ph_p, 1 if nyquist_quirk else 0, src, out)
    if rc:
        raise ValueError("interpolation can only upsample")
    return out.view(np.complex128).reshape(th_p, ph_p)


def solve_tree(cloud, il: Illum, box_min, box_max, depth: int, n_theta, n_phi,
               nyquist_quirk: bool = True) -> np.ndarray:
    """Hierarchical solve restated from compareMie/sphere.cu:212-936."""
    nth = np.asarray(n_theta, dtype=np.int32)
    nph = np.asarray(n_phi, dtype=np.int32)
    out = np.zeros(int(nth[0]) * int(nph[0]))
    rc = lib().po_oracle_solve_tree(cloud.n, *_g(cloud), ctypes.byref(il), np.asarray(box_min, dtype=np.float32),
                                    np.asarray(box_max, dtype=np.float32), depth, nth, nph,
                                    1 if nyquist_quirk else 0, out)
    if rc:
        raise ValueError(f"unsupported tree configuration (rc={rc})")
    return out.reshape(int(nth[0]), int(nph[0]))


def fresnel(theta, n0=1.0 + 0j, nt=1.55 + 0j):
    rs = np.zeros(2)
    rp = np.zeros(2)
    lib().po_oracle_fresnel(float(theta), n0.real, n0.imag, nt.real, nt.imag, rs, rp)
    return complex(rs[0], rs[1]), complex(rp[0], rp[1])


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def height_field(hf, ring_begin: int = 0, ring_end=None):
    """util/geometry.h:76-179 restated in float (po_oracle_geometry.c).
    Returns ((7, n) float32 x, y, z, nx, ny, nz, area; origin-vertex flag)."""
    ring_end = hf.numel - 1 if ring_end is None else ring_end
    n = (ring_end - ring_begin + 1) * hf.numelvert
    out = np.zeros((7, n), dtype=np.float32)
    xy = np.ascontiguousarray(hf.xy, dtype=np.float32)
    bad = lib().po_oracle_height_field(xy.ravel(), hf.numel, hf.numelvert, hf.period, hf.unitz, ring_begin,
                                       ring_end, *[out[k] for k in range(7)])
    return out, bool(bad)


def average(pattern, nth_out: int, nph_out: int) -> np.ndarray:
    """util/fields.h:206-234 (average_cpu) restated in float."""
    p = np.ascontiguousarray(pattern, dtype=np.float32)
    out = np.zeros((nth_out, nph_out), dtype=np.float32)
    lib().po_oracle_average(p.ravel(), p.shape[0], p.shape[1], out.ravel(), nth_out, nph_out)
    return out


def solve_direct_f64(samples, il: Illum, n_theta: int, n_phi: int, center=(0.0, 0.0, 0.0)) -> np.ndarray:
    """Depth-0 FP64 solve of (7, n) float64 samples (x, y, z, nx, ny, nz, area)."""
    a = np.ascontiguousarray(samples, dtype=np.float64)
    out = np.zeros((n_theta, n_phi), dtype=np.float64)
    c = np.ascontiguousarray(center, dtype=np.float64)
    lib().po_oracle_solve_direct_d(a.shape[1], *[np.ascontiguousarray(a[k]) for k in range(7)], ctypes.byref(il),
                                   c, n_theta, n_phi, out)
    return out


def solve_sampled_f64(samples, il: Illum, n_theta: int, n_phi: int, dirs) -> np.ndarray:
    """FP64 intensity of (7, n) float64 samples at the flat direction indices dirs."""
    a = np.ascontiguousarray(samples, dtype=np.float64)
    d = np.ascontiguousarray(dirs, dtype=np.int64)
    out = np.zeros(d.size, dtype=np.float64)
    lib().po_oracle_solve_sampled_d(a.shape[1], *[np.ascontiguousarray(a[k]) for k in range(7)], ctypes.byref(il),
                                    n_theta, n_phi, d.size, d, out)
    return out


def fields_sampled_f64(samples, il: Illum, n_theta: int, n_phi: int, dirs, per_point: bool = False) -> np.ndarray:
    """FP64 far field of (7, n) float64 samples at the flat direction indices
    dirs: (m, 6) complex128, or (n, m, 6) with every point's own field."""
    a = np.ascontiguousarray(samples, dtype=np.float64)
    d = np.ascontiguousarray(dirs, dtype=np.int64)
    n = a.shape[1]
    out = np.zeros(((n if per_point else 1) * d.size, 12), dtype=np.float64)
    lib().po_oracle_fields_sampled_d(n, *[np.ascontiguousarray(a[k]) for k in range(7)], ctypes.byref(il), n_theta,
                                     n_phi, d.size, d, 1 if per_point else 0, out)
    f = out.view(np.complex128)
    return f.reshape(n, d.size, 6) if per_point else f


def project_sampled(fields, n_theta: int, n_phi: int, dirs) -> np.ndarray:
    """Transverse field E' (util/fields.h:172-204; intensity = |E'|^2) of
    fields (m, 6) at the flat direction indices dirs: (m, 3) complex128."""
    d = np.ascontiguousarray(dirs, dtype=np.int64)
    f = np.ascontiguousarray(fields, dtype=np.complex128).view(np.float64).reshape(-1)
    out = np.zeros((d.size, 6), dtype=np.float64)
    lib().po_oracle_project_sampled(n_theta, n_phi, d.size, d, f, out)
    return out.view(np.complex128)


def point_gradient_fd(samples, il: Illum, n_theta: int, n_phi: int, dirs, weights, points, steps) -> np.ndarray:
    """Central differences, per point and per component, of the FP64 loss
    L = sum_j weights[j] * I(dirs[j]) of (7, n) float64 samples.

    Perturbing one sample q of one point p changes the field only by that
    point's own contribution f_p, so the difference is taken on f_p alone:
      dL/dq = sum_j w_j 2 Re(conj(E'_j(F)) . E'_j(f_p(q + h) - f_p(q - h))) / (2 h)
    (E' the linear transverse projection, F the total field).  This is the
    same central difference as (L(q + h) - L(q - h)) / 2h up to O(h^2), without
    the cancellation of two nearly equal sums over all points.
    steps: (7,) step per component (the area step is taken relative).
    Returns (7, len(points))."""
    a = np.ascontiguousarray(samples, dtype=np.float64)
    dirs = np.ascontiguousarray(dirs, dtype=np.int64)
    w = np.asarray(weights, dtype=np.float64)
    ep = project_sampled(fields_sampled_f64(a, il, n_theta, n_phi, dirs), n_theta, n_phi, dirs)
    pts = np.asarray(points)
    pert = np.repeat(a[:, pts], 14, axis=1).reshape(7, pts.size, 7, 2)  # [comp][point][q][+/-]
    hs = np.zeros((pts.size, 7))
    for q in range(7):
        h = steps[q] * (a[6, pts] if q == 6 else 1.0)
        hs[:, q] = h
        pert[q, :, q, 0] += h
        pert[q, :, q, 1] -= h
    f = fields_sampled_f64(pert.reshape(7, -1), il, n_theta, n_phi, dirs, per_point=True)
    f = f.reshape(pts.size, 7, 2, dirs.size, 6)
    df = (f[:, :, 0] - f[:, :, 1]).reshape(-1, 6)
    dp = project_sampled(df, n_theta, n_phi, np.tile(dirs, pts.size * 7)).reshape(pts.size, 7, dirs.size, 3)
    g = 2.0 * np.einsum("j,pqjc->pq", w, np.real(np.conj(ep)[None, None] * dp)) / (2.0 * hs)
    return g.T
