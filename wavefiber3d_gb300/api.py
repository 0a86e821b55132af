"""Python mirror of the reference's PO operators, running on the CUDA library.

Names follow the reference's host functions so that a driver written against
util/*.h maps one to one:

  compute_local_tangent_plane   util/tangentplane.h:84   (+ field_times_area fields.h:123,
                                                          multiply_current_factor fields.h:147)
  build_octree                  util/tree.h:290          (+ active lists, sphere.cu:255-307)
  current_times_green_center    util/fields.h:41 + per-node thrust::reduce (depth 0)
  copyandinterp                 util/interpolation.h:82
  compute_intensity             util/fields.h:172
  Solver.solve                  the driver main() of compareMie/sphere.cu:212-936

Arrays are torch tensors on the current CUDA device (PyTorch is used only for
device memory and streams).  Errors raise WavePOError instead of exiting the
process as the reference does (util/helper_cuda.h:583-595).
"""
from __future__ import annotations

import ctypes
import dataclasses
import math
from typing import Sequence

import numpy as np

from . import _lib
from ._lib import (PO_INTERP_FFT, PO_INTERP_TENSOR, PO_LEAF_AUTO, PO_LEAF_TCGEN05, PO_LEAF_WARP, PO_POL_TE,
                   PO_POL_TM, PO_PREC_FP32, PO_PREC_FP64, PO_PREC_SPLIT_BF16, PO_THETA_DOUBLE_COVER,
                   PO_THETA_REFERENCE, WavePOError, check)

__all__ = ["Config", "Illumination", "Solver", "compute_local_tangent_plane", "build_octree",
           "current_times_green_center", "copyandinterp", "compute_intensity", "wavelength_from_index",
           "incidence_from_index", "WavePOError", "PO_POL_TM", "PO_POL_TE", "PO_PREC_FP32", "PO_PREC_FP64", "PO_PREC_SPLIT_BF16",
           "PO_THETA_DOUBLE_COVER", "PO_THETA_REFERENCE", "PO_INTERP_FFT", "PO_INTERP_TENSOR", "PO_LEAF_AUTO",
           "PO_LEAF_WARP", "PO_LEAF_TCGEN05"]


def _torch():
    import torch
    return torch


def _stream_ptr(stream=None):
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _dev(t, dtype=None):
    torch = _torch()
    if not isinstance(t, torch.Tensor):
        t = torch.as_tensor(np.asarray(t))
    if dtype is not None:
        t = t.to(dtype)
    return t.cuda().contiguous()


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def wavelength_from_index(i: int, n: int = 25, lo_nm: float = 400.0, hi_nm: float = 700.0) -> float:
    """Reference wavelength list (compareMie/sphere.cu:489): lo + (hi-lo)/n * i nm, in metres."""
    return (lo_nm + (hi_nm - lo_nm) / n * i) * 1e-9


def incidence_from_index(theta_index: int, phi_index: int, n_theta: int = 180, n_phi: int = 360):
    """Incident angles of fibersim/treePO.cu:559-564 from the 180 x 360 index grid."""
    th = -math.pi / 2 + 1e-10 + math.pi / n_theta * theta_index
    ph = 2 * math.pi / n_phi * phi_index
    return th, ph


@dataclasses.dataclass
class Config:
    """Mirror of po_config.  Use Config.reference_rule for the reference's grids."""
    max_depth: int
    n_theta: Sequence[int]
    n_phi: Sequence[int]
    box_min: Sequence[float]
    box_max: Sequence[float]
    precision: int = PO_PREC_FP32
    theta_mode: int = PO_THETA_DOUBLE_COVER
    nyquist_quirk: bool = True
    distance: float = 1.0
    interp_method: int = PO_INTERP_TENSOR
    max_workspace_bytes: int = 0
    interp_tile: int = 0
    leaf_kernel: int = PO_LEAF_AUTO
    leaf_slots: int = 0

    @classmethod
    def reference_rule(cls, max_depth, n_theta_out, n_phi_out, box_min, box_max, theta_extent, phi_extent,
                       ratio, beta=6.0, lambda_min=0.4e-6, **kw):
        c = _lib.po_config()
        bmin = (ctypes.c_float * 3)(*box_min)
        bmax = (ctypes.c_float * 3)(*box_max)
        check(_lib.load().po_config_init(ctypes.byref(c), max_depth, n_theta_out, n_phi_out, bmin, bmax,
                                         theta_extent, phi_extent, ratio, beta, lambda_min))
        return cls(max_depth, list(c.n_theta[:max_depth + 1]), list(c.n_phi[:max_depth + 1]), list(box_min),
                   list(box_max), **kw)

    def to_c(self) -> _lib.po_config:
        c = _lib.po_config()
        c.max_depth = self.max_depth
        for i, (t, p) in enumerate(zip(self.n_theta, self.n_phi)):
            c.n_theta[i] = int(t)
            c.n_phi[i] = int(p)
        for a in range(3):
            c.box_min[a] = float(self.box_min[a])
            c.box_max[a] = float(self.box_max[a])
        c.precision = int(self.precision)
        c.theta_mode = int(self.theta_mode)
        c.nyquist_quirk = 1 if self.nyquist_quirk else 0
        c.distance = float(self.distance)
        c.interp_method = int(self.interp_method)
        c.max_workspace_bytes = int(self.max_workspace_bytes)
        c.interp_tile = int(self.interp_tile)
        c.leaf_kernel = int(self.leaf_kernel)
        c.leaf_slots = int(self.leaf_slots)
        return c


@dataclasses.dataclass
class Illumination:
    """Mirror of po_illum: every (wavelength, incidence, polarisation) is one pattern."""
    wavelengths_m: Sequence[float]
    theta_i: Sequence[float]
    phi_i: Sequence[float]
    pol_mask: int = PO_POL_TM
    eta: complex = 1.55 + 0j
    sigma: float = 1e-2

    @property
    def n_patterns(self) -> int:
        npol = (1 if self.pol_mask & PO_POL_TM else 0) + (1 if self.pol_mask & PO_POL_TE else 0)
        return len(self.wavelengths_m) * len(self.theta_i) * npol

    def to_c(self):
        lam = np.ascontiguousarray(self.wavelengths_m, dtype=np.float64)
        th = np.ascontiguousarray(self.theta_i, dtype=np.float64)
        ph = np.ascontiguousarray(self.phi_i, dtype=np.float64)
        if th.shape != ph.shape:
            raise ValueError("theta_i and phi_i must have the same length")
        il = _lib.po_illum(lam.size, lam.ctypes.data, th.size, th.ctypes.data, ph.ctypes.data, int(self.pol_mask),
                           float(np.real(self.eta)), float(np.imag(self.eta)), float(self.sigma))
        return il, (lam, th, ph)


class Solver:
    """Whole PO solve (po_create / po_solve / po_destroy)."""

    def __init__(self, config: Config):
        self.config = config
        self._c = config.to_c()
        h = ctypes.c_void_p()
        check(_lib.load().po_create(ctypes.byref(h), ctypes.byref(self._c)))
        self._h = h
        self.last_report: dict = {}

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().po_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def out_shape(self, illum: Illumination):
        npol = (1 if illum.pol_mask & PO_POL_TM else 0) + (1 if illum.pol_mask & PO_POL_TE else 0)
        return (len(illum.wavelengths_m), len(illum.theta_i), npol, int(self.config.n_theta[0]),
                int(self.config.n_phi[0]))

    def check(self, stream=None):
        """po_check: waits for the stream; raises if a bounded device wait of
        this context's kernels gave up since the last check."""
        check(_lib.load().po_check(self._h, _stream_ptr(stream)))

    def solve(self, cloud, illum: Illumination, out=None, stream=None, report: bool = True):
        """cloud: PointCloud (host numpy) or a (7, n) float32 CUDA tensor / tuple of 7 CUDA tensors.
        Returns intensity [L][I][P][n_theta][n_phi] float32 (numpy for host geometry without `out`,
        else the CUDA tensor `out` or a new CUDA tensor).  report=True fills `last_report` (per-kernel
        times: the call then waits for the solve to finish); report=False leaves a device-output solve
        asynchronous on the stream and sets `last_report` to None."""
        torch = _torch()
        il, keep = illum.to_c()
        host = hasattr(cloud, "soa")
        if host:
            soa = np.ascontiguousarray(cloud.soa(), dtype=np.float32)
            n = soa.shape[1]
            base = soa.ctypes.data
            ptrs = [base + 4 * n * k for k in range(7)]
            g = _lib.po_geometry(n, *ptrs, 0)
        else:
            arrs = [cloud[k] for k in range(7)]
            on_dev = arrs[0].is_cuda
            for a in arrs:
                if not (a.is_cuda == on_dev and a.dtype == torch.float32 and a.is_contiguous()):
                    raise ValueError("geometry must be 7 contiguous float32 arrays, all on the GPU or all on the host")
            n = arrs[0].numel()
            g = _lib.po_geometry(n, *[a.data_ptr() for a in arrs], 1 if on_dev else 0)
        rep = _lib.po_report()
        rep_ref = ctypes.byref(rep) if report else None
        shape = self.out_shape(illum)
        if out is None and host:
            res = np.empty(shape, dtype=np.float32)
            check(_lib.load().po_solve(self._h, ctypes.byref(g), ctypes.byref(il), res.ctypes.data, 0,
                                       _stream_ptr(stream), rep_ref))
        else:
            res = out if out is not None else torch.empty(shape, dtype=torch.float32, device="cuda")
            if not (res.is_contiguous() and res.dtype == torch.float32 and res.numel() == int(np.prod(shape))):
                raise ValueError(f"out must be a contiguous float32 tensor with {int(np.prod(shape))} elements")
            check(_lib.load().po_solve(self._h, ctypes.byref(g), ctypes.byref(il), ctypes.c_void_p(res.data_ptr()),
                                       1 if res.is_cuda else 0, _stream_ptr(stream), rep_ref))
        self.last_report = rep.as_dict() if report else None
        del keep
        return res

    def grad(self, samples, illum: Illumination, dl_di, with_intensity: bool = False, stream=None):
        """Gradient of a loss with respect to the surface samples (po_grad).

        samples: (7, n) float32 CUDA tensor (x, y, z, nx, ny, nz, area);
        dl_di: dL/dI shaped like the solve output.  Returns the (7, n) float32
        gradient (and the recomputed intensity if with_intensity)."""
        torch = _torch()
        g7 = samples.to(device="cuda", dtype=torch.float32).contiguous()
        n = g7.shape[1]
        g = _lib.po_geometry(n, *[g7[k].data_ptr() for k in range(7)], 1)
        il, keep = illum.to_c()
        shape = self.out_shape(illum)
        w = dl_di.to(device="cuda", dtype=torch.float32).contiguous()
        if w.numel() != int(np.prod(shape)):
            raise ValueError(f"dl_di must have {int(np.prod(shape))} elements")
        grad = torch.empty((7, max(n, 1)), dtype=torch.float32, device="cuda")
        inten = torch.empty(shape, dtype=torch.float32, device="cuda") if with_intensity else None
        rep = _lib.po_report()
        check(_lib.load().po_grad(self._h, ctypes.byref(g), ctypes.byref(il), ctypes.c_void_p(w.data_ptr()),
                                  ctypes.c_void_p(grad.data_ptr()),
                                  ctypes.c_void_p(inten.data_ptr()) if inten is not None else None,
                                  _stream_ptr(stream), ctypes.byref(rep)))
        self.last_report = rep.as_dict()
        del keep
        return (grad[:, :n], inten) if with_intensity else grad[:, :n]


def compute_local_tangent_plane(x, y, z, nx, ny, nz, area, wavelength_m, theta_i, phi_i, mode="M", eta=1.55 + 0j,
                                sigma=1e-2, distance=1.0, scale=True, stream=None):
    """Surface currents (n, 6) complex64 [Jx,Jy,Jz,Mx,My,Mz]: computeLocalTangentPlane
    (tangentplane.h:84) and, if `scale`, field_times_area and multiply_current_factor."""
    torch = _torch()
    t = [_dev(a, torch.float32) for a in (x, y, z, nx, ny, nz, area)]
    n = t[0].numel()
    out = torch.empty((n, 6), dtype=torch.complex64, device="cuda")
    pol = PO_POL_TE if mode in ("E", "TE", PO_POL_TE) else PO_POL_TM
    check(_lib.load().po_tangent_plane_currents(n, *[_ptr(a) for a in t], wavelength_m, theta_i, phi_i, pol,
                                                float(np.real(eta)), float(np.imag(eta)), sigma, distance,
                                                1 if scale else 0, _ptr(out), _stream_ptr(stream)))
    return out


def build_octree(x, y, z, box_min, box_max, depth: int, heap_ranges: bool = True, stream=None):
    """Octree of util/tree.h:290: returns (perm, heap_range) where perm[i] is the input
    index of the point at tree position i and heap_range[h] = (begin, end) of heap node h."""
    torch = _torch()
    t = [_dev(a, torch.float32) for a in (x, y, z)]
    n = t[0].numel()
    perm = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    nn = (8 ** (depth + 1) - 1) // 7
    hr = torch.empty((nn, 2), dtype=torch.int32, device="cuda") if heap_ranges else None
    bmin = (ctypes.c_float * 3)(*box_min)
    bmax = (ctypes.c_float * 3)(*box_max)
    check(_lib.load().po_build_octree(n, *[_ptr(a) for a in t], bmin, bmax, depth, _ptr(perm),
                                      _ptr(hr) if hr is not None else None, _stream_ptr(stream)))
    return perm[:n], hr


def current_times_green_center(x, y, z, currents, k, center, n_theta, n_phi, precision=PO_PREC_FP32, stream=None):
    """Depth-0 far field: sum_p exp(+i k s.(x_p - center)) currents_p on the
    n_theta x n_phi grid; returns (6, n_theta, n_phi) complex64."""
    torch = _torch()
    t = [_dev(a, torch.float32) for a in (x, y, z)]
    cur = _dev(currents, torch.complex64)
    n = t[0].numel()
    out = torch.empty((6, n_theta, n_phi), dtype=torch.complex64, device="cuda")
    c = (ctypes.c_double * 3)(*center)
    check(_lib.load().po_far_field_direct(n, *[_ptr(a) for a in t], _ptr(cur), float(k), c, n_theta, n_phi,
                                          precision, _ptr(out), _stream_ptr(stream)))
    return out


def copyandinterp(patterns, th_p, ph_p, theta_mode=PO_THETA_REFERENCE, nyquist_quirk=True, stream=None):
    """Trigonometric upsampling of (batch, th_c, ph_c) complex patterns (interpolation.h:82)."""
    torch = _torch()
    p = _dev(patterns, torch.complex64)
    squeeze = p.dim() == 2
    if squeeze:
        p = p.unsqueeze(0)
    b, th_c, ph_c = p.shape
    out = torch.empty((b, th_p, ph_p), dtype=torch.complex64, device="cuda")
    check(_lib.load().po_interp_fft(_ptr(p), th_c, ph_c, _ptr(out), th_p, ph_p, b, theta_mode,
                                    1 if nyquist_quirk else 0, _stream_ptr(stream)))
    return out[0] if squeeze else out


def compute_intensity(fields, stream=None):
    """computeintensity (fields.h:172): (6, n_theta, n_phi) complex -> (n_theta, n_phi) float32."""
    torch = _torch()
    f = _dev(fields, torch.complex64)
    _, nth, nph = f.shape
    out = torch.empty((nth, nph), dtype=torch.float32, device="cuda")
    check(_lib.load().po_compute_intensity(_ptr(f), nth, nph, _ptr(out), _stream_ptr(stream)))
    return out


def height_field_points(hf, ring_begin: int = 0, ring_end=None, stream=None):
    """Surface samples of a fiber height field (util/geometry.h:76-179,
    set_sourcepoint): one sample per quad of the ring segment
    [ring_begin, ring_end] (default: the full ring).  ``hf`` is a
    geometry.HeightField.  Returns a (7, n) float32 CUDA tensor in the order
    x, y, z, nx, ny, nz, area, n = (ring_end - ring_begin + 1) * numelvert,
    sample (j, i) at i * (ring_end - ring_begin + 1) + (j - ring_begin)."""
    torch = _torch()
    ring_end = hf.numel - 1 if ring_end is None else int(ring_end)
    h = _dev(hf.xy, torch.float32)
    n = (ring_end - ring_begin + 1) * hf.numelvert
    out = torch.empty((7, max(n, 1)), dtype=torch.float32, device="cuda")
    check(_lib.load().po_height_field_points(_ptr(h), hf.numel, hf.numelvert, float(hf.period), float(hf.unitz),
                                             int(ring_begin), ring_end, *[_ptr(out[k]) for k in range(7)],
                                             _stream_ptr(stream)))
    return out[:, :n]


def average_pattern(patterns, nth_out: int = 180, nph_out: int = 360, stream=None):
    """Box average of (..., nth_in, nph_in) float32 patterns onto nth_out x
    nph_out (util/fields.h:206-234, average_cpu, with its integer ratios)."""
    torch = _torch()
    p = _dev(patterns, torch.float32)
    lead = p.shape[:-2]
    nth_in, nph_in = p.shape[-2:]
    b = int(np.prod(lead)) if lead else 1
    out = torch.empty((*lead, nth_out, nph_out), dtype=torch.float32, device="cuda")
    check(_lib.load().po_average_pattern(_ptr(p), nth_in, nph_in, _ptr(out), nth_out, nph_out, b,
                                         _stream_ptr(stream)))
    return out


def height_field_points_tensor(xy, period: float, unitz: float, ring_begin: int, ring_end: int, stream=None):
    """po_height_field_points on a (2, numel, numelvert) float32 CUDA tensor; returns (7, n)."""
    torch = _torch()
    x = xy.to(device="cuda", dtype=torch.float32).contiguous()
    numel, numelvert = int(x.shape[1]), int(x.shape[2])
    n = (ring_end - ring_begin + 1) * numelvert
    out = torch.empty((7, max(n, 1)), dtype=torch.float32, device="cuda")
    check(_lib.load().po_height_field_points(_ptr(x), numel, numelvert, float(period), float(unitz), int(ring_begin),
                                             int(ring_end), *[_ptr(out[k]) for k in range(7)], _stream_ptr(stream)))
    return out[:, :n]


def height_field_adjoint(xy, period: float, unitz: float, ring_begin: int, ring_end: int, grad_samples, stream=None):
    """dL/d(vertex xy) (2, numel, numelvert) from dL/d(samples) (7, n)."""
    torch = _torch()
    x = xy.to(device="cuda", dtype=torch.float32).contiguous()
    numel, numelvert = int(x.shape[1]), int(x.shape[2])
    g = grad_samples.to(device="cuda", dtype=torch.float32).contiguous()
    out = torch.empty_like(x)
    check(_lib.load().po_height_field_adjoint(_ptr(x), numel, numelvert, float(period), float(unitz),
                                              int(ring_begin), int(ring_end), _ptr(g), _ptr(out),
                                              _stream_ptr(stream)))
    return out


class Batch:
    """Independent solves captured in one CUDA graph (po_batch_*).

    ``Batch(configs, n_streams)`` creates one engine context per item;
    ``prepare(samples, illums)`` builds every octree and table and captures the
    pattern computations of all items into a graph (items spread over
    ``n_streams`` concurrent branches); ``launch()`` replays it.  Geometry is a
    list of (7, n) float32 CUDA tensors; results are CUDA tensors
    ``self.outputs[i]`` shaped like Solver.solve's."""

    def __init__(self, configs, n_streams: int = 8):
        self.configs = list(configs)
        arr = (_lib.po_config * len(self.configs))(*[c.to_c() for c in self.configs])
        h = ctypes.c_void_p()
        check(_lib.load().po_batch_create(ctypes.byref(h), len(self.configs), arr, int(n_streams)))
        self._h = h
        self._keep = []
        self.outputs = []

    def prepare(self, samples, illums, stream=None):
        torch = _torch()
        if len(samples) != len(self.configs) or len(illums) != len(self.configs):
            raise ValueError("one geometry and one illumination per configuration")
        items = (_lib.po_batch_item * len(self.configs))()
        keep, outs = [], []
        for i, (s, il, cfg) in enumerate(zip(samples, illums, self.configs)):
            g7 = s.to(device="cuda", dtype=torch.float32).contiguous()
            n = g7.shape[1]
            ilc, ka = il.to_c()
            npol = (1 if il.pol_mask & PO_POL_TM else 0) + (1 if il.pol_mask & PO_POL_TE else 0)
            out = torch.empty((len(il.wavelengths_m), len(il.theta_i), npol, int(cfg.n_theta[0]), int(cfg.n_phi[0])),
                              dtype=torch.float32, device="cuda")
            items[i].geom = _lib.po_geometry(n, *[g7[k].data_ptr() for k in range(7)], 1)
            items[i].illum = ilc
            items[i].intensity = out.data_ptr()
            keep += [g7, ka]
            outs.append(out)
        check(_lib.load().po_batch_prepare(self._h, items, _stream_ptr(stream)))
        self._keep, self.outputs = keep, outs
        return outs

    def launch(self, stream=None):
        check(_lib.load().po_batch_launch(self._h, _stream_ptr(stream)))
        return self.outputs

    def check(self, stream=None):
        """po_batch_check: waits for the stream; raises if an item's kernels
        gave up a bounded device wait."""
        check(_lib.load().po_batch_check(self._h, _stream_ptr(stream)))

    def info(self) -> dict:
        nodes, ws, ms = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_double()
        check(_lib.load().po_batch_info(self._h, ctypes.byref(nodes), ctypes.byref(ws), ctypes.byref(ms)))
        return {"graph_nodes": nodes.value, "workspace_bytes": ws.value, "ms_prepare": ms.value}

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().po_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def selftest_device_waits(which: int, stream=None) -> int:
    """po_selftest_device_waits: the status (an int, not raised) that the
    deliberately failing kernel launch of case `which` (1..3) reported."""
    return int(_lib.load().po_selftest_device_waits(int(which), _stream_ptr(stream)))
