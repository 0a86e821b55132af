"""ctypes binding of libwavepo.so (the C ABI declared in include/wavepo.h).

The library is built in-tree by wavefiber3d_gb300/build.py.  There is no
fallback: if the library is missing, loading fails with an error that says how
to build it.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_build" / "libwavepo.so"

PO_MAX_DEPTH = 10
PO_OK = 0
PO_PREC_FP32, PO_PREC_FP64, PO_PREC_SPLIT_BF16, PO_PREC_SPLIT_FP16 = 0, 1, 2, 3
PO_THETA_DOUBLE_COVER, PO_THETA_REFERENCE = 0, 1
PO_POL_TM, PO_POL_TE = 1, 2
PO_INTERP_FFT, PO_INTERP_TENSOR = 0, 1
PO_LEAF_AUTO, PO_LEAF_WARP, PO_LEAF_TCGEN05 = 0, 1, 2

STATUS_NAMES = {0: "PO_OK", 1: "PO_ERR_INVALID_ARGUMENT", 2: "PO_ERR_CUDA", 3: "PO_ERR_OUT_OF_MEMORY",
                4: "PO_ERR_UNSUPPORTED", 5: "PO_ERR_TIMEOUT", 6: "PO_ERR_INTERNAL"}


class WavePOError(RuntimeError):
    def __init__(self, status: int, message: str):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")


class po_config(ctypes.Structure):
    _fields_ = [("max_depth", ctypes.c_int),
                ("n_theta", ctypes.c_int * (PO_MAX_DEPTH + 1)),
                ("n_phi", ctypes.c_int * (PO_MAX_DEPTH + 1)),
                ("box_min", ctypes.c_float * 3), ("box_max", ctypes.c_float * 3),
                ("precision", ctypes.c_int), ("theta_mode", ctypes.c_int), ("nyquist_quirk", ctypes.c_int),
                ("distance", ctypes.c_double), ("interp_method", ctypes.c_int),
                ("max_workspace_bytes", ctypes.c_int64), ("interp_tile", ctypes.c_int),
                ("leaf_kernel", ctypes.c_int), ("leaf_slots", ctypes.c_int)]


class po_geometry(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64),
                ("x", ctypes.c_void_p), ("y", ctypes.c_void_p), ("z", ctypes.c_void_p),
                ("nx", ctypes.c_void_p), ("ny", ctypes.c_void_p), ("nz", ctypes.c_void_p),
                ("area", ctypes.c_void_p), ("on_device", ctypes.c_int)]


class po_illum(ctypes.Structure):
    _fields_ = [("n_lambda", ctypes.c_int), ("lambda_m", ctypes.c_void_p),
                ("n_inc", ctypes.c_int), ("theta_i", ctypes.c_void_p), ("phi_i", ctypes.c_void_p),
                ("pol_mask", ctypes.c_int), ("eta_re", ctypes.c_double), ("eta_im", ctypes.c_double),
                ("sigma", ctypes.c_double)]


class po_batch_item(ctypes.Structure):
    _fields_ = [("geom", po_geometry), ("illum", po_illum), ("intensity", ctypes.c_void_p)]


class po_report(ctypes.Structure):
    _fields_ = [("ms_total", ctypes.c_double), ("ms_build", ctypes.c_double), ("ms_leaf", ctypes.c_double),
                ("ms_aggregate", ctypes.c_double), ("ms_intensity", ctypes.c_double),
                ("n_leaves", ctypes.c_int64), ("n_nodes_total", ctypes.c_int64),
                ("root_theta", ctypes.c_int), ("root_phi", ctypes.c_int),
                ("workspace_bytes", ctypes.c_int64), ("kernel_launches", ctypes.c_int64),
                ("ms_leaf_kernel", ctypes.c_double), ("ms_rows", ctypes.c_double), ("ms_cols", ctypes.c_double),
                ("n_leaf_launches", ctypes.c_int), ("n_row_launches", ctypes.c_int), ("n_col_launches", ctypes.c_int),
                ("n_chunks", ctypes.c_int), ("chunk_slots", ctypes.c_int),
                ("leaf_point_dirs", ctypes.c_double), ("rows_bytes", ctypes.c_double), ("cols_bytes", ctypes.c_double),
                ("ms_rows_level", ctypes.c_double * PO_MAX_DEPTH), ("ms_cols_level", ctypes.c_double * PO_MAX_DEPTH),
                ("agg_bytes", ctypes.c_double), ("n_nodes_level", ctypes.c_int64 * (PO_MAX_DEPTH + 1))]

    def as_dict(self):
        d = {f: getattr(self, f) for f, _ in self._fields_}
        for k in ("ms_rows_level", "ms_cols_level", "n_nodes_level"):
            d[k] = list(d[k])
        return d


EXPORTS = ("po_config_init", "po_status_string", "po_last_error", "po_create", "po_destroy", "po_solve",
           "po_tangent_plane_currents", "po_build_octree", "po_far_field_direct", "po_interp_fft",
           "po_compute_intensity", "po_version", "po_interp_fft_noalloc", "po_height_field_points",
           "po_average_pattern", "po_grad", "po_height_field_adjoint", "po_batch_create", "po_batch_prepare",
           "po_batch_launch", "po_batch_info", "po_batch_destroy", "po_shifted_fft2", "po_acf_from_patterns",
           "po_check", "po_batch_check", "po_selftest_device_waits")

_lib = None


def load():
    """Loads libwavepo.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                          "or `python wavefiber3d_gb300/build.py`")
    L = ctypes.CDLL(str(LIB_PATH))
    vp, i64, i32, dbl, st = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_double, ctypes.c_int
    L.po_config_init.argtypes = [ctypes.POINTER(po_config), i32, i32, i32, vp, vp, dbl, dbl, dbl, dbl, dbl]
    L.po_status_string.argtypes = [st]
    L.po_status_string.restype = ctypes.c_char_p
    L.po_last_error.restype = ctypes.c_char_p
    L.po_version.restype = ctypes.c_char_p
    L.po_create.argtypes = [ctypes.POINTER(vp), ctypes.POINTER(po_config)]
    L.po_destroy.argtypes = [vp]
    L.po_solve.argtypes = [vp, ctypes.POINTER(po_geometry), ctypes.POINTER(po_illum), vp, i32, vp,
                           ctypes.POINTER(po_report)]
    L.po_tangent_plane_currents.argtypes = [i64] + [vp] * 7 + [dbl, dbl, dbl, i32, dbl, dbl, dbl, dbl, i32, vp, vp]
    L.po_build_octree.argtypes = [i64, vp, vp, vp, vp, vp, i32, vp, vp, vp]
    L.po_far_field_direct.argtypes = [i64, vp, vp, vp, vp, dbl, vp, i32, i32, i32, vp, vp]
    L.po_interp_fft.argtypes = [vp, i32, i32, vp, i32, i32, i32, i32, i32, vp]
    L.po_interp_fft_noalloc.argtypes = [vp, i32, i32, vp, i32, i32, i32, i32, i32, vp]
    L.po_compute_intensity.argtypes = [vp, i32, i32, vp, vp]
    L.po_grad.argtypes = [vp, ctypes.POINTER(po_geometry), ctypes.POINTER(po_illum), vp, vp, vp, vp,
                          ctypes.POINTER(po_report)]
    L.po_height_field_adjoint.argtypes = [vp, i32, i32, ctypes.c_float, ctypes.c_float, i32, i32, vp, vp, vp]
    L.po_batch_create.argtypes = [ctypes.POINTER(vp), i32, ctypes.POINTER(po_config), i32]
    L.po_batch_prepare.argtypes = [vp, ctypes.POINTER(po_batch_item), vp]
    L.po_batch_launch.argtypes = [vp, vp]
    L.po_batch_info.argtypes = [vp, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                                ctypes.POINTER(ctypes.c_double)]
    L.po_batch_destroy.argtypes = [vp]
    L.po_check.argtypes = [vp, vp]
    L.po_batch_check.argtypes = [vp, vp]
    L.po_selftest_device_waits.argtypes = [i32, vp]
    L.po_shifted_fft2.argtypes = [vp, vp, i32, i32, i32, i32, vp]
    L.po_acf_from_patterns.argtypes = [vp, i32, i32, i32, vp, vp, vp, vp]
    L.po_average_pattern.argtypes = [vp, i32, i32, vp, i32, i32, i32, vp]
    L.po_height_field_points.argtypes = [vp, i32, i32, ctypes.c_float, ctypes.c_float, i32, i32] + [vp] * 8
    for name in EXPORTS:
        f = getattr(L, name)
        if name not in ("po_status_string", "po_last_error", "po_version"):
            f.restype = ctypes.c_int
    _lib = L
    return L


def check(status: int):
    if status != PO_OK:
        raise WavePOError(status, load().po_last_error().decode())
