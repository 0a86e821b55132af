"""The C-ABI library without a GPU: it loads, exports every entry point that
include/wavepo.h declares, and its host-only logic (grid rule, argument
checks, status strings) behaves as documented."""
import ctypes
import re
from pathlib import Path

import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def lib():
    from wavefiber3d_gb300 import _lib, build
    if not _lib.LIB_PATH.exists():
        build.build()
    return _lib.load()


def declared_functions():
    text = (ROOT / "include" / "wavepo.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(po_[a-z_0-9]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert "po_solve" in names and len(names) >= 12
    for n in names:
        assert hasattr(lib, n), n


def test_library_is_built_for_sm103a():
    from wavefiber3d_gb300 import build
    assert "arch=compute_103a,code=sm_103a" in " ".join(build.ARCH)


def test_config_rule_matches_reference_numbers(lib):
    """Level grids of the reference rule (compareMie/sphere.cu:345-352) for the
    ellipsoid workload (extent 16 um, ratio 1.3) and the fiber segment
    (fibersim/treePO.cu:353-359, theta 60 um, phi 50 um, ratio 1.2)."""
    from wavefiber3d_gb300 import _lib, grids
    c = _lib.po_config()
    b0, b1 = (ctypes.c_float * 3)(-1, -1, -1), (ctypes.c_float * 3)(1, 1, 1)
    assert lib.po_config_init(ctypes.byref(c), 5, 180, 360, b0, b1, 16e-6, 16e-6, 1.3, 6.0, 0.4e-6) == 0
    assert list(c.n_theta[:6]) == [180, 197, 108, 62, 37, 24]
    assert list(c.n_phi[:6]) == [360, 197, 108, 62, 37, 24]
    assert lib.po_config_init(ctypes.byref(c), 7, 180, 360, b0, b1, 60e-6, 50e-6, 1.2, 6.0, 0.4e-6) == 0
    assert list(c.n_theta[1:8]) == [616, 323, 173, 96, 56, 34, 22]
    assert list(c.n_phi[1:8]) == [518, 273, 148, 83, 48, 30, 20]
    py = grids.level_grids(180, 360, 7, 60e-6, 50e-6, 1.2)
    assert py[0] == list(c.n_theta[:8]) and py[1] == list(c.n_phi[:8])
    assert c.theta_mode == 0 and c.precision == 0 and c.interp_method == 1 and c.distance == 1.0


def test_invalid_configurations_fail_before_touching_cuda(lib):
    from wavefiber3d_gb300 import _lib
    c = _lib.po_config()
    b0, b1 = (ctypes.c_float * 3)(-1, -1, -1), (ctypes.c_float * 3)(1, 1, 1)
    assert lib.po_config_init(ctypes.byref(c), 11, 180, 360, b0, b1, 1e-6, 1e-6, 1.3, 6.0, 0.4e-6) == 1
    assert lib.po_config_init(None, 1, 180, 360, b0, b1, 1e-6, 1e-6, 1.3, 6.0, 0.4e-6) == 1
    lib.po_config_init(ctypes.byref(c), 2, 16, 32, b0, b1, 1e-6, 1e-6, 1.3, 6.0, 0.4e-6)
    c.n_theta[2] = 999  # a child grid finer than its parent
    h = ctypes.c_void_p()
    assert lib.po_create(ctypes.byref(h), ctypes.byref(c)) == 1
    assert b"grow" in lib.po_last_error()
    lib.po_config_init(ctypes.byref(c), 2, 16, 32, b0, b1, 1e-6, 1e-6, 1.3, 6.0, 0.4e-6)
    c.box_max[0] = c.box_min[0]
    assert lib.po_create(ctypes.byref(h), ctypes.byref(c)) == 1
    lib.po_config_init(ctypes.byref(c), 2, 16, 32, b0, b1, 1e-6, 1e-6, 1.3, 6.0, 0.4e-6)
    c.precision = 1  # FP64 is the depth-0 plain sum only
    assert lib.po_create(ctypes.byref(h), ctypes.byref(c)) == 4
    # leaf schedule: a known kernel, for split-BF16 trees only; whole groups of 8 patterns up to 64
    for prec, kern, slots in ((2, 3, 0), (0, 2, 0), (2, 0, 12), (2, 2, 72), (2, 1, -8)):
        lib.po_config_init(ctypes.byref(c), 2, 16, 32, b0, b1, 1e-6, 1e-6, 1.3, 6.0, 0.4e-6)
        c.precision, c.leaf_kernel, c.leaf_slots = prec, kern, slots
        assert lib.po_create(ctypes.byref(h), ctypes.byref(c)) == 1, (prec, kern, slots)
        assert b"leaf" in lib.po_last_error()
    for s in range(7):
        assert lib.po_status_string(s)
    assert b"sm_103a" in lib.po_version()


def test_single_step_argument_checks(lib):
    # null pointers / negative sizes are rejected before any CUDA call
    assert lib.po_interp_fft(None, 4, 4, None, 8, 8, 1, 1, 1, None) == 1
    assert lib.po_interp_fft_noalloc(None, 4, 4, None, 8, 8, 1, 1, 1, None) == 1
    assert lib.po_build_octree(-1, None, None, None, None, None, 2, None, None, None) == 1
    assert lib.po_tangent_plane_currents(-5, *([None] * 7), 5e-7, 0.0, 0.0, 1, 1.55, 0.0, 1e-2, 1.0, 1, None,
                                         None) == 1
    # height field: null arrays, empty grids and bad ring segments
    fake = ctypes.c_void_p(16)
    assert lib.po_height_field_points(None, 8, 4, 1e-6, 2.5e-7, 0, 7, *([fake] * 7), None) == 1
    assert lib.po_height_field_points(fake, 1, 4, 1e-6, 2.5e-7, 0, 0, *([fake] * 7), None) == 1
    assert lib.po_height_field_points(fake, 8, 0, 1e-6, 2.5e-7, 0, 7, *([fake] * 7), None) == 1
    assert lib.po_height_field_points(fake, 8, 4, 1e-6, 2.5e-7, 5, 4, *([fake] * 7), None) == 1
    assert lib.po_height_field_points(fake, 8, 4, 1e-6, 2.5e-7, 0, 8, *([fake] * 7), None) == 1
    assert lib.po_height_field_points(fake, 8, 4, 1e-6, 0.0, 0, 7, *([fake] * 7), None) == 1
    # pattern statistics: null arrays and bad sizes
    assert lib.po_shifted_fft2(None, fake, 1, 8, 8, 0, None) == 1
    assert lib.po_shifted_fft2(fake, fake, 1, 0, 8, 0, None) == 1
    assert lib.po_shifted_fft2(fake, fake, -1, 8, 8, 0, None) == 1
    assert lib.po_shifted_fft2(fake, fake, 1, 8, 8, 2, None) == 1
    assert lib.po_acf_from_patterns(fake, 0, 8, 8, fake, fake, fake, None) == 1
    assert lib.po_acf_from_patterns(fake, 4, 8, 8, None, fake, fake, None) == 1
