"""The drop-in drivers on a GPU: their output files equal the library's own
solve of the same workload (same presets, grids and illumination) bit for
bit, and keep the reference's file names and raw float32 layout."""
import math
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from wavefiber3d_gb300 import api, build, geometry  # noqa: E402


@pytest.fixture(scope="module")
def clis():
    build.build()
    return {p.name: p for p in build.build_cli()}


def run(exe, args, cwd):
    r = subprocess.run([str(exe), *map(str, args)], cwd=cwd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return r


def ref_lambda(i):
    return float(np.float32(np.float32(400.0 + np.float32(300.0) / np.float32(25) * i) * np.float32(1e-9)))


def test_sphere_driver(clis, tmp_path):
    (tmp_path / "mesh").mkdir()
    cloud = geometry.fibonacci_sphere(10e-6, 20000)
    geometry.write_reference_mesh(cloud, tmp_path / "mesh" / "sphere10um")
    run(clis["wavepo_sphere"], [3, 5, 2, "--theta-mode", "reference"], tmp_path)
    box = [-11e-6] * 3, [11e-6] * 3
    cfg = api.Config.reference_rule(2, 900, 1440, *box, 20e-6, 20e-6, 1.3, theta_mode=api.PO_THETA_REFERENCE)
    il = api.Illumination([ref_lambda(3), ref_lambda(4)], [0.0], [0.0], api.PO_POL_TM | api.PO_POL_TE, 1.55, 1e-2)
    with api.Solver(cfg) as s:
        want = s.solve(cloud, il)
    for li, lam in enumerate((3, 4)):
        for pi, mode in enumerate("ME"):
            f = tmp_path / "output" / f"sphere_10um_lambda{lam}_T{mode}_depth2.binary"
            got = np.fromfile(f, dtype=np.float32)
            assert got.size == 900 * 1440
            assert np.array_equal(got, want[li, 0, pi].ravel())


def test_ellipsoid_drivers(clis, tmp_path):
    (tmp_path / "mesh" / "PO").mkdir(parents=True)
    cloud = geometry.PointCloud.load(GOLDEN / "geom_ellipsoid_n3000.bin")
    geometry.write_reference_mesh(cloud, tmp_path / "mesh" / "PO" / "ellipsoid_3_3_2")
    run(clis["wavepo_ellipsoid"], [1], tmp_path)
    box = [-10e-6, -10e-6, -5e-6], [10e-6, 10e-6, 5e-6]
    cfg = api.Config.reference_rule(1, 900, 1440, *box, 10e-6, 20e-6, 3.0)
    il = api.Illumination([float(np.float32(500.0) * np.float32(1e-9))], [0.0], [0.0],
                          api.PO_POL_TM | api.PO_POL_TE, 1.55 + 0.3j, 1e-2)
    with api.Solver(cfg) as s:
        want = s.solve(cloud, il)
    for pi, mode in enumerate("ME"):
        got = np.fromfile(tmp_path / "output" / f"ellipsoid_lambda0_T{mode}_depth1_kappa0.3.binary", np.float32)
        assert np.array_equal(got, want[0, 0, pi].ravel())
    run(clis["wavepo_ellipsoid_simple"], [], tmp_path)
    ring = np.fromfile(tmp_path / "output" / "ellipsoid_TM_kappa0.3.binary", dtype=np.float64)
    cfg0 = api.Config(0, [2], [3600], *box, precision=api.PO_PREC_FP64)
    with api.Solver(cfg0) as s:
        w0 = s.solve(cloud, api.Illumination([500e-9], [0.0], [0.0], api.PO_POL_TM, 1.55 + 0.3j, 1e-2))
    assert ring.size == 3600 and np.array_equal(ring, w0[0, 0, 0, 1].astype(np.float64))


def test_treepo_driver(clis, tmp_path):
    """fibersim/treePO.cu preset 0 (20 um circular fiber, period 20 um,
    3000 x 478 vertices, 450 x 880 output) on half a ring."""
    (tmp_path / "mesh").mkdir()
    numel, numelvert, period = 3000, 478, 20e-6
    phi = 2 * np.pi * np.arange(numel) / numel
    rng = np.random.default_rng(4)
    r = 20e-6 + 0.02e-6 * rng.standard_normal((numel, numelvert))
    xy = np.stack([r * np.cos(phi)[:, None], r * np.sin(phi)[:, None]]).astype(np.float32)
    xy.tofile(tmp_path / "mesh" / "fiber0.binary")
    run(clis["wavepo_treepo"], [2, 4, 90, 0, 0, 3, 700, 2300], tmp_path)
    hf = geometry.HeightField.load(tmp_path / "mesh" / "fiber0.binary", numel, numelvert, period)
    g = api.height_field_points(hf, 700, 2300)
    bmin = [-22e-6, -22e-6, float(np.float32(-period * 0.5) * np.float32(1.1))]
    bmax = [22e-6, 22e-6, -bmin[2]]
    bmin[:2] = [float(np.float32(-20e-6) * np.float32(1.1))] * 2
    bmax[:2] = [-bmin[0]] * 2
    cfg = api.Config.reference_rule(3, 450, 880, bmin, bmax, period, 40e-6, 1.2)
    ti = float(np.float32(-math.pi / 2 + float(np.float32(1e-10)) + math.pi / 180 * 90))
    il = api.Illumination([ref_lambda(2), ref_lambda(3)], [ti], [0.0], api.PO_POL_TM, 1.55, 10e-6)
    with api.Solver(cfg) as s:
        want = s.solve(tuple(g[k] for k in range(7)), il).cpu().numpy()
    for li, lam in enumerate((2, 3)):
        got = np.fromfile(tmp_path / "output" / f"fiber_0_lambda{lam}_TM_depth3.binary", dtype=np.float32)
        assert got.size == 450 * 880
        assert np.array_equal(got, want[li, 0, 0].ravel())
