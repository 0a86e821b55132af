"""Parity at the sizes of the benchmark workloads, against the FP64 oracle.

  * the plain method (depth 0): sphere of radius 2 um, 20,000 Fibonacci
    points, n = 1.55, 500 nm, plane wave along +z polarised along x, on the
    full 180 x 360 grid -- FP64 engine <= 1e-6, FP32 engine <= 1e-5,
    split-BF16 tcgen05 engine <= 1e-4 over all 64,800 directions; the
    engine's forward lobe against the Mie series;
  * the fiber segment (3.40M points from the seeded height field, depth 7,
    reference level grids, 180 x 360, split-BF16 tcgen05 leaf sums): eight
    incidences of the 64-incidence sweep at 400 nm, two of them against the
    FP64 oracle on 512 seeded directions <= 1e-3;
  * a batch of independent solves in one CUDA graph: every item against the
    FP64 oracle on 64 seeded directions <= 1e-3.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import oracle  # noqa: E402
from oracle import mie  # noqa: E402
from wavefiber3d_gb300 import api, geometry  # noqa: E402

NTH, NPH = 180, 360


def rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


# ------------------------------------------------------------ plain method
@pytest.fixture(scope="module")
def sphere20k():
    cloud = geometry.fibonacci_sphere(2e-6, 20000)
    # +z incidence, E along x: theta_i = pi/2, phi_i = pi, mode M (sphere.cu:559-579)
    il_o = oracle.make_illum(500e-9, math.pi / 2, math.pi, "M", 1.55, 1e-2)
    ref = oracle.solve_direct(cloud, il_o, NTH, NPH)
    return cloud, ref


@pytest.mark.parametrize("prec,tol", [(api.PO_PREC_FP64, 1e-6), (api.PO_PREC_FP32, 1e-5)])
def test_sphere_20k_depth0_full_grid(sphere20k, prec, tol):
    cloud, ref = sphere20k
    cfg = api.Config(0, [NTH], [NPH], [-2.2e-6] * 3, [2.2e-6] * 3, precision=prec)
    il = api.Illumination([500e-9], [math.pi / 2], [math.pi], api.PO_POL_TM, 1.55 + 0j, 1e-2)
    with api.Solver(cfg) as s:
        out = s.solve(cloud, il).reshape(NTH, NPH)
    assert rel(out, ref) <= tol


def test_sphere_20k_depth0_tensor_core_full_grid(sphere20k):
    """Config 1 on the tensor cores: the split-BF16 tcgen05 sum over one leaf of
    all 20,000 points (its 507 direction tiles spread over CTAs) against the
    FP64 oracle on all 64,800 directions; and with 70 patterns (two slot
    groups) every pattern against the FP32 direct sum."""
    cloud, ref = sphere20k
    box = [-2.2e-6] * 3, [2.2e-6] * 3
    il = api.Illumination([500e-9], [math.pi / 2], [math.pi], api.PO_POL_TM, 1.55 + 0j, 1e-2)
    with api.Solver(api.Config(0, [NTH], [NPH], *box, precision=api.PO_PREC_SPLIT_BF16)) as s:
        out = s.solve(cloud, il).reshape(NTH, NPH)
        assert s.last_report["n_leaf_launches"] == 2, s.last_report  # operands + sums: the tcgen05 path
    assert rel(out, ref) <= 1e-4
    rng = np.random.default_rng(12)
    th, ph = list(rng.uniform(-1.3, 1.3, 35)), list(rng.uniform(0, 2 * math.pi, 35))
    il70 = api.Illumination([620e-9], th, ph, api.PO_POL_TM | api.PO_POL_TE, 1.55 + 0.1j, 1e-2)
    outs = []
    for prec in (api.PO_PREC_FP32, api.PO_PREC_SPLIT_BF16):
        with api.Solver(api.Config(0, [90], [180], *box, precision=prec)) as s:
            outs.append(s.solve(cloud, il70))
    assert rel(outs[1], outs[0]) <= 1e-4


def test_sphere_20k_forward_lobe_vs_mie(sphere20k):
    """Scattering angles 1-10 degrees along the phi = 0 meridian (the plane of
    E and k), normalised at 1 degree: the engine's PO diffraction lobe follows
    the Mie series (PO neglects the transmitted light, so only the lobe's
    shape is compared, as compareMie/mie.ipynb does)."""
    cloud, _ = sphere20k
    cfg = api.Config(0, [NTH], [NPH], [-2.2e-6] * 3, [2.2e-6] * 3, precision=api.PO_PREC_FP32)
    il = api.Illumination([500e-9], [math.pi / 2], [math.pi], api.PO_POL_TM, 1.55 + 0j, 1e-2)
    with api.Solver(cfg) as s:
        out = s.solve(cloud, il).reshape(NTH, NPH).astype(np.float64)
    rows = np.arange(NTH - 1, NTH - 11, -1)  # elevation 89 .. 80 degrees = scattering angle 1 .. 10
    th = -math.pi / 2 + 1e-10 + math.pi / NTH * rows
    sdir = np.stack([np.cos(th), np.zeros_like(th), np.sin(th)], 1)
    mi = mie.polarised_intensity(2e-6, 500e-9, 1.55, [0, 0, 1], [1, 0, 0], sdir)
    po = out[rows, 0]
    assert rel(po / po[0], mi / mi[0]) < 0.1


# --------------------------------------------------------------- fiber segment
def test_fiber_segment_vs_fp64_oracle():
    import bench
    hf = geometry.fiber_height_field(bench.FIBER_RADII, bench.FIBER_LENGTH, seed=bench.FIBER_SEED)
    g = api.height_field_points(hf)
    th, ph = bench.fiber_incidences()
    sel = list(range(0, 64, 8))  # 8 incidences of the sweep: the tcgen05 leaf path
    il = api.Illumination([400e-9], [th[i] for i in sel], [ph[i] for i in sel], api.PO_POL_TM, bench.ETA,
                          bench.FIBER_SIGMA)
    with api.Solver(bench.fiber_config("split_bf16")) as s:
        out = s.solve(tuple(g[k] for k in range(7)), il)
        rep = s.last_report
    assert rep["n_leaves"] > 50000 and rep["n_leaf_launches"] == 2, rep
    cloud = geometry.PointCloud.from_soa(g.cpu().numpy())
    dirs = np.sort(np.random.default_rng(20231203).choice(NTH * NPH, 512, replace=False))
    ctr = [0.5 * (a + b) for a, b in zip(np.float32(bench.FIBER_BOX_MIN), np.float32(bench.FIBER_BOX_MAX))]
    for j in (0, len(sel) - 1):
        il_o = oracle.make_illum(400e-9, th[sel[j]], ph[sel[j]], "M", bench.ETA, bench.FIBER_SIGMA)
        cur = oracle.currents(cloud, il_o)
        f = oracle.far_field_sampled(cloud, cur, 2 * math.pi / 400e-9, ctr, NTH, NPH, dirs)
        ref = oracle.intensity_sampled(f, NTH, NPH, dirs)
        got = out[0, j, 0].reshape(-1).cpu().numpy()[dirs]
        assert rel(got, ref) <= 1e-3, j


# ------------------------------------------------------------------- batch
def test_batch_items_vs_fp64_oracle():
    """Spheres and ellipsoids of 5k-60k points, depths 0-4, FP32 and
    split-BF16 leaves, one or eight incidences, captured in one graph."""
    rng = np.random.default_rng(21)
    its = []
    for i in range(8):
        r = float(rng.uniform(1e-6, 4e-6))
        n = int(round(math.exp(rng.uniform(math.log(5e3), math.log(6e4)))))
        cloud = geometry.fibonacci_sphere(r, n) if i % 2 == 0 else geometry.ellipsoid((r, 0.7 * r, 0.55 * r), n)
        depth = i % 5
        prec = api.PO_PREC_SPLIT_BF16 if (i % 3 and depth > 0) else api.PO_PREC_FP32
        n_inc = 8 if i in (3, 6) else 1
        lam = float(rng.uniform(400e-9, 700e-9))
        th = list(rng.uniform(-1.3, 1.3, n_inc))
        ph = list(rng.uniform(0, 2 * math.pi, n_inc))
        cfg = api.Config.reference_rule(depth, 90, 180, [-1.1 * r] * 3, [1.1 * r] * 3, 2 * r, 2 * r, 1.3,
                                        precision=prec)
        il = api.Illumination([lam], th, ph, api.PO_POL_TM, 1.55 + 0.1j, 1.0)
        its.append((cloud, torch.from_numpy(cloud.soa()).cuda(), cfg, il))
    with api.Batch([c for _, _, c, _ in its], n_streams=4) as b:
        b.prepare([g for _, g, _, _ in its], [il for _, _, _, il in its])
        outs = b.launch()
        torch.cuda.synchronize()
        dirs = np.sort(np.random.default_rng(7).choice(90 * 180, 64, replace=False))
        for (cloud, _, cfg, il), o in zip(its, outs):
            o = o.cpu().numpy().reshape(len(il.theta_i), -1)
            for j in sorted({0, len(il.theta_i) - 1}):
                il_o = oracle.make_illum(il.wavelengths_m[0], il.theta_i[j], il.phi_i[j], "M", 1.55 + 0.1j, 1.0)
                ref = oracle.solve_sampled_f64(cloud.soa().astype(np.float64), il_o, 90, 180, dirs)
                assert rel(o[j][dirs], ref) <= 1e-3, (cfg.max_depth, cfg.precision, j)
