"""GPU parity of every step of the PO path against the FP64 oracle and the
reference's own CUDA outputs (tests/golden/ref_*.bin).

Tolerances (relative L2 over the whole output):
  currents, direct sums, intensity, interpolation : 1e-5 (FP32 engine vs FP64)
  octree                                           : bit-exact
  tree solve vs FP64 direct sum (double cover)     : 1e-4
  tree solve, reference theta mode vs oracle tree  : 1e-4
  anything vs the reference's FP32 CUDA build      : 1e-4
"""
import dataclasses
import math

import numpy as np
import pytest

from conftest import GOLDEN, case_illum, load_case_geometry

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import oracle  # noqa: E402
from wavefiber3d_gb300 import api, geometry  # noqa: E402

TOL_FP32 = 1e-5
TOL_TREE = 1e-4


def rel(a, b):
    a = np.asarray(a, dtype=np.complex128 if np.iscomplexobj(a) else np.float64)
    b = np.asarray(b, dtype=np.complex128 if np.iscomplexobj(b) else np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def ref_fixture(name, dtype=np.float32):
    p = GOLDEN / f"{name}.bin"
    if not p.exists():
        pytest.fail(f"golden fixture {p.name} missing")
    return np.fromfile(p, dtype=dtype)


def illum_of(case):
    il = case["illum"]
    pol = api.PO_POL_TE if il["mode"] == "E" else api.PO_POL_TM
    return api.Illumination([il["lambda_m"]], [il["theta_i"]], [il["phi_i"]], pol, complex(*il["eta"]), il["sigma"])


def cur_gpu(cloud, il, scale):
    return api.compute_local_tangent_plane(cloud.x, cloud.y, cloud.z, cloud.nx, cloud.ny, cloud.nz, cloud.area,
                                           il.lambda_m, il.theta_i, il.phi_i, "E" if il.mode_te else "M",
                                           complex(il.eta_re, il.eta_im), il.sigma, 1.0, scale).cpu().numpy()


# ------------------------------------------------------------------ currents
@pytest.mark.parametrize("name", ["ref_currents_sphere_M", "ref_currents_ellipsoid_E"])
@pytest.mark.parametrize("scale", [False, True])
def test_currents_vs_oracle(cases, name, scale):
    c = cases[name]
    cloud, il = load_case_geometry(c), case_illum(c)
    g = cur_gpu(cloud, il, scale)
    o = oracle.currents(cloud, il, scale=scale)
    assert rel(g, o) < TOL_FP32
    # shadowed points carry no current (tangentplane.h:64-67)
    lit = np.abs(o).sum(1) > 0
    assert np.all(np.abs(g[~lit]) == 0)


@pytest.mark.parametrize("name", ["ref_currents_sphere_M", "ref_currents_ellipsoid_E"])
def test_currents_vs_reference_build(cases, name):
    c = cases[name]
    cloud, il = load_case_geometry(c), case_illum(c)
    g = cur_gpu(cloud, il, False)
    r = ref_fixture(name).reshape(-1, 12).astype(np.float64).view(np.complex128)
    assert rel(g, r) < TOL_FP32


# ------------------------------------------------------------------- octree
def _octree_case(cloud, box, depth):
    perm, hr = api.build_octree(cloud.x, cloud.y, cloud.z, box[:3], box[3:], depth)
    operm, orng, _ = oracle.octree(cloud, box[:3], box[3:], depth)
    assert np.array_equal(perm.cpu().numpy(), operm)
    assert np.array_equal(hr.cpu().numpy(), orng)


@pytest.mark.parametrize("depth", [0, 1, 3, 5])
def test_octree_vs_oracle(cases, depth):
    c = cases["ref_octree_ellipsoid_d3"]
    _octree_case(load_case_geometry(c), c["box"], depth)


def test_octree_boundary_points():
    # points exactly on the float split planes and outside the root box
    rng = np.random.default_rng(7)
    box = [-1.0, -1.0, -1.0, 1.0, 1.0, 1.0]
    pts = rng.choice(np.array([-1.0, -0.5, -0.25, 0.0, 0.25, 0.5, 0.999, 1.0, 1.5, -1.5], np.float32), size=(3, 4000))
    z = np.zeros(4000, np.float32)
    cloud = geometry.PointCloud(pts[0], pts[1], pts[2], z, z, z + 1, z + 1)
    for depth in (1, 2, 4):
        _octree_case(cloud, box, depth)


def test_octree_vs_reference_build(cases):
    c = cases["ref_octree_ellipsoid_d3"]
    cloud = load_case_geometry(c)
    n, d = cloud.n, c["depth"]
    raw = ref_fixture(c["name"], np.uint8)
    geo = np.frombuffer(raw[: 28 * n].tobytes(), dtype=np.float32).reshape(7, n)
    rng = np.frombuffer(raw[28 * n:].tobytes(), dtype=np.int32).reshape(-1, 2)
    perm, hr = api.build_octree(cloud.x, cloud.y, cloud.z, c["box"][:3], c["box"][3:], d)
    perm = perm.cpu().numpy()
    assert np.array_equal(cloud.soa()[:, perm], geo)
    assert np.array_equal(hr.cpu().numpy(), rng)


# ------------------------------------------------------------ interpolation
@pytest.mark.parametrize("src,dst,quirk", [((20, 30), (33, 300), True), ((20, 30), (33, 300), False),
                                           ((21, 25), (40, 64), True), ((16, 16), (16, 16), True),
                                           ((37, 37), (48, 96), True), ((24, 50), (394, 197), False),
                                           ((7, 11), (13, 1440), True)])
def test_interp_vs_oracle(src, dst, quirk):
    rng = np.random.default_rng(src[0] * 1000 + dst[1])
    z = (rng.standard_normal(src) + 1j * rng.standard_normal(src)).astype(np.complex64)
    g = api.copyandinterp(torch.from_numpy(z), dst[0], dst[1], api.PO_THETA_REFERENCE, quirk).cpu().numpy()
    o = oracle.interp(z.astype(np.complex128), dst[0], dst[1], quirk)
    assert rel(g, o) < TOL_FP32


def test_interp_batched_matches_single():
    rng = np.random.default_rng(3)
    z = (rng.standard_normal((5, 12, 18)) + 1j * rng.standard_normal((5, 12, 18))).astype(np.complex64)
    b = api.copyandinterp(torch.from_numpy(z), 30, 40).cpu().numpy()
    for i in range(5):
        s = api.copyandinterp(torch.from_numpy(z[i]), 30, 40).cpu().numpy()
        assert np.array_equal(b[i], s)


@pytest.mark.parametrize("name", ["ref_interp_even", "ref_interp_odd"])
def test_interp_vs_reference_build(cases, name):
    c = cases[name]
    z = np.fromfile(GOLDEN / c["input"], dtype=np.complex64).reshape(c["src"])
    g = api.copyandinterp(torch.from_numpy(z), *c["dst"], api.PO_THETA_REFERENCE, True).cpu().numpy()
    r = ref_fixture(name).view(np.complex64).reshape(c["dst"])
    assert rel(g, r) < TOL_FP32


# ------------------------------------------------------ direct sum, intensity
@pytest.mark.parametrize("prec,tol", [(api.PO_PREC_FP32, TOL_FP32), (api.PO_PREC_FP64, 1e-6)])
def test_direct_sum_vs_oracle(cases, prec, tol):
    c = cases["ref_currents_ellipsoid_E"]
    cloud, il = load_case_geometry(c), case_illum(c)
    cur = oracle.currents(cloud, il, scale=True)
    k = 2 * math.pi / il.lambda_m
    ctr = (0.1e-6, -0.2e-6, 0.05e-6)
    g = api.current_times_green_center(cloud.x, cloud.y, cloud.z, torch.from_numpy(cur.astype(np.complex64)), k, ctr,
                                       24, 48, prec).cpu().numpy()
    o = oracle.far_field(cloud, cur, k, ctr, 24, 48)  # [dir][6]
    assert rel(g.reshape(6, -1).T, o) < tol


def test_intensity_vs_oracle():
    rng = np.random.default_rng(11)
    f = (rng.standard_normal((6, 20, 36)) + 1j * rng.standard_normal((6, 20, 36))) * 1e-6
    g = api.compute_intensity(torch.from_numpy(f.astype(np.complex64))).cpu().numpy()
    o = oracle.intensity(f.reshape(6, -1).T.copy(), 20, 36)
    assert rel(g, o) < TOL_FP32


# ---------------------------------------------------------------- full solve
def _solve(cloud, cfg, illum, device_io=False):
    with api.Solver(cfg) as s:
        if device_io:
            g = torch.from_numpy(cloud.soa()).cuda()
            out = s.solve(tuple(g[k] for k in range(7)), illum).cpu().numpy()
        else:
            out = s.solve(cloud, illum)
        return out, s.last_report


@pytest.mark.parametrize("prec,tol", [(api.PO_PREC_FP32, TOL_FP32), (api.PO_PREC_FP64, 1e-6)])
def test_solve_depth0_vs_oracle(cases, prec, tol):
    c = cases["ref_solve_sphere_d0"]
    cloud, il = load_case_geometry(c), case_illum(c)
    cfg = api.Config(0, [48], [96], c["box"][:3], c["box"][3:], precision=prec)
    out, _ = _solve(cloud, cfg, illum_of(c))
    o = oracle.solve_direct(cloud, il, 48, 96)
    assert rel(out.reshape(48, 96), o) < tol


@pytest.mark.parametrize("name", ["ref_solve_sphere_d3", "ref_solve_ellipsoid_d2", "ref_solve_sphere_quirk_d1"])
def test_solve_tree_vs_fp64_direct(cases, name):
    c = cases[name]
    cloud, il = load_case_geometry(c), case_illum(c)
    cfg = api.Config(c["depth"], c["n_theta"], c["n_phi"], c["box"][:3], c["box"][3:])
    out, rep = _solve(cloud, cfg, illum_of(c), device_io=True)
    ctr = [(c["box"][i] + c["box"][i + 3]) / 2 for i in range(3)]
    o = oracle.solve_direct(cloud, il, c["n_theta"][0], c["n_phi"][0], center=ctr)
    assert rel(out.reshape(o.shape), o) < TOL_TREE, rep


@pytest.mark.parametrize("interp", [api.PO_INTERP_TENSOR, api.PO_INTERP_FFT])
@pytest.mark.parametrize("name", ["ref_solve_sphere_d3", "ref_solve_ellipsoid_d2", "ref_solve_sphere_quirk_d1"])
def test_solve_reference_mode_vs_oracle_tree(cases, name, interp):
    c = cases[name]
    cloud, il = load_case_geometry(c), case_illum(c)
    cfg = api.Config(c["depth"], c["n_theta"], c["n_phi"], c["box"][:3], c["box"][3:],
                     theta_mode=api.PO_THETA_REFERENCE, nyquist_quirk=True, interp_method=interp)
    out, _ = _solve(cloud, cfg, illum_of(c))
    o = oracle.solve_tree(cloud, il, c["box"][:3], c["box"][3:], c["depth"], c["n_theta"], c["n_phi"], True)
    assert rel(out.reshape(o.shape), o) < TOL_TREE


@pytest.mark.parametrize("interp", [api.PO_INTERP_TENSOR, api.PO_INTERP_FFT])
@pytest.mark.parametrize("name", ["ref_solve_sphere_d0", "ref_solve_sphere_d3", "ref_solve_ellipsoid_d2",
                                  "ref_solve_sphere_quirk_d1"])
def test_solve_vs_reference_build(cases, name, interp):
    c = cases[name]
    cloud = load_case_geometry(c)
    cfg = api.Config(c["depth"], c["n_theta"], c["n_phi"], c["box"][:3], c["box"][3:],
                     theta_mode=api.PO_THETA_REFERENCE, nyquist_quirk=True, interp_method=interp)
    out, _ = _solve(cloud, cfg, illum_of(c))
    r = ref_fixture(name).reshape(c["n_theta"][0], c["n_phi"][0])
    assert rel(out.reshape(r.shape), r) < TOL_TREE


def test_batched_patterns_match_single_solves():
    cloud = geometry.ellipsoid((1.5e-6, 1.0e-6, 0.8e-6), 3000)
    box = [-1.65e-6, -1.1e-6, -0.88e-6, 1.65e-6, 1.1e-6, 0.88e-6]
    cfg = api.Config.reference_rule(2, 32, 64, box[:3], box[3:], 1.6e-6, 3.0e-6, 1.2)
    lams, ths, phs = [450e-9, 600e-9], [0.2, -0.4, 1.0], [0.3, 2.0, -1.0]
    il = api.Illumination(lams, ths, phs, api.PO_POL_TM | api.PO_POL_TE, 1.55 + 0.1j, 2e-6)
    with api.Solver(cfg) as s:
        allp = s.solve(cloud, il)
        for li, lam in enumerate(lams):
            for ii in range(3):
                for pi, pol in enumerate((api.PO_POL_TM, api.PO_POL_TE)):
                    one = s.solve(cloud, api.Illumination([lam], [ths[ii]], [phs[ii]], pol, 1.55 + 0.1j, 2e-6))
                    assert rel(allp[li, ii, pi], one[0, 0, 0]) < 1e-6


def test_empty_and_single_point():
    box = [-1e-6] * 3 + [1e-6] * 3
    il = api.Illumination([500e-9], [0.3], [0.2])
    for depth in (0, 2):
        cfg = api.Config.reference_rule(depth, 16, 32, box[:3], box[3:], 2e-6, 2e-6, 1.3)
        z = np.zeros(0, np.float32)
        out, _ = _solve(geometry.PointCloud(z, z, z, z, z, z, z), cfg, il)
        assert np.all(out == 0)
        one = geometry.PointCloud([0.3e-6], [-0.2e-6], [0.1e-6], [-1.0], [0.0], [0.0], [1e-14])
        out, _ = _solve(one, cfg, il)
        o = oracle.solve_direct(one, oracle.make_illum(500e-9, 0.3, 0.2), 16, 32)
        assert rel(out.reshape(16, 32), o) < TOL_TREE


def test_invalid_arguments_raise():
    box = [-1e-6] * 3 + [1e-6] * 3
    with pytest.raises(api.WavePOError):
        api.Solver(api.Config(2, [16, 40, 20], [32, 40, 50], box[:3], box[3:]))  # grids grow with depth
    with pytest.raises(api.WavePOError):
        api.Solver(api.Config(1, [16, 8], [32, 8], box[:3], box[:3]))  # empty box
    cfg = api.Config.reference_rule(1, 16, 32, box[:3], box[3:], 2e-6, 2e-6, 1.3)
    with api.Solver(cfg) as s, pytest.raises(api.WavePOError):
        s.solve(geometry.fibonacci_sphere(1e-6, 100), api.Illumination([-5e-7], [0.0], [0.0]))


# ------------------------------------------------ split-precision tensor path
@pytest.mark.parametrize("name", ["ref_solve_sphere_d3", "ref_solve_ellipsoid_d2"])
def test_split_bf16_leaf_vs_fp64_direct(cases, name):
    c = cases[name]
    cloud, il = load_case_geometry(c), case_illum(c)
    cfg = api.Config(c["depth"], c["n_theta"], c["n_phi"], c["box"][:3], c["box"][3:],
                     precision=api.PO_PREC_SPLIT_BF16)
    out, _ = _solve(cloud, cfg, illum_of(c))
    ctr = [(c["box"][i] + c["box"][i + 3]) / 2 for i in range(3)]
    o = oracle.solve_direct(cloud, il, c["n_theta"][0], c["n_phi"][0], center=ctr)
    assert rel(out.reshape(o.shape), o) < TOL_TREE


def test_split_bf16_many_slots_match_fp32():
    """Seven incidences x two polarisations per wavelength (14 slots: the
    tensor-core leaf kernel's slot groups) against the FP32 CUDA-core path."""
    cloud = geometry.ellipsoid((1.5e-6, 1.0e-6, 0.8e-6), 3000)
    box = [-1.65e-6, -1.1e-6, -0.88e-6, 1.65e-6, 1.1e-6, 0.88e-6]
    th = list(np.linspace(-1.2, 1.2, 7))
    ph = list(np.linspace(0.1, 5.9, 7))
    il = api.Illumination([450e-9, 620e-9], th, ph, api.PO_POL_TM | api.PO_POL_TE, 1.55 + 0.1j, 2e-6)
    outs = []
    for prec in (api.PO_PREC_FP32, api.PO_PREC_SPLIT_BF16):
        cfg = api.Config.reference_rule(2, 32, 64, box[:3], box[3:], 1.6e-6, 3.0e-6, 1.2, precision=prec)
        outs.append(_solve(cloud, cfg, il)[0])
    assert rel(outs[1], outs[0]) < 1e-4


# ------------------------------------------------------------ slot chunking
@pytest.mark.parametrize("depth,prec", [(0, api.PO_PREC_FP32), (0, api.PO_PREC_FP64), (2, api.PO_PREC_FP32),
                                        (2, api.PO_PREC_SPLIT_BF16)])
def test_chunked_solve_matches_single_pass(depth, prec):
    """A workspace cap splits the patterns into chunks (single slots, runs of
    one wavelength's slots, groups of whole wavelengths); every chunking gives
    the single-pass result bit for bit."""
    cloud = geometry.ellipsoid((1.5e-6, 1.0e-6, 0.8e-6), 3000)
    box = [-1.65e-6, -1.1e-6, -0.88e-6, 1.65e-6, 1.1e-6, 0.88e-6]
    il = api.Illumination([450e-9, 560e-9, 620e-9], [0.2, -0.4, 1.0], [0.3, 2.0, -1.0],
                          api.PO_POL_TM | api.PO_POL_TE, 1.55 + 0.1j, 2e-6)  # 3 wavelengths x 6 slots
    cfg = api.Config.reference_rule(depth, 24, 48, box[:3], box[3:], 1.6e-6, 3.0e-6, 1.2, precision=prec)
    full, rep = _solve(cloud, cfg, il)
    assert rep["n_chunks"] == 1 and rep["chunk_slots"] == 18
    cfg.max_workspace_bytes = 1
    one, rep1 = _solve(cloud, cfg, il)
    assert rep1["n_chunks"] == 18 and rep1["chunk_slots"] == 1
    assert np.array_equal(one, full)
    per_slot = rep["workspace_bytes"] / 18.0  # roughly: the fixed buffers are small here
    seen = set()
    for k in (4, 7, 13):  # runs of a few slots inside a wavelength; whole wavelengths
        cfg.max_workspace_bytes = int(per_slot * k)
        out, r = _solve(cloud, cfg, il)
        seen.add((r["n_chunks"], r["chunk_slots"]))
        assert np.array_equal(out, full), (k, r["n_chunks"], r["chunk_slots"])
    assert len(seen) >= 2, seen


@pytest.mark.parametrize("prec", [api.PO_PREC_FP32, api.PO_PREC_SPLIT_BF16])
def test_large_level_grids_vs_fp64_direct(prec):
    """The fiber preset's upper level grids (616 x 518 and 323 x 273 under the
    180 x 360 output): theta matrices with 40 k-steps and phi matrices too large
    to stage in shared memory take the reduced-tile paths."""
    cloud = geometry.fibonacci_sphere(1.0e-6, 2000)
    box = [-1.1e-6] * 3 + [1.1e-6] * 3
    cfg = api.Config(2, [180, 616, 323], [360, 518, 273], box[:3], box[3:], precision=prec)
    il = api.Illumination([500e-9], [0.3], [0.7], api.PO_POL_TM, 1.55 + 0.1j, 2e-6)
    out, rep = _solve(cloud, cfg, il)
    o = oracle.solve_direct(cloud, oracle.make_illum(500e-9, 0.3, 0.7, "M", 1.55 + 0.1j, 2e-6), 180, 360)
    assert rel(out.reshape(o.shape), o) < TOL_TREE, rep


@pytest.mark.parametrize("prec", [api.PO_PREC_FP32, api.PO_PREC_SPLIT_BF16])
def test_partial_theta_tiles_vs_fp64_direct(prec):
    """Parent levels of 109, 201 and 241 theta rows (one partly filled 128-row
    tile, two tiles at 78% and at 94%) on the tcgen05 theta pass, with 54,
    100 and 120 column pairs (partly filled 64-pair column chunks), a 61-row
    level on the warp-task kernel, and a 40 x 40 leaf grid whose phi pass to
    60 columns runs in the leaf kernel's epilogue (split-bf16) or as its own
    pass (FP32)."""
    cloud = geometry.ellipsoid((1.5e-6, 1.0e-6, 0.8e-6), 3000)
    box = [-1.65e-6, -1.1e-6, -0.88e-6, 1.65e-6, 1.1e-6, 0.88e-6]
    cfg = api.Config(4, [60, 200, 108, 60, 40], [120, 200, 108, 60, 40], box[:3], box[3:], precision=prec)
    il = api.Illumination([500e-9], [0.3], [0.7], api.PO_POL_TM, 1.55 + 0.1j, 2e-6)
    out, rep = _solve(cloud, cfg, il)
    o = oracle.solve_direct(cloud, oracle.make_illum(500e-9, 0.3, 0.7, "M", 1.55 + 0.1j, 2e-6), 60, 120)
    assert rel(out.reshape(o.shape), o) < TOL_TREE, rep


@pytest.mark.parametrize("prec", [api.PO_PREC_FP32, api.PO_PREC_SPLIT_BF16])
def test_large_leaf_phases_vs_fp64_direct(prec):
    """Leaves of 8.8 um at 500 nm: leaf-local phases reach ~100 rad, so the
    leaf kernels take their range-reduced phasor path (the fast path covers
    |phase| <= 16 rad only)."""
    cloud = geometry.fibonacci_sphere(8.0e-6, 4000)
    box = [-8.8e-6] * 3 + [8.8e-6] * 3
    cfg = api.Config.reference_rule(1, 24, 48, box[:3], box[3:], 17.6e-6, 17.6e-6, 1.2, precision=prec)
    il = api.Illumination([500e-9], [0.3], [0.7], api.PO_POL_TM, 1.55 + 0.1j, 2e-5)
    out, rep = _solve(cloud, cfg, il)
    o = oracle.solve_direct(cloud, oracle.make_illum(500e-9, 0.3, 0.7, "M", 1.55 + 0.1j, 2e-5), 24, 48)
    assert rel(out.reshape(o.shape), o) < TOL_TREE, rep


# ------------------------------------------------------- tcgen05 leaf sums
def _many_incidences(n_inc, seed=3):
    rng = np.random.default_rng(seed)
    return list(rng.uniform(-1.3, 1.3, n_inc)), list(rng.uniform(0.0, 2 * math.pi, n_inc))


def test_leaf_tcgen05_vs_fp64_direct_and_fp32():
    """35 incidences x both polarisations per wavelength (70 patterns: two
    slot groups of the tcgen05 leaf kernel, 64 + 6, and a partly filled
    column tile): every pattern against the FP32 CUDA-core path, and four of
    them against the FP64 oracle direct sum."""
    cloud = geometry.ellipsoid((1.5e-6, 1.0e-6, 0.8e-6), 3000)
    box = [-1.65e-6, -1.1e-6, -0.88e-6, 1.65e-6, 1.1e-6, 0.88e-6]
    th, ph = _many_incidences(35)
    il = api.Illumination([480e-9], th, ph, api.PO_POL_TM | api.PO_POL_TE, 1.55 + 0.1j, 2e-6)
    outs, reps = [], []
    for prec in (api.PO_PREC_FP32, api.PO_PREC_SPLIT_BF16):
        cfg = api.Config.reference_rule(2, 32, 64, box[:3], box[3:], 1.6e-6, 3.0e-6, 1.2, precision=prec)
        o, r = _solve(cloud, cfg, il)
        outs.append(o.reshape(35, 2, 32, 64))
        reps.append(r)
    assert reps[1]["n_leaf_launches"] == 4, reps[1]  # operands + sums, two slot groups
    assert rel(outs[1], outs[0]) < 1e-4
    ctr = [(box[i] + box[i + 3]) / 2 for i in range(3)]
    for ii, pol in ((0, 0), (17, 1), (34, 0), (34, 1)):
        o = oracle.solve_direct(cloud, oracle.make_illum(480e-9, th[ii], ph[ii], "E" if pol else "M", 1.55 + 0.1j,
                                                         2e-6), 32, 64, center=ctr)
        assert rel(outs[1][ii, pol], o) < TOL_TREE, (ii, pol)


def test_leaf_tcgen05_large_phases_vs_fp64_direct():
    """Leaves of 8.8 um at 500 nm (leaf-local phases up to ~100 rad: the
    range-reduced phasor path) with 8 incidences, the smallest pattern count
    that takes the tcgen05 leaf kernel."""
    cloud = geometry.fibonacci_sphere(8.0e-6, 4000)
    box = [-8.8e-6] * 3 + [8.8e-6] * 3
    th, ph = _many_incidences(8, seed=9)
    cfg = api.Config.reference_rule(1, 24, 48, box[:3], box[3:], 17.6e-6, 17.6e-6, 1.2,
                                    precision=api.PO_PREC_SPLIT_BF16)
    il = api.Illumination([500e-9], th, ph, api.PO_POL_TM, 1.55 + 0.1j, 2e-5)
    out, rep = _solve(cloud, cfg, il)
    out = out.reshape(8, 24, 48)
    for ii in (0, 7):
        o = oracle.solve_direct(cloud, oracle.make_illum(500e-9, th[ii], ph[ii], "M", 1.55 + 0.1j, 2e-5), 24, 48)
        assert rel(out[ii], o) < TOL_TREE, (ii, rep)


def test_leaf_tcgen05_chunked_matches_single_pass():
    """Workspace caps that split 2 wavelengths x 9 incidences into single
    slots, runs inside a wavelength and whole wavelengths give the single-pass
    result bit for bit (every output column of the tcgen05 products depends
    on its own column of the currents only)."""
    cloud = geometry.ellipsoid((1.5e-6, 1.0e-6, 0.8e-6), 3000)
    box = [-1.65e-6, -1.1e-6, -0.88e-6, 1.65e-6, 1.1e-6, 0.88e-6]
    th, ph = _many_incidences(9, seed=4)
    il = api.Illumination([450e-9, 620e-9], th, ph, api.PO_POL_TM, 1.55 + 0.1j, 2e-6)
    cfg = api.Config.reference_rule(2, 24, 48, box[:3], box[3:], 1.6e-6, 3.0e-6, 1.2,
                                    precision=api.PO_PREC_SPLIT_BF16)
    full, rep = _solve(cloud, cfg, il)
    assert rep["n_chunks"] == 1
    per_slot = rep["workspace_bytes"] / 18.0
    for cap in (1, int(per_slot * 4), int(per_slot * 11)):
        cfg.max_workspace_bytes = cap
        out, r = _solve(cloud, cfg, il)
        assert r["n_chunks"] > 1
        assert np.array_equal(out, full), (cap, r["n_chunks"], r["chunk_slots"])


@pytest.mark.parametrize("n_inc,kernel,slots", [(1, api.PO_LEAF_TCGEN05, 8), (3, api.PO_LEAF_TCGEN05, 0),
                                                 (20, api.PO_LEAF_TCGEN05, 16), (9, api.PO_LEAF_WARP, 0)])
def test_leaf_schedule_choices_vs_fp64_direct(n_inc, kernel, slots):
    """The autotuner's leaf-batch schedules: the tcgen05 leaf kernel forced
    below its automatic threshold (1 and 3 patterns per wavelength) and in
    passes of 16 patterns, the warp-level kernel forced above it.  Each
    against the FP64 oracle; the tcgen05 passes of any size give the
    automatic schedule's result bit for bit (every output column depends on
    its own column of the currents only)."""
    cloud = geometry.ellipsoid((1.5e-6, 1.0e-6, 0.8e-6), 3000)
    box = [-1.65e-6, -1.1e-6, -0.88e-6, 1.65e-6, 1.1e-6, 0.88e-6]
    th, ph = _many_incidences(n_inc, seed=5)
    il = api.Illumination([520e-9], th, ph, api.PO_POL_TM, 1.55 + 0.1j, 2e-6)
    cfg = api.Config.reference_rule(2, 24, 48, box[:3], box[3:], 1.6e-6, 3.0e-6, 1.2,
                                    precision=api.PO_PREC_SPLIT_BF16, leaf_kernel=kernel, leaf_slots=slots)
    out, rep = _solve(cloud, cfg, il)
    out = out.reshape(n_inc, 24, 48)
    per_pass = slots or 64
    want = 2 * -(-n_inc // per_pass) if kernel == api.PO_LEAF_TCGEN05 else -(-n_inc // 4)
    assert rep["n_leaf_launches"] == want, rep
    ctr = [(box[i] + box[i + 3]) / 2 for i in range(3)]
    for ii in sorted({0, n_inc - 1}):
        o = oracle.solve_direct(cloud, oracle.make_illum(520e-9, th[ii], ph[ii], "M", 1.55 + 0.1j, 2e-6), 24, 48,
                                center=ctr)
        assert rel(out[ii], o) < TOL_TREE, (ii, rep)
    if kernel == api.PO_LEAF_TCGEN05 and n_inc >= 8:
        auto, _ = _solve(cloud, dataclasses.replace(cfg, leaf_kernel=api.PO_LEAF_AUTO, leaf_slots=0), il)
        assert np.array_equal(out.reshape(auto.shape), auto)


def test_reference_mode_tensor_path_on_large_grids():
    """The reference theta mode on the tensor cores where its maps are real and
    column-independent: a 2,000-point sphere with even parent grids (the
    levels take the tcgen05 and warp-level tensor kernels) against the oracle's
    restatement of the reference's FFT interpolation, and the same solve with
    the FFT path."""
    cloud = geometry.fibonacci_sphere(1.0e-6, 2000)
    box = [-1.1e-6] * 3 + [1.1e-6] * 3
    nth, nph = [100, 75, 41], [200, 74, 40]  # root on the tcgen05 theta pass, level 1 on the warp-level one
    il = api.Illumination([500e-9], [0.3], [0.7], api.PO_POL_TM, 1.55 + 0.1j, 2e-6)
    outs = []
    for interp in (api.PO_INTERP_TENSOR, api.PO_INTERP_FFT):
        cfg = api.Config(2, nth, nph, box[:3], box[3:], theta_mode=api.PO_THETA_REFERENCE, nyquist_quirk=True,
                         interp_method=interp)
        outs.append(_solve(cloud, cfg, il)[0].reshape(nth[0], nph[0]))
    o = oracle.solve_tree(cloud, oracle.make_illum(500e-9, 0.3, 0.7, "M", 1.55 + 0.1j, 2e-6), box[:3], box[3:], 2,
                          nth, nph, True)
    assert rel(outs[0], o) < TOL_TREE
    assert rel(outs[0], outs[1]) < TOL_TREE


@pytest.mark.parametrize("prec", [api.PO_PREC_FP32, api.PO_PREC_SPLIT_BF16])
def test_reference_mode_tensor_path_on_odd_phi_grids(prec):
    """Odd parent phi grids in the reference theta mode, whose columns do not
    pair up as phi and phi + pi: the tensor path pairs column j with
    j + (Phi + 1)/2 (one phantom partner) and takes each partner's translation
    from its own table entry.  Level 1 (45 columns) and level 2 (27 columns,
    the deepest parent: its phi pass runs fused into the split-precision leaf
    kernel) are odd; checked against the oracle's restatement of the
    reference's FFT interpolation and against the FFT path."""
    cloud = geometry.fibonacci_sphere(1.0e-6, 2000)
    box = [-1.1e-6] * 3 + [1.1e-6] * 3
    nth, nph = [48, 40, 26, 16], [96, 45, 27, 16]
    il = api.Illumination([500e-9], [0.3], [0.7], api.PO_POL_TM, 1.55 + 0.1j, 2e-6)
    outs = []
    for interp in (api.PO_INTERP_TENSOR, api.PO_INTERP_FFT):
        cfg = api.Config(3, nth, nph, box[:3], box[3:], theta_mode=api.PO_THETA_REFERENCE, nyquist_quirk=True,
                         interp_method=interp, precision=prec)
        outs.append(_solve(cloud, cfg, il)[0].reshape(nth[0], nph[0]))
    o = oracle.solve_tree(cloud, oracle.make_illum(500e-9, 0.3, 0.7, "M", 1.55 + 0.1j, 2e-6), box[:3], box[3:], 3,
                          nth, nph, True)
    assert rel(outs[0], o) < TOL_TREE
    assert rel(outs[0], outs[1]) < TOL_TREE
