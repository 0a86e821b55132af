"""The differentiation workload at reduced size: a rough circular cylinder with
a normal displacement field h (Gaussian, sigma 0.02 um, correlation 0.5 um,
seeded; the same statistics and point spacing as the 1M-point workload), two
wavelengths x two incidences, TM, octree depth 3.  Loss
L = sum (I(h) - I_target)^2 with the target from a second seed.

Checks (tolerances are relative L2):
  * the tree gradient (FP32 and split-BF16 leaves) against the FP64 depth-0
    gradient of the whole chain, per group of components (positions,
    normals, areas) and for dL/dh through the height-field adjoint: <= 1e-3;
  * per point and per component on 64 random lit points, against central
    differences of the FP64 oracle (oracle.point_gradient_fd) of a loss over
    512 sampled directions: FP64 chain <= 1e-6, tree <= 1e-3.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import oracle  # noqa: E402
from wavefiber3d_gb300 import api, geometry  # noqa: E402

R, LEN, NPTS = 2.5e-6, 4e-6, 50_000
NTH, NPH = 90, 180
LAMS, THS = [400e-9, 688e-9], [0.0, 0.35]
ETA = 1.55 + 0.1j
BOX = [-1.1 * R, -1.1 * R, -0.55 * LEN]
GROUPS = {"positions": slice(0, 3), "normals": slice(3, 6), "areas": slice(6, 7)}
STEPS = [1e-10] * 3 + [1e-6] * 3 + [1e-6]


@pytest.fixture(scope="module")
def cyl():
    hf, h = geometry.cylinder_height_field(R, LEN, NPTS, seed=1)
    _, h_t = geometry.cylinder_height_field(R, LEN, NPTS, seed=2)
    phi = 2 * np.pi * np.arange(hf.numel) / hf.numel

    def xy_of(hh):
        r = R + hh
        return torch.from_numpy(np.stack([r * np.cos(phi)[:, None], r * np.sin(phi)[:, None]])).float().cuda()

    xy, xy_t = xy_of(h), xy_of(h_t)
    s0 = api.height_field_points_tensor(xy, hf.period, hf.unitz, 0, hf.numel - 1)
    s_t = api.height_field_points_tensor(xy_t, hf.period, hf.unitz, 0, hf.numel - 1)
    il = api.Illumination(LAMS, THS, [0.0] * len(THS), api.PO_POL_TM, ETA, 1.0)
    cfg64 = api.Config(0, [NTH], [NPH], BOX, [-v for v in BOX], precision=api.PO_PREC_FP64)
    with api.Solver(cfg64) as s64, torch.no_grad():
        i64 = s64.solve(tuple(s0[k] for k in range(7)), il)
        it = s64.solve(tuple(s_t[k] for k in range(7)), il)
        w = 2 * (i64 - it)
        g64 = s64.grad(s0, il, w).double()
    return dict(hf=hf, phi=phi, xy=xy, s0=s0, il=il, w=w, g64=g64, i64=i64, it=it)


def tree_config(precision):
    # level grids by the reference rule on a 7 um extent (the cells of the 5.5 x 5.5 x 4.4 um box)
    return api.Config.reference_rule(3, NTH, NPH, BOX, [-v for v in BOX], 7e-6, 7e-6, 1.2, precision=precision)


def dl_dh(c, g):
    hf = c["hf"]
    gh = api.height_field_adjoint(c["xy"], hf.period, hf.unitz, 0, hf.numel - 1, g.float()).double().cpu().numpy()
    return gh[0] * np.cos(c["phi"])[:, None] + gh[1] * np.sin(c["phi"])[:, None]


@pytest.mark.parametrize("precision", [api.PO_PREC_FP32, api.PO_PREC_SPLIT_BF16])
def test_tree_gradient_vs_fp64_gradient(cyl, precision):
    with api.Solver(tree_config(precision)) as s, torch.no_grad():
        g, inten = s.grad(cyl["s0"], cyl["il"], cyl["w"], with_intensity=True)
    fwd = float((inten.double() - cyl["i64"].double()).norm() / cyl["i64"].double().norm())
    assert fwd < 1e-4, fwd
    g, g64 = g.double(), cyl["g64"]
    errs = {k: float((g[r] - g64[r]).norm() / g64[r].norm()) for k, r in GROUPS.items()}
    h_ref = dl_dh(cyl, g64)
    errs["dL/dh"] = float(np.linalg.norm(dl_dh(cyl, g) - h_ref) / np.linalg.norm(h_ref))
    for k, e in errs.items():
        assert e <= 1e-3, (k, e, errs)


def test_per_point_gradient_vs_oracle_fd(cyl):
    """64 random lit points, every component, every pattern of the loss."""
    s0 = cyl["s0"].double().cpu().numpy()
    rng = np.random.default_rng(64)
    lit = np.flatnonzero(s0[3] < -0.1)  # lit under both incidences (k along +x, tilted)
    pts = np.sort(rng.choice(lit, 64, replace=False))
    dirs = np.sort(rng.choice(NTH * NPH, 512, replace=False))
    w_full = torch.zeros_like(cyl["w"])
    w_full.view(len(LAMS), len(THS), 1, -1)[..., dirs] = cyl["w"].view(len(LAMS), len(THS), 1, -1)[..., dirs]
    fd = np.zeros((7, pts.size))
    for li, lam in enumerate(LAMS):
        for ii, th in enumerate(THS):
            il_o = oracle.make_illum(lam, th, 0.0, "M", ETA, 1.0)
            wv = w_full[li, ii, 0].reshape(-1).double().cpu().numpy()[dirs]
            fd += oracle.point_gradient_fd(s0, il_o, NTH, NPH, dirs, wv, pts, STEPS)
    cfg64 = api.Config(0, [NTH], [NPH], BOX, [-v for v in BOX], precision=api.PO_PREC_FP64)
    for cfg, tol in ((cfg64, 1e-6), (tree_config(api.PO_PREC_FP32), 1e-3),
                     (tree_config(api.PO_PREC_SPLIT_BF16), 1e-3)):
        with api.Solver(cfg) as s, torch.no_grad():
            g = s.grad(cyl["s0"], cyl["il"], w_full).double().cpu().numpy()[:, pts]
        for q in range(7):
            err = np.linalg.norm(g[q] - fd[q]) / np.linalg.norm(fd[q])
            assert err <= tol, (cfg.precision, q, err)
