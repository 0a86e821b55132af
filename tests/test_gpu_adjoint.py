"""Gradients (po_grad, po_height_field_adjoint, the torch.autograd bindings)
against central finite differences of the FP64 oracle.

Loss: L = sum(w * I) with seeded weights w (so dL/dI = w).  The finite
differences perturb one coordinate of one sample at a time in the FP64
oracle (oracle.solve_direct_f64); points are taken well inside the lit
region so that no lit/shadow switch lies within a step.

Tolerances (relative L2 over the checked points, per group of components):
  FP64 depth 0 (the whole chain in FP64) ............ 1e-6
  FP32 depth 0 ...................................... 1e-4
  depth 2, split-BF16 leaf + tensor interpolation ... 1e-3 (the tree map itself
                                                       differs from the direct sum)
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import oracle  # noqa: E402
from wavefiber3d_gb300 import api, autograd, geometry  # noqa: E402

NTH, NPH = 24, 48
BOX = [-1.65e-6, -1.1e-6, -0.88e-6, 1.65e-6, 1.1e-6, 0.88e-6]
LAM, TH, PH, ETA, SIG = 600e-9, 0.4, -0.7, 1.55 + 0.1j, 3e-6
GROUPS = {"position": [0, 1, 2], "normal": [3, 4, 5], "area": [6]}


@pytest.fixture(scope="module")
def case():
    cloud = geometry.ellipsoid((1.5e-6, 1.0e-6, 0.8e-6), 2000)
    s64 = cloud.soa().astype(np.float64)
    rng = np.random.default_rng(5)
    w = rng.standard_normal((NTH, NPH))
    k = np.array([math.cos(TH) * math.cos(PH), math.cos(TH) * math.sin(PH), math.sin(TH)])
    dot = s64[3:6].T @ k
    lit = np.flatnonzero((dot < -0.25) & (dot > -0.95))
    pts = rng.choice(lit, size=8, replace=False)
    il_o = oracle.make_illum(LAM, TH, PH, "E", ETA, SIG)
    fd = np.zeros((7, pts.size))
    for j, p in enumerate(pts):
        for q in range(7):
            h = 2e-10 if q < 3 else (1e-6 if q < 6 else 1e-6 * s64[6, p])
            a, b = s64.copy(), s64.copy()
            a[q, p] += h
            b[q, p] -= h
            la = float((w * oracle.solve_direct_f64(a, il_o, NTH, NPH)).sum())
            lb = float((w * oracle.solve_direct_f64(b, il_o, NTH, NPH)).sum())
            fd[q, j] = (la - lb) / (2 * h)
    return cloud, w, pts, fd


def gpu_grad(cloud, w, depth, precision):
    il = api.Illumination([LAM], [TH], [PH], api.PO_POL_TE, ETA, SIG)
    if depth == 0:
        cfg = api.Config(0, [NTH], [NPH], BOX[:3], BOX[3:], precision=precision)
    else:
        cfg = api.Config.reference_rule(depth, NTH, NPH, BOX[:3], BOX[3:], 1.6e-6, 3.0e-6, 1.2, precision=precision)
    samples = torch.from_numpy(cloud.soa()).cuda()
    with api.Solver(cfg) as s:
        g, inten = s.grad(samples, il, torch.from_numpy(w).float(), with_intensity=True)
        plain = s.solve(tuple(samples[k] for k in range(7)), il)
    assert torch.equal(inten, plain)  # the recomputed forward is the solve
    return g.cpu().numpy().astype(np.float64)


def check(g, pts, fd, tol):
    for name, rows in GROUPS.items():
        a, b = g[rows][:, pts], fd[rows]
        err = np.linalg.norm(a - b) / np.linalg.norm(b)
        assert err < tol, (name, err)


def test_grad_fp64_depth0_vs_fd(case):
    cloud, w, pts, fd = case
    check(gpu_grad(cloud, w, 0, api.PO_PREC_FP64), pts, fd, 1e-6)


def test_grad_fp32_depth0_vs_fd(case):
    cloud, w, pts, fd = case
    check(gpu_grad(cloud, w, 0, api.PO_PREC_FP32), pts, fd, 1e-4)


@pytest.mark.parametrize("precision", [api.PO_PREC_FP32, api.PO_PREC_SPLIT_BF16])
def test_grad_tree_vs_fd(case, precision):
    cloud, w, pts, fd = case
    check(gpu_grad(cloud, w, 2, precision), pts, fd, 1e-3)


def test_grad_tree_matches_fp64_gradient_everywhere(case):
    """All points and components: the depth-3 tree gradient against the FP64
    depth-0 gradient (the FP64 reference gradient)."""
    cloud, w, _, _ = case
    ref = gpu_grad(cloud, w, 0, api.PO_PREC_FP64)
    g = gpu_grad(cloud, w, 3, api.PO_PREC_SPLIT_BF16)
    for name, rows in GROUPS.items():
        err = np.linalg.norm(g[rows] - ref[rows]) / np.linalg.norm(ref[rows])
        assert err < 1e-3, (name, err)


def test_grad_many_slots_and_chunks(case):
    """Two wavelengths x two incidences x both polarisations, with a workspace
    cap that splits them into chunks: equals the sum of single-pattern grads."""
    cloud, _, _, _ = case
    cfg = api.Config.reference_rule(2, NTH, NPH, BOX[:3], BOX[3:], 1.6e-6, 3.0e-6, 1.2)
    il = api.Illumination([450e-9, 600e-9], [0.2, -0.5], [0.3, 2.0], api.PO_POL_TM | api.PO_POL_TE, ETA, SIG)
    rng = np.random.default_rng(8)
    w = torch.from_numpy(rng.standard_normal((2, 2, 2, NTH, NPH))).float()
    samples = torch.from_numpy(cloud.soa()).cuda()
    with api.Solver(cfg) as s:
        g_all = s.grad(samples, il, w).cpu().numpy().astype(np.float64)
    cfg.max_workspace_bytes = 1
    with api.Solver(cfg) as s:
        g_chunk = s.grad(samples, il, w).cpu().numpy().astype(np.float64)
        assert s.last_report["n_chunks"] == 8
    assert np.allclose(g_chunk, g_all, rtol=1e-5, atol=1e-6 * np.abs(g_all).max())
    acc = np.zeros_like(g_all)
    with api.Solver(api.Config.reference_rule(2, NTH, NPH, BOX[:3], BOX[3:], 1.6e-6, 3.0e-6, 1.2)) as s:
        for li, lam in enumerate([450e-9, 600e-9]):
            for ii in range(2):
                for pi, pol in enumerate((api.PO_POL_TM, api.PO_POL_TE)):
                    one = api.Illumination([lam], [il.theta_i[ii]], [il.phi_i[ii]], pol, ETA, SIG)
                    acc += s.grad(samples, one, w[li, ii, pi]).cpu().numpy()
    assert np.linalg.norm(acc - g_all) / np.linalg.norm(g_all) < 1e-5


# ----------------------------------------------------- height-field adjoint
def hf_samples64(xy, period, unitz, b, e):
    """Float64 restatement of the quad map of util/geometry.h:76-179."""
    numel, numelvert = xy.shape[1], xy.shape[2]
    i = np.arange(numelvert)
    j = np.arange(b, e + 1)
    jj, ii = np.meshgrid(j, i)  # [i][j]
    pj = np.where(jj < numel - 1, jj + 1, 0)
    zi = np.where(ii < numelvert - 1, ii + 1, ii)
    z = (ii * np.float32(unitz)).astype(np.float32) - np.float32(period * 0.5)
    zn = ((ii + 1) * np.float32(unitz)).astype(np.float32) - np.float32(period * 0.5)
    P = [np.stack([xy[0][a, c], xy[1][a, c], zz.astype(np.float64)]) for a, c, zz in
         ((jj, ii, z), (pj, ii, z), (jj, zi, zn), (pj, zi, zn))]
    a1 = np.cross(P[1] - P[0], P[2] - P[0], axis=0)
    a2 = np.cross(P[3] - P[1], P[2] - P[1], axis=0)
    sm = a1 + a2
    nrm = sm / np.linalg.norm(sm, axis=0)
    ctr = (P[0] + P[1] + P[2] + P[3]) / 4
    area = 0.5 * (np.linalg.norm(a1, axis=0) + np.linalg.norm(a2, axis=0))
    return np.concatenate([ctr, nrm, area[None]]).reshape(7, -1)


def test_height_field_adjoint_vs_fd():
    hf = geometry.fiber_height_field(radii=(2e-6, 1.6e-6), length=1.0e-6, spacing=0.1e-6, seed=12)
    b, e = 10, 60
    rng = np.random.default_rng(3)
    n = (e - b + 1) * hf.numelvert
    gs = rng.standard_normal((7, n))
    gs[:3] *= 1e6  # comparable magnitudes of the position / normal / area terms
    gs[6] *= 1e12
    g = api.height_field_adjoint(torch.from_numpy(hf.xy), hf.period, hf.unitz, b, e,
                                 torch.from_numpy(gs).float()).cpu().numpy().astype(np.float64)
    xy = hf.xy.astype(np.float64)
    gsf = gs.astype(np.float32).astype(np.float64)
    got, want = [], []
    for (c, jv, iv) in [(0, 11, 3), (1, 11, 3), (0, 35, hf.numelvert - 1), (1, 60, 5), (0, 61, 2), (1, 10, 0),
                        (0, 9, 4)]:
        h = 1e-12
        a, bb = xy.copy(), xy.copy()
        a[c, jv, iv] += h
        bb[c, jv, iv] -= h
        fd = ((gsf * hf_samples64(a, hf.period, hf.unitz, b, e)).sum() -
              (gsf * hf_samples64(bb, hf.period, hf.unitz, b, e)).sum()) / (2 * h)
        got.append(g[c, jv, iv])
        want.append(fd)
    got, want = np.array(got), np.array(want)
    assert want[-1] == 0 and got[-1] == 0  # vertex column 9 is outside the segment
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-5


# ------------------------------------------------------------ autograd
def test_autograd_chain_height_field_to_loss():
    hf = geometry.fiber_height_field(radii=(2e-6, 1.6e-6), length=1.2e-6, spacing=0.05e-6, seed=4)
    box = [-2.4e-6, -2.0e-6, -0.7e-6, 2.4e-6, 2.0e-6, 0.7e-6]
    cfg = api.Config.reference_rule(2, NTH, NPH, box[:3], box[3:], 1.2e-6, 4.0e-6, 1.2)
    il = api.Illumination([500e-9], [0.1], [0.0], api.PO_POL_TM, ETA, 2e-6)
    xy = torch.from_numpy(hf.xy).cuda().requires_grad_(True)
    w = torch.from_numpy(np.random.default_rng(2).standard_normal((1, 1, 1, NTH, NPH))).float().cuda()
    with api.Solver(cfg) as s:
        samples = autograd.height_field_samples(xy, hf.period, hf.unitz)
        inten = autograd.far_field_intensity(s, il, samples)
        loss = (inten * w).sum()
        loss.backward()
        g_samples = s.grad(samples.detach(), il, w)
    want = api.height_field_adjoint(xy.detach(), hf.period, hf.unitz, 0, hf.numel - 1, g_samples)
    assert torch.allclose(xy.grad, want, rtol=1e-6, atol=0)
    assert torch.isfinite(xy.grad).all() and xy.grad.abs().max() > 0
