"""Batched solves captured in one CUDA graph (po_batch_*) against the same
solves run one by one through po_solve: bit-identical, on replay too; and a
batch of autotuned solves against the FP64 oracle."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from wavefiber3d_gb300 import api, geometry  # noqa: E402


def items():
    rng = np.random.default_rng(11)
    out = []
    for i, (kind, r, n, depth, prec) in enumerate([
            ("sphere", 1.0e-6, 3000, 0, api.PO_PREC_FP32), ("ellipsoid", 1.5e-6, 6000, 2, api.PO_PREC_FP32),
            ("sphere", 2.0e-6, 20000, 3, api.PO_PREC_SPLIT_BF16), ("ellipsoid", 1.2e-6, 5000, 1, api.PO_PREC_SPLIT_BF16),
            ("sphere", 0.8e-6, 2000, 2, api.PO_PREC_FP32), ("ellipsoid", 2.5e-6, 30000, 3, api.PO_PREC_FP32)]):
        cloud = geometry.fibonacci_sphere(r, n) if kind == "sphere" else geometry.ellipsoid((r, 0.7 * r, 0.6 * r), n)
        box = [-1.1 * r] * 3, [1.1 * r] * 3
        cfg = api.Config.reference_rule(depth, 24, 48, *box, 2 * r, 2 * r, 1.3, precision=prec,
                                        interp_tile=[0, 8, 16][i % 3])
        lam = float(rng.uniform(400e-9, 700e-9))
        il = api.Illumination([lam], [float(rng.uniform(-1.2, 1.2))], [float(rng.uniform(0, 2 * math.pi))],
                              api.PO_POL_TM, 1.55 + 0.1j, 1.0)
        out.append((torch.from_numpy(cloud.soa()).cuda(), cfg, il))
    return out


def test_batch_matches_single_solves():
    its = items()
    want = []
    for g, cfg, il in its:
        with api.Solver(cfg) as s:
            want.append(s.solve(tuple(g[k] for k in range(7)), il).clone())
    with api.Batch([c for _, c, _ in its], n_streams=3) as b:
        b.prepare([g for g, _, _ in its], [il for _, _, il in its])
        for rep in range(2):
            for o in b.outputs:
                o.fill_(-1.0)
            outs = b.launch()
            torch.cuda.synchronize()
            for o, w in zip(outs, want):
                assert torch.equal(o, w)
        info = b.info()
        assert info["graph_nodes"] > len(its) and info["workspace_bytes"] > 0


def test_batch_argument_errors():
    g, cfg, il = items()[0]
    with pytest.raises(api.WavePOError):
        api.Batch([cfg], n_streams=0)
    fp64 = api.Config(0, [24], [48], [-1e-6] * 3, [1e-6] * 3, precision=api.PO_PREC_FP64)
    with pytest.raises(api.WavePOError, match="UNSUPPORTED"):
        api.Batch([fp64])
    with api.Batch([cfg]) as b, pytest.raises(api.WavePOError):
        b.launch()  # nothing captured yet


def test_autotuned_batch_vs_fp64_oracle():
    """The autotuner on the GPU (real timings) for three geometry classes, one
    of them with 16 patterns per wavelength (its leaf-batch schedule is
    searched), then the chosen configs in one captured batch: every item
    against the FP64 oracle on 64 seeded directions, and the batch's device
    waits checked (po_batch_check)."""
    import oracle
    from wavefiber3d_gb300 import autotune
    rng = np.random.default_rng(5)
    tuner = autotune.Autotuner(reps=1)
    its = []
    for r, n, n_inc in ((1.0e-6, 4000, 1), (2.0e-6, 30000, 1), (1.5e-6, 12000, 16)):
        cloud = geometry.ellipsoid((r, 0.75 * r, 0.6 * r), n)
        g = torch.from_numpy(cloud.soa()).cuda()
        th = list(rng.uniform(-1.2, 1.2, n_inc))
        ph = list(rng.uniform(0, 2 * math.pi, n_inc))
        il = api.Illumination([float(rng.uniform(400e-9, 700e-9))], th, ph, api.PO_POL_TM, 1.55 + 0.1j, 1.0)

        def make(depth, prec, r=r):
            return api.Config.reference_rule(depth, 30, 60, [-1.1 * r] * 3, [1.1 * r] * 3, 2 * r, 2 * r, 1.3,
                                             precision=prec)
        ch = tuner.choose(g, il, make, 2 * r)
        assert ch["ms"] > 0 and set(ch) == {"depth", "precision", "tile", "leaf_kernel", "leaf_slots", "ms"}
        its.append((cloud, g, autotune.apply(make(ch["depth"], ch["precision"]), ch), il))
    assert tuner.trials >= 3 * 3 and len(tuner.cache) == 3
    with api.Batch([c for _, _, c, _ in its], n_streams=2) as b:
        b.prepare([g for _, g, _, _ in its], [il for _, _, _, il in its])
        outs = b.launch()
        b.check()
        dirs = np.sort(np.random.default_rng(8).choice(30 * 60, 64, replace=False))
        for (cloud, _, cfg, il), o in zip(its, outs):
            o = o.cpu().numpy().reshape(len(il.theta_i), -1)
            for j in sorted({0, len(il.theta_i) - 1}):
                il_o = oracle.make_illum(il.wavelengths_m[0], il.theta_i[j], il.phi_i[j], "M", 1.55 + 0.1j, 1.0)
                ref = oracle.solve_sampled_f64(cloud.soa().astype(np.float64), il_o, 30, 60, dirs)
                err = np.linalg.norm(o[j][dirs] - ref) / np.linalg.norm(ref)
                assert err <= 1e-3, (cfg.max_depth, cfg.precision, cfg.leaf_kernel, cfg.leaf_slots, j, err)
