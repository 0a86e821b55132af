"""Failure handling of the bounded device waits (po_selftest_device_waits,
po_check): a tcgen05 kernel that finds its operand buffer too small records
PO_ERR_INTERNAL without issuing a copy; one whose first copy stage is
withheld gives up its waits after the 1-s limit and records PO_ERR_TIMEOUT.
After each, a normal solve in the same process (same CUDA context, same
solver) still matches the FP64 oracle, and po_check reports nothing stale."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import oracle  # noqa: E402
from wavefiber3d_gb300 import api, geometry  # noqa: E402
from wavefiber3d_gb300._lib import STATUS_NAMES  # noqa: E402


@pytest.fixture(scope="module")
def solver_case():
    cloud = geometry.ellipsoid((1.5e-6, 1.0e-6, 0.8e-6), 3000)
    box = [-1.65e-6, -1.1e-6, -0.88e-6, 1.65e-6, 1.1e-6, 0.88e-6]
    # 201-row level: the tcgen05 theta pass; 8 incidences: the tcgen05 leaf sums
    cfg = api.Config(2, [60, 200, 108], [120, 200, 108], box[:3], box[3:], precision=api.PO_PREC_SPLIT_BF16)
    th = list(np.linspace(-1.0, 1.0, 8))
    il = api.Illumination([500e-9], th, [0.7] * 8, api.PO_POL_TM, 1.55 + 0.1j, 2e-6)
    refs = [oracle.solve_direct(cloud, oracle.make_illum(500e-9, th[i], 0.7, "M", 1.55 + 0.1j, 2e-6), 60, 120)
            for i in (0, 7)]
    s = api.Solver(cfg)
    yield s, cloud, il, refs
    s.close()


def solve_and_check(s, cloud, il, refs):
    out = s.solve(cloud, il)
    assert s.last_report["n_leaf_launches"] == 2  # the tcgen05 leaf path
    for j, ref in zip((0, 7), refs):
        got = out[0, j, 0].astype(np.float64)
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-4
    s.check()  # nothing recorded


@pytest.mark.parametrize("which,expected", [(1, "PO_ERR_INTERNAL"), (2, "PO_ERR_TIMEOUT"), (3, "PO_ERR_TIMEOUT")])
def test_wait_failure_is_reported_and_context_stays_usable(solver_case, which, expected):
    s, cloud, il, refs = solver_case
    solve_and_check(s, cloud, il, refs)
    status = api.selftest_device_waits(which)
    assert STATUS_NAMES[status] == expected
    torch.cuda.synchronize()  # the context answers
    solve_and_check(s, cloud, il, refs)


def test_selftest_rejects_unknown_case():
    assert STATUS_NAMES[api.selftest_device_waits(0)] == "PO_ERR_INVALID_ARGUMENT"
