"""GPU pattern statistics (po_shifted_fft2 both directions, po_acf_from_patterns and the
fitting module) against the numpy restatement of fitting/fittingutil.py
(oracle/acf.py).  Tolerance: relative L2 1e-5 (FP32 DFT accumulation)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from oracle import acf as ref  # noqa: E402
from wavefiber3d_gb300 import fitting  # noqa: E402

TOL = 1e-5


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("shape", [(3, 180, 360), (2, 45, 88), (1, 7, 13), (4, 33, 32)])
def test_shifted_fft2_vs_numpy(shape):
    rng = np.random.default_rng(sum(shape))
    a = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
    got = fitting.forward_fft_shifted(a).cpu().numpy()
    inv = fitting.inverse_fft_shifted(a).cpu().numpy()
    for b in range(shape[0]):
        assert rel(got[b], ref.forward_fft_shifted(a[b].astype(np.complex128))) < TOL
        assert rel(inv[b], ref.inverse_fft_shifted(a[b].astype(np.complex128))) < TOL


def test_acf_pipeline_vs_numpy():
    """weightedsum -> ACFfromFT and ACFweightedFT on band noise fields of the
    fitting notebook's layout ([theta][phi][instance][band])."""
    rng = np.random.default_rng(9)
    raw = rng.exponential(1.0, (90, 180, 24, 3)).astype(np.float32)
    w = [0.7, 1.1, 0.4]
    nm, mean = fitting.weightedsum(raw, w)
    nm_r, mean_r = ref.weightedsum(raw, w)
    assert rel(nm.cpu().numpy(), nm_r) < TOL and rel(mean.cpu().numpy(), mean_r) < TOL
    spec, acf, mean_g = fitting.acf_from_ft(nm)
    spec_r, acf_r = ref.acf_from_ft(nm_r, mean_r)
    assert rel(mean_g.cpu().numpy(), mean_r) < TOL
    assert rel(spec.cpu().numpy(), spec_r) < TOL
    assert rel(acf.cpu().numpy(), acf_r) < TOL
    fm = np.stack([spec_r, 0.5 * spec_r, spec_r ** 0.5], axis=-1)
    wft, acfw = fitting.acf_weighted_ft(fm, w)
    wft_r, acfw_r = ref.acf_weighted_ft(fm, w)
    assert rel(wft.cpu().numpy(), wft_r) < TOL and rel(acfw.cpu().numpy(), acfw_r) < TOL
