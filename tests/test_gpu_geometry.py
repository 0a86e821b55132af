"""GPU parity of the height-field sampler (po_height_field_points) against
the reference's own set_sourcepoint (tests/golden/ref_heightfield_*.bin) and
the float oracle restatement: bit-exact."""
import numpy as np
import pytest

from conftest import GOLDEN, load_case_height_field

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import oracle  # noqa: E402
from wavefiber3d_gb300 import api, geometry  # noqa: E402
from wavefiber3d_gb300._lib import WavePOError  # noqa: E402


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


@pytest.mark.parametrize("name", ["ref_heightfield_full", "ref_heightfield_segment", "ref_heightfield_wrap"])
def test_height_field_vs_reference_build(cases, name):
    hf, b, e = load_case_height_field(cases[name])
    out = api.height_field_points(hf, b, e).cpu().numpy()
    ref = np.fromfile(GOLDEN / f"{name}.bin", dtype=np.float32).reshape(7, -1)
    assert np.array_equal(bits(out), bits(ref))


def test_height_field_fiber_segment_vs_oracle():
    """The 25 x 20 um x 60 um fiber segment at 0.05 um spacing (3.4 M samples)."""
    hf = geometry.fiber_height_field(seed=3)
    out = api.height_field_points(hf).cpu().numpy()
    ref, bad = oracle.height_field(hf)
    assert not bad and out.shape == (7, 3403200)
    assert np.array_equal(bits(out), bits(ref))


@pytest.mark.parametrize("ring", [(0, 0), (0, 31), (1, 33), (7, 112), (112, 112)])
def test_height_field_ring_segments_vs_oracle(ring):
    hf = geometry.fiber_height_field(radii=(2e-6, 1.6e-6), length=4.1e-6, spacing=0.1e-6, seed=5)
    assert hf.numel == 113 and hf.numelvert == 41  # ragged against the 32 x 32 tiles
    out = api.height_field_points(hf, *ring).cpu().numpy()
    ref, _ = oracle.height_field(hf, *ring)
    assert np.array_equal(bits(out), bits(ref))


def test_height_field_single_row():
    hf = geometry.fiber_height_field(radii=(2e-6, 1.6e-6), length=0.1e-6, spacing=0.1e-6, seed=6)
    assert hf.numelvert == 1
    out = api.height_field_points(hf).cpu().numpy()
    ref, _ = oracle.height_field(hf)
    assert np.array_equal(bits(out), bits(ref))


def test_height_field_errors():
    hf = geometry.fiber_height_field(radii=(2e-6, 1.6e-6), length=0.5e-6, spacing=0.1e-6, seed=2)
    with pytest.raises(WavePOError, match="INVALID_ARGUMENT"):
        api.height_field_points(hf, 10, 5)
    with pytest.raises(WavePOError, match="INVALID_ARGUMENT"):
        api.height_field_points(hf, 0, hf.numel)
    bad = geometry.HeightField(hf.xy.copy(), hf.period, hf.unitz)
    bad.xy[:, 5, 3] = 0.0
    with pytest.raises(WavePOError, match="origin"):
        api.height_field_points(bad)
    api.height_field_points(bad, 20, 40)  # the zero vertex lies outside this segment


# ------------------------------------------------------- pattern averaging
@pytest.mark.parametrize("name", ["ref_average_leftover", "ref_average_even", "ref_average_ragged"])
def test_average_vs_reference_build(cases, name):
    c = cases[name]
    inp = np.fromfile(GOLDEN / c["input"], dtype=np.float32).reshape(c["src"])
    out = api.average_pattern(inp, *c["dst"]).cpu().numpy()
    ref = np.fromfile(GOLDEN / f"{name}.bin", dtype=np.float32).reshape(c["dst"])
    assert np.array_equal(bits(out), bits(ref))


def test_average_batched_fiber_preset_vs_oracle():
    """450 x 880 -> 180 x 360 (the fiber preset), three patterns in one launch."""
    rng = np.random.default_rng(9)
    p = rng.exponential(1.0, (3, 450, 880)).astype(np.float32)
    out = api.average_pattern(p, 180, 360).cpu().numpy()
    for b in range(3):
        assert np.array_equal(bits(out[b]), bits(oracle.average(p[b], 180, 360)))
    with pytest.raises(WavePOError, match="INVALID_ARGUMENT"):
        api.average_pattern(p[0], 451, 360)
