"""po_interp_fft_noalloc: the interpolation for callers that must not allocate
device memory (its scratch is a fixed device array inside the library).

Checked through the C ABI against po_interp_fft on two calls in a row with
different inputs and sizes, so that a stale scratch from the first call would
show up in the second.  Kept in its own file, collected last."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from wavefiber3d_gb300 import _lib, api  # noqa: E402

TOL = 1e-5  # the FP32 tolerance of the other interpolation tests


def _noalloc(z, th_p, ph_p, theta_mode, quirk):
    L = _lib.load()
    z = z.cuda().contiguous()
    b, th_c, ph_c = z.shape
    out = torch.empty((b, th_p, ph_p), dtype=torch.complex64, device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(L.po_interp_fft_noalloc(ctypes.c_void_p(z.data_ptr()), th_c, ph_c, ctypes.c_void_p(out.data_ptr()),
                                       th_p, ph_p, b, theta_mode, 1 if quirk else 0, st))
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_noalloc_matches_allocating_entry_point_twice():
    rng = np.random.default_rng(42)
    calls = [((3, 20, 30), (33, 300), api.PO_THETA_REFERENCE, True),
             ((5, 24, 37), (48, 62), api.PO_THETA_DOUBLE_COVER, False)]
    for shape, (th_p, ph_p), mode, quirk in calls:
        z = torch.from_numpy((rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64))
        got = _noalloc(z, th_p, ph_p, mode, quirk)
        want = api.copyandinterp(z, th_p, ph_p, mode, quirk).cpu().numpy()
        assert _rel(got, want) < TOL


def test_noalloc_rejects_requests_beyond_its_scratch():
    L = _lib.load()
    z = torch.zeros((1, 8, 8), dtype=torch.complex64, device="cuda")
    out = torch.zeros(1, dtype=torch.complex64, device="cuda")
    # 64 * 1024 * 8192 complex64 = 512 MiB of row-pass scratch, far above the fixed array
    rc = L.po_interp_fft_noalloc(ctypes.c_void_p(z.data_ptr()), 1024, 8, ctypes.c_void_p(out.data_ptr()), 1024,
                                 8192, 64, api.PO_THETA_REFERENCE, 1, None)
    assert rc == 1 and b"scratch" in L.po_last_error()
