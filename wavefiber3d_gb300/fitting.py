"""GPU statistics of rough-fiber pattern ensembles (the fitting side).

Mirrors fitting/fittingutil.py, the helpers the fitting notebook
(fitting/fitnoise.ipynb) applies to noise patterns of many rough-fiber
instances, on the engine's device kernels (po_shifted_fft2,
po_acf_from_patterns).  Arrays use the reference's layouts: noise fields are
[theta][phi][instance] (and [..][band] for the raw band fields); results are
torch tensors on the GPU.

* forward_fft_shifted(A)                     fittingutil.py:22-33
* inverse_fft_shifted(A)                     fittingutil.py:35-46
* weightedsum(noiserawmat, weight)           fittingutil.py:55-65
* acf_from_ft(noisemat)                      fittingutil.py:67-74
* acf_weighted_ft(Fnoiseaveragemat, weight)  fittingutil.py:48-53
"""
from __future__ import annotations

import numpy as np

from . import _lib, api


def _torch():
    import torch
    return torch


def _shifted(a, inverse, stream):
    torch = _torch()
    x = api._dev(a).to(torch.complex64).contiguous()
    lead = x.shape[:-2]
    nth, nph = x.shape[-2:]
    b = int(np.prod(lead)) if lead else 1
    out = torch.empty_like(x)
    api.check(_lib.load().po_shifted_fft2(api._ptr(x), api._ptr(out), b, nth, nph, inverse,
                                          api._stream_ptr(stream)))
    return out


def forward_fft_shifted(a, stream=None):
    """Shifted unnormalised forward 2-D DFT of [..., n_theta, n_phi] arrays (complex64 result)."""
    return _shifted(a, 0, stream)


def inverse_fft_shifted(a, stream=None):
    """Shifted unnormalised backward 2-D DFT (FFTW_BACKWARD, no 1/n) of [..., n_theta, n_phi] arrays."""
    return _shifted(a, 1, stream)


def weightedsum(noiserawmat, weight):
    """(noisemat [theta][phi][inst], mean [theta][phi]) of band fields [theta][phi][inst][band]."""
    torch = _torch()
    raw = api._dev(noiserawmat, torch.float32)
    w = api._dev(np.asarray(weight, dtype=np.float32), torch.float32)
    noisemat = (raw * w).sum(dim=-1)
    return noisemat, noisemat.mean(dim=-1)


def acf_from_ft(noisemat, stream=None):
    """(Fnoiseaverage, acf, mean) of noise fields [theta][phi][inst]: the mean |shifted
    FFT| of the centred instances and the real part of the shifted FFT of its square."""
    torch = _torch()
    x = api._dev(noisemat, torch.float32)
    nth, nph, ni = x.shape
    inst = x.permute(2, 0, 1).contiguous()  # [inst][theta][phi]
    mean = torch.empty((nth, nph), dtype=torch.float32, device="cuda")
    spec = torch.empty_like(mean)
    acf = torch.empty_like(mean)
    api.check(_lib.load().po_acf_from_patterns(api._ptr(inst), ni, nth, nph, api._ptr(mean), api._ptr(spec),
                                               api._ptr(acf), api._stream_ptr(stream)))
    return spec, acf, mean


def acf_weighted_ft(fnoiseaveragemat, weight):
    """(weightedFT, acf): sum_b w_b^2 F_b^2 over bands [theta][phi][band] and Re of its shifted FFT."""
    torch = _torch()
    f = api._dev(fnoiseaveragemat, torch.float32)
    w = api._dev(np.asarray(weight, dtype=np.float32), torch.float32)
    wft = (w * w * f * f).sum(dim=-1)
    return wft, forward_fft_shifted(wft).real.contiguous()
