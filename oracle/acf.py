"""numpy restatement of fitting/fittingutil.py:22-74 (test infrastructure).

The reference runs these with pyfftw (FFTW plans, absent here); FFTW's forward
transform is the unnormalised DFT exp(-2 pi i jk/n), which numpy.fft.fft2
computes too, so numpy stands in for it.  `shifted_dft_direct` evaluates the
definition term by term (small sizes) and pins the numpy form."""
import numpy as np


def forward_fft_shifted(a):
    """fittingutil.py:22-33."""
    a = np.asarray(a)
    s = np.floor(np.array(a.shape[-2:]) / 2).astype(int)
    a = np.roll(a, tuple(s), axis=(-2, -1))
    r = np.fft.fft2(a, axes=(-2, -1))
    return np.roll(r, tuple(-s), axis=(-2, -1))


def inverse_fft_shifted(a):
    """fittingutil.py:35-46 (FFTW_BACKWARD is unnormalised: n * numpy's ifft2)."""
    a = np.asarray(a)
    s = np.floor(np.array(a.shape[-2:]) / 2).astype(int)
    a = np.roll(a, tuple(-s), axis=(-2, -1))
    n = a.shape[-2] * a.shape[-1]
    r = np.fft.ifft2(a, axes=(-2, -1)) * n
    return np.roll(r, tuple(s), axis=(-2, -1))


def shifted_idft_direct(a):
    """The inverse transform as a direct double sum."""
    a = np.asarray(a, dtype=np.complex128)
    n0, n1 = a.shape
    s0, s1 = n0 // 2, n1 // 2
    k0 = np.arange(n0)
    k1 = np.arange(n1)
    w0 = np.exp(2j * np.pi * np.outer((k0 - s0) % n0, (k0 - s0) % n0) / n0)
    w1 = np.exp(2j * np.pi * np.outer((k1 - s1) % n1, (k1 - s1) % n1) / n1)
    return w0 @ a @ w1.T


def shifted_dft_direct(a):
    """The same transform as a direct double sum."""
    a = np.asarray(a, dtype=np.complex128)
    n0, n1 = a.shape
    s0, s1 = n0 // 2, n1 // 2
    k0 = np.arange(n0)
    k1 = np.arange(n1)
    w0 = np.exp(-2j * np.pi * np.outer((k0 + s0) % n0, (k0 + s0) % n0) / n0)
    w1 = np.exp(-2j * np.pi * np.outer((k1 + s1) % n1, (k1 + s1) % n1) / n1)
    return w0 @ a @ w1.T


def weightedsum(noiserawmat, weight):
    """fittingutil.py:55-65: noisemat[:,:,i] = sum_b w_b raw[:,:,i,b], mean over i."""
    raw = np.asarray(noiserawmat, dtype=np.float64)
    noisemat = np.einsum("tpib,b->tpi", raw, np.asarray(weight, dtype=np.float64))
    return noisemat, noisemat.mean(axis=2)


def acf_from_ft(noisemat, mean):
    """fittingutil.py:67-74."""
    ni = noisemat.shape[2]
    f = np.zeros(noisemat.shape[:2])
    for i in range(ni):
        f = f + np.abs(forward_fft_shifted(noisemat[:, :, i] - mean)) / ni
    return f, np.real(forward_fft_shifted(f ** 2))


def acf_weighted_ft(fnoiseaveragemat, weight):
    """fittingutil.py:48-53."""
    w = np.asarray(weight, dtype=np.float64)
    wft = np.einsum("tpb,b->tp", np.asarray(fnoiseaveragemat, dtype=np.float64) ** 2, w * w)
    return wft, np.real(forward_fft_shifted(wft))
