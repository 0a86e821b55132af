"""Mie series for a homogeneous sphere -- analytic sanity check of the PO path.

TEST INFRASTRUCTURE ONLY.  Own implementation of the Bohren & Huffman
formulation ("Absorption and Scattering of Light by Small Particles", 1983,
sec. 4.4 and appendix A): Riccati-Bessel functions by upward recurrence,
the logarithmic derivative D_n(mx) by downward recurrence, angular functions
pi_n / tau_n by their three-term recurrences.  The reference compares its PO
sphere against PyMieScatt (compareMie/mie.ipynb, cell 4); this module stands
in for that library, which is not installed here.
"""
from __future__ import annotations

import math

import numpy as np


def mie_coefficients(x: float, m: complex):
    """a_n, b_n for n = 1..nstop (size parameter x, relative index m)."""
    nstop = int(x + 4.0 * x ** (1.0 / 3.0) + 2.0)
    mx = m * x
    nmx = int(max(nstop, abs(mx)) + 16)
    d = np.zeros(nmx + 1, dtype=np.complex128)
    for n in range(nmx, 0, -1):
        d[n - 1] = n / mx - 1.0 / (d[n] + n / mx)
    psi_m1, psi_0 = math.cos(x), math.sin(x)
    chi_m1, chi_0 = -math.sin(x), math.cos(x)
    xi_0 = complex(psi_0, -chi_0)
    a = np.zeros(nstop, dtype=np.complex128)
    b = np.zeros(nstop, dtype=np.complex128)
    for n in range(1, nstop + 1):
        psi = (2.0 * n - 1.0) / x * psi_0 - psi_m1
        chi = (2.0 * n - 1.0) / x * chi_0 - chi_m1
        xi = complex(psi, -chi)
        ta = d[n] / m + n / x
        tb = d[n] * m + n / x
        a[n - 1] = (ta * psi - psi_0) / (ta * xi - xi_0)
        b[n - 1] = (tb * psi - psi_0) / (tb * xi - xi_0)
        psi_m1, psi_0 = psi_0, psi
        chi_m1, chi_0 = chi_0, chi
        xi_0 = complex(psi_0, -chi_0)
    return a, b


def amplitudes(x: float, m: complex, scatter_angle: np.ndarray):
    """S1, S2 at scattering angles (radians from the forward direction)."""
    a, b = mie_coefficients(x, m)
    mu = np.cos(np.asarray(scatter_angle, dtype=np.float64))
    s1 = np.zeros(mu.shape, dtype=np.complex128)
    s2 = np.zeros(mu.shape, dtype=np.complex128)
    pi_m1 = np.zeros_like(mu)
    pi_0 = np.ones_like(mu)
    for n in range(1, a.size + 1):
        tau = n * mu * pi_0 - (n + 1) * pi_m1
        f = (2.0 * n + 1.0) / (n * (n + 1.0))
        s1 += f * (a[n - 1] * pi_0 + b[n - 1] * tau)
        s2 += f * (a[n - 1] * tau + b[n - 1] * pi_0)
        pi_next = ((2.0 * n + 1.0) * mu * pi_0 - (n + 1.0) * pi_m1) / n
        pi_m1, pi_0 = pi_0, pi_next
    return s1, s2


def polarised_intensity(radius: float, wavelength: float, m: complex, khat, ehat, s: np.ndarray):
    """Relative far-field intensity |S2|^2 cos^2(psi) + |S1|^2 sin^2(psi) for an
    incident plane wave along `khat` polarised along `ehat`, observed along the
    unit vectors s (..., 3); psi is the azimuth of s about khat measured from ehat."""
    khat = np.asarray(khat, dtype=np.float64)
    ehat = np.asarray(ehat, dtype=np.float64)
    hhat = np.cross(khat, ehat)
    s = np.asarray(s, dtype=np.float64)
    ct = np.clip(s @ khat, -1.0, 1.0)
    ang = np.arccos(ct)
    s1, s2 = amplitudes(2.0 * math.pi * radius / wavelength, m, ang)
    pe, ph = s @ ehat, s @ hhat
    r = np.hypot(pe, ph)
    cos2 = np.where(r > 0, (pe / np.where(r > 0, r, 1.0)) ** 2, 1.0)
    return np.abs(s2) ** 2 * cos2 + np.abs(s1) ** 2 * (1.0 - cos2)
