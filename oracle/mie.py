"""Mie-series known answers -- TEST INFRASTRUCTURE ONLY.

* :func:`pec_backscatter` restates ``analysis/sphereRCSvsFreq.m:3-31``: the
  monostatic RCS of a perfectly conducting sphere from half-integer-order
  Bessel/Hankel functions (100 orders, c = 3e8).
* :func:`sphere_backscatter` is the Mie series of a homogeneous sphere of
  relative permittivity ``eps_r`` (complex; a cold collisional plasma has
  eps_r = 1 - wp^2 / (w (w + i nu)) in the exp(-i w t) convention), written
  from the standard coefficients a_n, b_n (Bohren & Huffman, eq. 4.53) with
  Riccati-Bessel functions; the reference has no such routine.  Backscatter:
  sigma = (pi a^2 / x^2) |sum_n (2n+1) (-1)^n (a_n - b_n)|^2.
"""
from __future__ import annotations

import math

import numpy as np
from scipy import special as sp

C_MIE = 3e8


def pec_backscatter(f, radius: float, iterations: int = 100) -> np.ndarray:
    """analysis/sphereRCSvsFreq.m: conducting-sphere backscatter RCS (m^2)."""
    f = np.atleast_1d(np.asarray(f, dtype=np.float64))
    rcs = np.zeros_like(f)
    n = np.arange(1, iterations + 1)
    for q, freq in enumerate(f):
        lam = C_MIE / freq
        ka = 2 * math.pi * radius / lam
        s = math.sqrt(math.pi / 2 / ka)
        B1 = sp.jv(n + 0.5, ka)
        B2 = sp.hankel2(n + 0.5, ka)
        B3 = sp.jv(n + 0.5 - 1, ka)
        B4 = sp.hankel2(n + 0.5 - 1, ka)
        a = (s * B1) / (s * B2)
        b = (ka * s * B3 - n * s * B1) / (ka * s * B4 - n * s * B2)
        rcs[q] = (lam ** 2 / math.pi) * abs(np.sum((-1.0) ** n * (n + 0.5) * (b - a))) ** 2
    return rcs


def sphere_coefficients(x: float, m: complex, nmax: int = None):
    """Mie a_n, b_n for size parameter x = k a and relative index m, with the
    logarithmic derivative D_n(mx) from downward recurrence (stable for
    lossy and negative-permittivity spheres); m = inf gives the perfect
    conductor (a_n = psi_n'/xi_n', b_n = psi_n/xi_n)."""
    if nmax is None:
        nmax = int(x + 4 * x ** (1 / 3) + 2) + 2
    n = np.arange(1, nmax + 1)
    nn = np.arange(0, nmax + 1)
    jn = sp.spherical_jn(nn, x)
    yn = sp.spherical_yn(nn, x)
    psi = x * jn                       # psi_0..psi_nmax
    xi = x * (jn + 1j * yn)            # xi_n = x h1_n(x)
    if np.isinf(m):
        dpsi = psi[:-1] - n * psi[1:] / x      # psi_n' = psi_{n-1} - n psi_n / x
        dxi = xi[:-1] - n * xi[1:] / x
        return n, dpsi / dxi, psi[1:] / xi[1:]
    mx = m * x
    nstart = int(max(nmax, abs(mx))) + 16
    D = np.zeros(nstart + 1, dtype=complex)
    for q in range(nstart, 0, -1):
        D[q - 1] = q / mx - 1.0 / (D[q] + q / mx)
    Dn = D[1:nmax + 1]
    ta = Dn / m + n / x
    tb = m * Dn + n / x
    a = (ta * psi[1:] - psi[:-1]) / (ta * xi[1:] - xi[:-1])
    b = (tb * psi[1:] - psi[:-1]) / (tb * xi[1:] - xi[:-1])
    return n, a, b


def sphere_backscatter(f, radius: float, eps_r) -> np.ndarray:
    """Monostatic RCS (m^2) of a homogeneous sphere, relative permittivity eps_r
    (scalar or per-frequency array)."""
    f = np.atleast_1d(np.asarray(f, dtype=np.float64))
    eps = np.broadcast_to(np.asarray(eps_r, dtype=complex), f.shape) if not np.isinf(eps_r).all() else np.full(f.shape, np.inf)
    out = np.zeros_like(f)
    for q, freq in enumerate(f):
        k = 2 * math.pi * freq / C_MIE
        x = k * radius
        m = np.inf if np.isinf(eps[q]) else np.sqrt(eps[q])
        if not np.isinf(m) and m.imag < 0:
            m = -m
        n, a, b = sphere_coefficients(x, m)
        s = np.sum((2 * n + 1) * (-1.0) ** n * (a - b))
        out[q] = math.pi * radius ** 2 / x ** 2 * abs(s) ** 2
    return out


def plasma_eps(f, wp: float, nu: float):
    """Cold collisional plasma permittivity, exp(-i w t) convention."""
    w = 2 * math.pi * np.asarray(f, dtype=np.float64)
    return 1 - wp ** 2 / (w * (w + 1j * nu))
