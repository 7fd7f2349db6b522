"""Mie series for a perfectly conducting sphere — test infrastructure only.

The exact bistatic radar cross-section of a PEC sphere of radius a under a
plane wave, the analytic check the method's RCS (modRCS.f90:339-432 restated
in oracle/mlfma_oracle.c) is compared against.  Nothing here is part of the
product.

Series (exp(+j w t) time convention folded away: only |S|^2 enters sigma):
    x = k a,   h_n = j_n + j y_n   (spherical Hankel, first kind)
    a_n = [x j_n(x)]' / [x h_n(x)]',     b_n = j_n(x) / h_n(x)
    pi_n(u) = P_n^1(u) / sin(theta),     tau_n(u) = d P_n^1(cos theta) / d theta
    S1 = sum_n (2n+1)/(n(n+1)) (a_n pi_n + b_n tau_n)
    S2 = sum_n (2n+1)/(n(n+1)) (a_n tau_n + b_n pi_n)
Incidence along +z with the electric field along +x; theta is measured from
+z (theta = 0 is forward scattering) and phi from +x:
    sigma(theta, phi) = (4 pi / k^2) (cos^2 phi |S2|^2 + sin^2 phi |S1|^2).
Backscatter reduces to (pi / k^2) |sum_n (-1)^n (2n+1) (a_n - b_n)|^2, which
tends to pi a^2 for large spheres.
"""
from __future__ import annotations

import numpy as np
from scipy.special import spherical_jn, spherical_yn


def _coefficients(x: float, nmax: int):
    n = np.arange(1, nmax + 1)
    jn = spherical_jn(n, x)
    yn = spherical_yn(n, x)
    jnp = spherical_jn(n, x, derivative=True)
    ynp = spherical_yn(n, x, derivative=True)
    hn = jn + 1j * yn
    hnp = jnp + 1j * ynp
    a = (jn + x * jnp) / (hn + x * hnp)     # [x j_n]' / [x h_n]'
    b = jn / hn
    return n, a, b


def _angular(nmax: int, theta: np.ndarray):
    """pi_n and tau_n by the upward recurrences (Bohren & Huffman 4.47)."""
    u = np.cos(theta)
    pi = np.zeros((nmax + 1, theta.size))
    tau = np.zeros((nmax + 1, theta.size))
    pi[1] = 1.0
    tau[1] = u
    for n in range(2, nmax + 1):
        pi[n] = ((2 * n - 1) * u * pi[n - 1] - n * pi[n - 2]) / (n - 1)
        tau[n] = n * u * pi[n] - (n + 1) * pi[n - 1]
    return pi[1:], tau[1:]


def sphere_rcs(radius: float, lam: float, theta, phi) -> np.ndarray:
    """Bistatic RCS (m^2, not dB) of a PEC sphere; theta, phi in radians,
    broadcast together."""
    theta, phi = np.broadcast_arrays(np.asarray(theta, float), np.asarray(phi, float))
    k = 2 * np.pi / lam
    x = k * radius
    nmax = int(np.ceil(x + 4.05 * x ** (1 / 3) + 8))     # Wiscombe's criterion
    n, a, b = _coefficients(x, nmax)
    pi, tau = _angular(nmax, theta.ravel())
    f = ((2 * n + 1) / (n * (n + 1)))[:, None]
    S1 = np.sum(f * (a[:, None] * pi + b[:, None] * tau), axis=0)
    S2 = np.sum(f * (a[:, None] * tau + b[:, None] * pi), axis=0)
    ph = phi.ravel()
    sig = 4 * np.pi / k ** 2 * (np.cos(ph) ** 2 * np.abs(S2) ** 2 + np.sin(ph) ** 2 * np.abs(S1) ** 2)
    return sig.reshape(theta.shape)


def sphere_backscatter(radius: float, lam: float) -> float:
    k = 2 * np.pi / lam
    x = k * radius
    nmax = int(np.ceil(x + 4.05 * x ** (1 / 3) + 8))
    n, a, b = _coefficients(x, nmax)
    s = np.sum((-1.0) ** n * (2 * n + 1) * (a - b))
    return float(np.pi / k ** 2 * abs(s) ** 2)
