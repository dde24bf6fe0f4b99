"""Analytic bistatic RCS of a PEC sphere (the Mie series) -- TEST
INFRASTRUCTURE, NOT PRODUCT CODE.

An independent check of the discretised solvers: the exact far field of a
perfectly conducting sphere under a plane wave, from the published series
(Bohren & Huffman, "Absorption and Scattering of Light by Small Particles",
section 4.4, with the perfect-conductor limit of the coefficients):

    a_n = psi_n'(x) / xi_n'(x),   b_n = psi_n(x) / xi_n(x),   x = k a
    S1(T) = sum_n (2n+1)/(n(n+1)) [a_n pi_n(cos T) + b_n tau_n(cos T)]
    S2(T) = sum_n (2n+1)/(n(n+1)) [a_n tau_n(cos T) + b_n pi_n(cos T)]

with psi_n(x) = x j_n(x), xi_n(x) = x h_n(x), pi_n/tau_n the angular
functions by their upward recurrence, T the scattering angle (0 = forward)
and the sum to n = x + 4 x^(1/3) + 2.  A point at azimuth p from the plane
that holds the incident polarisation sees

    sigma = (lambda^2 / pi) (cos^2 p |S2(T)|^2 + sin^2 p |S1(T)|^2).

The reference's conventions (EMSolver/EM.cpp:33-34): the incident wave
travels along k_hat = -r_hat(theta, phi) with polarisation e_hat; RCS
directions are observation directions r_hat.
"""
from __future__ import annotations

import numpy as np
from scipy import special


def _coefficients(x: float):
    nmax = int(np.ceil(x + 4.0 * x ** (1.0 / 3.0) + 2.0))
    n = np.arange(1, nmax + 1)
    jn = special.spherical_jn(n, x)
    jnp = special.spherical_jn(n, x, derivative=True)
    yn = special.spherical_yn(n, x)
    ynp = special.spherical_yn(n, x, derivative=True)
    psi = x * jn
    psip = jn + x * jnp
    xi = x * (jn + 1j * yn)
    xip = (jn + 1j * yn) + x * (jnp + 1j * ynp)
    return n, psip / xip, psi / xi


def _angular(nmax: int, mu: np.ndarray):
    pi = np.zeros((nmax + 1,) + mu.shape)
    tau = np.zeros_like(pi)
    pi[1] = 1.0
    tau[1] = mu
    for n in range(2, nmax + 1):
        pi[n] = ((2 * n - 1) * mu * pi[n - 1] - n * pi[n - 2]) / (n - 1)
        tau[n] = n * mu * pi[n] - (n + 1) * pi[n - 1]
    return pi[1:], tau[1:]


def pec_sphere_rcs_db(radius: float, freq: float, k_inc, e_inc, dirs) -> np.ndarray:
    """Bistatic RCS in dBsm of a PEC sphere of the given radius for an
    incident plane wave travelling along unit k_inc with unit polarisation
    e_inc, at observation directions dirs (M x 3)."""
    lam = 299792458.0 / freq
    x = 2.0 * np.pi / lam * radius
    k_inc = np.asarray(k_inc, dtype=np.float64)
    e_inc = np.asarray(e_inc, dtype=np.float64)
    d = np.asarray(dirs, dtype=np.float64).reshape(-1, 3)
    d = d / np.linalg.norm(d, axis=1, keepdims=True)
    mu = np.clip(d @ k_inc, -1.0, 1.0)  # cos of the scattering angle (1 = forward)
    n, a, b = _coefficients(x)
    pi, tau = _angular(int(n[-1]), mu)
    w = ((2 * n + 1) / (n * (n + 1)))[:, None]
    S1 = np.sum(w * (a[:, None] * pi + b[:, None] * tau), axis=0)
    S2 = np.sum(w * (a[:, None] * tau + b[:, None] * pi), axis=0)
    # azimuth from the polarisation plane: components of the observation
    # direction across k_inc along e_inc and along k_inc x e_inc
    h_inc = np.cross(k_inc, e_inc)
    ce, ch = d @ e_inc, d @ h_inc
    rho = np.hypot(ce, ch)
    cos2 = np.where(rho > 1e-12, (ce / np.where(rho > 0, rho, 1.0)) ** 2, 1.0)
    sigma = lam ** 2 / np.pi * (cos2 * np.abs(S2) ** 2 + (1.0 - cos2) * np.abs(S1) ** 2)
    return 10.0 * np.log10(sigma)
