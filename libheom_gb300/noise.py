"""Exponential decomposition of a Drude-Lorentz bath, and unit conversion.

The reference library takes the decomposition as input (its Python front end,
which computes it, is a separate project).  This module restates the standard
high-temperature-series (Matsubara) expansion of the Drude-Lorentz correlation

    C(t) = sum_k c_k exp(-nu_k t),
    nu_0 = gamma_c,          c_0 = lambda*gamma_c*(cot(beta*gamma_c/2) - i),
    nu_m = 2*pi*m/beta,      c_m = 4*lambda*gamma_c*nu_m / (beta*(nu_m^2 - gamma_c^2)),

and maps it onto the reference's noise members (qme_base.h:32-67) so that the
hierarchy reproduces  -i[V, rho_{n+1_k}] - i n_k (c_k V rho_{n-1_k} - c_k^* rho_{n-1_k} V)
through heom_hilb.h:171-208:  gamma = diag(nu), phi_0 = sigma = 1,
S = diag(Re c), A = diag(Im c), s_delta = 0.
Units: hbar = 1; energies and rates share one unit.
"""
from __future__ import annotations

import math

import numpy as np

# 1 cm^-1 expressed as an angular frequency in rad/fs: 2*pi*c with c in cm/fs.
CM1_TO_RAD_PER_FS = 2.0 * math.pi * 2.99792458e-5
# Boltzmann constant in cm^-1 per kelvin.
KB_CM1_PER_K = 0.69503476


def drude_lorentz_terms(lam: float, gamma_c: float, beta: float, n_matsubara: int):
    """Return (nu, c) arrays: 1 Drude term + n_matsubara Matsubara terms."""
    nu = [gamma_c]
    c = [lam * gamma_c * (1.0 / math.tan(beta * gamma_c / 2.0) - 1j)]
    for m in range(1, n_matsubara + 1):
        nu_m = 2.0 * math.pi * m / beta
        nu.append(nu_m)
        c.append(4.0 * lam * gamma_c * nu_m / (beta * (nu_m * nu_m - gamma_c * gamma_c)) + 0j)
    return np.array(nu, dtype=np.complex128), np.array(c, dtype=np.complex128)


def noise_members(nu: np.ndarray, c: np.ndarray):
    """Map (nu_k, c_k) to the reference's (gamma, phi_0, sigma, S, A, s_delta)."""
    k = len(nu)
    gamma = np.diag(np.asarray(nu, dtype=np.complex128))
    phi_0 = np.ones(k, dtype=np.complex128)
    sigma = np.ones(k, dtype=np.complex128)
    S = np.diag(np.real(c).astype(np.complex128))
    A = np.diag(np.imag(c).astype(np.complex128))
    return gamma, phi_0, sigma, S, A, 0j
