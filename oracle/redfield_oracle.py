"""Test infrastructure: numpy restatement of libheom's Redfield models.

THE ORACLE, NOT THE PRODUCT: tests use it beside the golden fixtures that the
reference's own redfield_hilb / redfield_liou (built by oracle/Makefile) wrote.

* Set-up (redfield.h:42-173): eigen-decomposition H = U diag(w) U^dagger; per
  bath u, C_u = S_u + i A_u, the correlation
  corr(omega) = sigma_u^T C_u (gamma_u - i omega)^-1 phi_0 + s_delta_u
  (redfield.h:32-41, the full gamma matrix), and
  Lambda_u = U [ (U^dagger V_u U)_ij corr(w_j - w_i) ] U^dagger.
* Right-hand side (redfield_hilb.h:66-89): drho = beta drho - alpha D with
  D = i[H, rho] + sum_u [V_u, Lambda_u rho - rho Lambda_u^dagger].
"""
from __future__ import annotations

import numpy as np


def lambdas(p):
    w, U = np.linalg.eigh(p.H)
    out = []
    for u in range(p.n_noise):
        C = p.S[u] + 1j * p.A[u]
        stc = p.sigma[u] @ C
        Vv = U.conj().T @ p.V[u] @ U
        L = np.empty_like(Vv)
        K = len(p.sigma[u])
        for i in range(len(w)):
            for j in range(len(w)):
                x = np.linalg.solve(p.gamma[u] - 1j * (w[j] - w[i]) * np.eye(K), p.phi_0[u])
                L[i, j] = Vv[i, j] * (stc @ x + p.s_delta[u])
        out.append(U @ L @ U.conj().T)
    return out


def calc_diff(p, rho, drho=None, alpha=1.0, beta=0.0):
    """rho, drho: (n, n) or (1, n, n)."""
    r = np.asarray(rho).reshape(p.n_level, p.n_level)
    D = 1j * (p.H @ r - r @ p.H)
    for u, lam in enumerate(lambdas(p)):
        T = lam @ r - r @ lam.conj().T
        D = D + p.V[u] @ T - T @ p.V[u]
    out = -alpha * D
    if drho is not None and beta != 0:
        out = out + beta * np.asarray(drho).reshape(p.n_level, p.n_level)
    return out.reshape(np.shape(rho))
