"""Seeded test cases shared by the fixture generator and the tests."""
from __future__ import annotations

import numpy as np

from libheom_gb300.params import HeomParams


def _herm(rng, n, scale=1.0):
    m = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    return scale * (m + m.conj().T) / 2


def generic_case(seed=5) -> HeomParams:
    """Every coupling form the reference accepts: complex Hermitian H, a dense
    (non-diagonal) V and a diagonal complex V, nonzero s_delta, dense S and A,
    complex phi_0 / sigma, and off-diagonal gamma entries (which the reference
    ignores; heom.h:110)."""
    rng = np.random.default_rng(seed)
    n = 3
    H = _herm(rng, n)
    V0 = _herm(rng, n, 0.5)
    V1 = np.diag(rng.standard_normal(n) + 0.3j * rng.standard_normal(n))
    lens = [2, 1]
    gam, phi, sig, S, A = [], [], [], [], []
    for L in lens:
        g = np.diag(rng.uniform(0.5, 2.0, L) + 0.1j * rng.standard_normal(L)).astype(complex)
        if L > 1:
            g[0, 1] = 0.3 + 0.1j
        gam.append(g)
        phi.append(rng.standard_normal(L) + 1j * rng.standard_normal(L))
        sig.append(rng.standard_normal(L) + 1j * rng.standard_normal(L))
        S.append(rng.standard_normal((L, L)) + 1j * rng.standard_normal((L, L)))
        A.append(rng.standard_normal((L, L)) + 1j * rng.standard_normal((L, L)))
    return HeomParams(H=H, V=[V0, V1], gamma=gam, phi_0=phi, sigma=sig, S=[s * 0.3 for s in S],
                      A=[a * 0.3 for a in A], s_delta=[0.05 + 0.01j, 0.02], max_depth=3, name="generic")


def projector_case(seed=6, n=4, depth=3) -> HeomParams:
    """Site-local projector baths (the exciton-aggregate structure), 2 modes each, real H."""
    rng = np.random.default_rng(seed)
    H = rng.standard_normal((n, n))
    H = (H + H.T) / 2
    Vs, gam, phi, sig, S, A = [], [], [], [], [], []
    for j in range(n):
        V = np.zeros((n, n), complex)
        V[j, j] = 1
        Vs.append(V)
        nu = rng.uniform(0.5, 3.0, 2)
        c = rng.standard_normal(2) + 1j * rng.standard_normal(2)
        gam.append(np.diag(nu).astype(complex))
        phi.append(np.ones(2, complex))
        sig.append(np.ones(2, complex))
        S.append(np.diag(c.real).astype(complex) * 0.2)
        A.append(np.diag(c.imag).astype(complex) * 0.2)
    return HeomParams(H=H.astype(complex), V=Vs, gamma=gam, phi_0=phi, sigma=sig, S=S, A=A,
                      s_delta=[0.01 * (j + 1) for j in range(n)], max_depth=depth, name="projector")


def params_to_dict(p: HeomParams) -> dict:
    d = dict(H=p.H, V=np.array(p.V), s_delta=np.array(p.s_delta, complex), max_depth=np.array(p.max_depth),
             normalization=np.array(p.normalization), order=np.array(p.order))
    for u in range(p.n_noise):
        d[f"gamma_{u}"] = p.gamma[u]
        d[f"phi_0_{u}"] = p.phi_0[u]
        d[f"sigma_{u}"] = p.sigma[u]
        d[f"S_{u}"] = p.S[u]
        d[f"A_{u}"] = p.A[u]
    return d


def params_from_npz(z) -> HeomParams:
    V = list(z["V"])
    U = len(V)
    return HeomParams(H=z["H"], V=V, gamma=[z[f"gamma_{u}"] for u in range(U)],
                      phi_0=[z[f"phi_0_{u}"] for u in range(U)], sigma=[z[f"sigma_{u}"] for u in range(U)],
                      S=[z[f"S_{u}"] for u in range(U)], A=[z[f"A_{u}"] for u in range(U)],
                      s_delta=list(z["s_delta"]), max_depth=int(z["max_depth"]),
                      normalization=str(z["normalization"]) if "normalization" in z.files else "integer",
                      order=str(z["order"]) if "order" in z.files else "row_major")


# Hierarchy filters (alloc_hrchy_space's hrchy_filter, filter_flag on) used by
# the golden fixtures and the tests: name -> (n_dim, max_depth, filter).
def _weighted(idx, depth):
    w = [1, 2, 1, 3, 1, 2]
    return sum(a * b for a, b in zip(idx, w)) <= 5


FILTERS = {
    "weighted": (5, 4, _weighted),
    "cap0": (4, 6, lambda idx, depth: idx[0] <= 2 and depth <= 5),
    "nonmonotone": (6, 5, lambda idx, depth: idx[5] == 0 or idx[0] > 0),
}
