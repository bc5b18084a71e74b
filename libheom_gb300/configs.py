"""Seeded synthetic workloads (the shapes the engine is measured on).

* ``spin_boson``      n=2, one Drude-Lorentz bath (1 Drude + 2 Matsubara terms,
                      K=3), depth 10 -> 286 ADOs; RK4 dt=0.005 x 2000 steps.
* ``exciton_7site``   n=7, seed 1; 7 site-local baths (1 Drude + 1 Matsubara each,
                      K=14), depth 4 -> 3060 ADOs; Dormand-Prince to 1 ps.
* ``aggregate_24site`` n=24, seed 3; 24 site-local baths x 2 modes (K=48),
                      depth 3 -> 20825 ADOs; LSRK4 x 2000 steps.
* ``batched_sweep``   1024 uneven spin-boson / 4-level-chain instances, seed 2.

Energies in cm^-1 are converted to rad/fs and times are in fs (hbar = 1).
Choices the workload descriptions leave open are fixed here and documented:
the 7-site run uses rtol = 1e-8 and an initial step of 0.1 fs; the 24-site run
uses dt = 0.5 fs (2000 steps = 1 ps) and the 7-site bath parameters; the chains
of the batched sweep couple site 0 to one bath of 2 modes (1 Drude + 1 Matsubara).
"""
from __future__ import annotations

import math

import numpy as np

from .noise import CM1_TO_RAD_PER_FS, KB_CM1_PER_K, drude_lorentz_terms, noise_members
from .params import HeomParams


def spin_boson(eps=0.0, delta=1.0, lam=0.5, gamma_c=1.0, beta=1.0, n_matsubara=2, depth=10,
               coupling="z") -> HeomParams:
    H = np.array([[eps / 2, delta], [delta, -eps / 2]], dtype=np.complex128)
    if coupling == "z":
        V = np.array([[1, 0], [0, -1]], dtype=np.complex128)
    elif coupling == "x":
        V = np.array([[0, 1], [1, 0]], dtype=np.complex128)
    else:
        raise ValueError(coupling)
    nu, c = drude_lorentz_terms(lam, gamma_c, beta, n_matsubara)
    g, p, s, S, A, sd = noise_members(nu, c)
    return HeomParams(H=H, V=[V], gamma=[g], phi_0=[p], sigma=[s], S=[S], A=[A], s_delta=[sd],
                      max_depth=depth, name="spin_boson",
                      meta=dict(solver="rk4", dt=0.005, n_steps=2000))


def _site_bath(lam_cm, gamma_c_fs, temp_k, n_matsubara):
    lam = lam_cm * CM1_TO_RAD_PER_FS
    beta = 1.0 / (KB_CM1_PER_K * temp_k * CM1_TO_RAD_PER_FS)
    return drude_lorentz_terms(lam, gamma_c_fs, beta, n_matsubara)


def _aggregate(n, eps, J, lam_cm, gamma_c_fs, temp_k, n_matsubara, depth, name, meta):
    H = (np.diag(eps) + J) * CM1_TO_RAD_PER_FS
    nu, c = _site_bath(lam_cm, gamma_c_fs, temp_k, n_matsubara)
    g, p, s, S, A, sd = noise_members(nu, c)
    Vs = []
    for j in range(n):
        V = np.zeros((n, n), dtype=np.complex128)
        V[j, j] = 1.0
        Vs.append(V)
    U = n
    return HeomParams(H=H.astype(np.complex128), V=Vs, gamma=[g] * U, phi_0=[p] * U, sigma=[s] * U,
                      S=[S] * U, A=[A] * U, s_delta=[sd] * U, max_depth=depth, name=name, meta=meta)


def exciton_7site(seed=1, depth=4, lam_cm=35.0, temp_k=300.0, gamma_c_fs=1.0 / 50.0) -> HeomParams:
    """The 7-site aggregate; lam_cm, temp_k and gamma_c_fs vary the baths
    (the defaults are the measured workload's)."""
    rng = np.random.default_rng(seed)
    n = 7
    eps = rng.normal(0.0, 100.0, n)
    J = rng.uniform(-100.0, 100.0, (n, n))
    J = np.triu(J, 1)
    J = J + J.T
    return _aggregate(n, eps, J, lam_cm, gamma_c_fs, temp_k, 1, depth, "exciton_7site",
                      dict(solver="rkdp", dt=0.1, atol=1e-8, rtol=1e-8, t_final=1000.0))


def aggregate_24site(seed=3, depth=3, n_sites=24) -> HeomParams:
    """Random aggregate (24 sites unless n_sites says otherwise)."""
    rng = np.random.default_rng(seed)
    n = n_sites
    eps = rng.normal(0.0, 200.0, n)
    J = rng.uniform(-50.0, 50.0, (n, n))
    J = np.triu(J, 1)
    J = J + J.T
    return _aggregate(n, eps, J, 35.0, 1.0 / 50.0, 300.0, 1, depth, "aggregate_24site",
                      dict(solver="lsrk4", dt=0.5, n_steps=2000))


def chain_4level(J, eps, depth, lam=0.5, gamma_c=1.0, beta=1.0) -> HeomParams:
    n = 4
    H = np.diag(eps).astype(np.complex128)
    for i in range(n - 1):
        H[i, i + 1] = H[i + 1, i] = J[i]
    V = np.zeros((n, n), dtype=np.complex128)
    V[0, 0] = 1.0
    nu, c = drude_lorentz_terms(lam, gamma_c, beta, 1)
    g, p, s, S, A, sd = noise_members(nu, c)
    return HeomParams(H=H, V=[V], gamma=[g], phi_0=[p], sigma=[s], S=[S], A=[A], s_delta=[sd],
                      max_depth=depth, name="chain_4level")


def batched_sweep(seed=2, n_spin_boson=768, n_chain=256):
    """Instances of the batched sweep: uneven n_state (2 or 4) and depth."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_spin_boson):
        lam = math.exp(rng.uniform(math.log(0.05), math.log(5.0)))
        beta = rng.uniform(0.1, 10.0)
        eps = rng.uniform(-2.0, 2.0)
        depth = int(rng.integers(4, 15))
        out.append(spin_boson(eps=eps, delta=1.0, lam=lam, gamma_c=1.0, beta=beta, n_matsubara=2,
                              depth=depth))
    for _ in range(n_chain):
        J = rng.uniform(-1.0, 1.0, 3)
        eps = rng.normal(0.0, 1.0, 4)
        depth = int(rng.integers(4, 9))
        out.append(chain_4level(J, eps, depth))
    return out


def exciton_7site_ensemble(seed=1, count=16, depth=4):
    """Static-disorder ensemble of the 7-site aggregate: `count` seeded
    Hamiltonians (seeds seed .. seed+count-1), the same baths."""
    return [exciton_7site(seed=seed + i, depth=depth) for i in range(count)]
