"""Parameter set of one HEOM instance.

The fields are the public parameter members a libheom caller fills before
``set_param`` (``include/qme_base.h:32-67``; depth from ``include/heom.h:44-50``):
system Hamiltonian ``H``, and per bath ``u`` the coupling operator ``V[u]``, the
noise-decomposition matrices ``gamma[u]``, ``S[u]``, ``A[u]``, vectors
``phi_0[u]``, ``sigma[u]`` and the scalar ``s_delta[u]``.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List

import numpy as np


@dataclass
class HeomParams:
    H: np.ndarray                      # (n, n) complex128
    V: List[np.ndarray]                # U x (n, n) complex128
    gamma: List[np.ndarray]            # U x (K_u, K_u) complex128
    phi_0: List[np.ndarray]            # U x (K_u,) complex128
    sigma: List[np.ndarray]            # U x (K_u,) complex128
    S: List[np.ndarray]                # U x (K_u, K_u) complex128
    A: List[np.ndarray]                # U x (K_u, K_u) complex128
    s_delta: List[complex]             # U
    max_depth: int
    name: str = "heom"
    meta: dict = field(default_factory=dict)
    # "integer" (the reference's default) or "sqrt" (LIBHEOM_SQRT_NORMALIZATION)
    normalization: str = "integer"
    # storage of every ADO in the state vector: the reference's `order`
    order: str = "row_major"
    # hrchy_filter(index, depth) -> bool of alloc_hrchy_space; None: full hierarchy
    hrchy_filter: object = None

    def __post_init__(self):
        self.H = np.ascontiguousarray(self.H, dtype=np.complex128)
        n = self.H.shape[0]
        if self.H.shape != (n, n):
            raise ValueError("H must be square")
        U = len(self.V)
        for name in ("gamma", "phi_0", "sigma", "S", "A", "s_delta"):
            if len(getattr(self, name)) != U:
                raise ValueError(f"{name} must have one entry per bath")
        self.V = [np.ascontiguousarray(v, dtype=np.complex128) for v in self.V]
        self.gamma = [np.ascontiguousarray(np.atleast_2d(g), dtype=np.complex128) for g in self.gamma]
        self.S = [np.ascontiguousarray(np.atleast_2d(g), dtype=np.complex128) for g in self.S]
        self.A = [np.ascontiguousarray(np.atleast_2d(g), dtype=np.complex128) for g in self.A]
        self.phi_0 = [np.ascontiguousarray(np.atleast_1d(g), dtype=np.complex128) for g in self.phi_0]
        self.sigma = [np.ascontiguousarray(np.atleast_1d(g), dtype=np.complex128) for g in self.sigma]
        self.s_delta = [complex(x) for x in self.s_delta]
        if self.normalization not in ("integer", "sqrt"):
            raise ValueError("normalization must be 'integer' or 'sqrt'")
        if self.order not in ("row_major", "col_major"):
            raise ValueError("order must be 'row_major' or 'col_major'")
        for u in range(U):
            k = self.gamma[u].shape[0]
            if self.V[u].shape != (n, n):
                raise ValueError("V[u] must be n x n")
            if (self.gamma[u].shape != (k, k) or self.S[u].shape != (k, k) or self.A[u].shape != (k, k)
                    or self.phi_0[u].shape != (k,) or self.sigma[u].shape != (k,)):
                raise ValueError(f"bath {u}: inconsistent mode count")

    @property
    def n_level(self) -> int:
        return self.H.shape[0]

    @property
    def n_noise(self) -> int:
        return len(self.V)

    @property
    def len_gamma(self) -> List[int]:
        return [g.shape[0] for g in self.gamma]

    @property
    def n_modes(self) -> int:
        return int(sum(self.len_gamma))

    def n_hrchy(self) -> int:
        from math import comb
        if self.hrchy_filter is None:
            return comb(self.n_modes + self.max_depth, self.max_depth)
        return len(hierarchy_indices(self.n_modes, self.max_depth, self.hrchy_filter))

    def rho0_ground(self) -> np.ndarray:
        """|0><0| in the system block, zero auxiliary ADOs."""
        n = self.n_level
        rho = np.zeros((self.n_hrchy(), n, n), dtype=np.complex128)
        rho[0, 0, 0] = 1.0
        return rho


def hierarchy_indices(n_dim: int, max_depth: int, hrchy_filter=None):
    """Multi-indices in the reference's breadth-first order (hrchy_space.cc:
    160-198), with the optional filter applied to each candidate."""
    from collections import deque
    out, pending = [], deque([((0,) * n_dim, 0)])
    while pending:
        idx, first = pending.popleft()
        out.append(idx)
        depth = sum(idx)
        if depth + 1 > max_depth:
            continue
        for k in range(first, n_dim):
            child = idx[:k] + (idx[k] + 1,) + idx[k + 1:]
            if hrchy_filter is None or hrchy_filter(list(child), depth + 1):
                pending.append((child, k))
    return out
