"""Learned closure of the truncated hierarchy tier (the "terminator").

Plain truncation drops the ADOs of tier N+1 (ptr_p1 == ptr_void in
heom_hilb.h:315-326).  Here a small MLP, trained by this library's own CUDA
forward / backward / Adam kernels (csrc/mlp.cu), predicts each dropped
rho_{n+1_k} from its tier-N parent rho_n, and an inference launch before every
right-hand side feeds the predictions to the +1 coupling term.

Network input per (tier-N ADO, mode k): [Re rho_n/s, Im rho_n/s, onehot(k),
Re A/s, Im A/s] with s = max |rho_n| and A the adiabatic estimate of
rho_{n+1_k}.  The adiabatic estimate carries the bath constants of mode k;
without it one network cannot serve a range of (lambda, beta): measured on
spin-boson data, the best linear closure of the bare inputs explains under a
third of the variance.

Training data: trajectories of the plain method at a deeper hierarchy; since
the breadth-first ADO order is tier-ascending, the first C(K+N, N) ADOs of a
deep state are exactly the ADOs of the depth-N model, in the same order.
"""
from __future__ import annotations

import ctypes
import math
from math import comb

import numpy as np

from . import _lib
from ._lib import check
from .params import HeomParams


class MLP:
    """x (d_in) -> Linear(h) -> GELU -> Linear(h) -> GELU -> Linear(d_out)."""

    def __init__(self, d_in: int, d_hidden: int = 256, d_out: int = 8, seed: int = 0):
        self._lib = _lib.load()
        self._h = ctypes.c_void_p()
        check(self._lib.heomgb_mlp_create(d_in, d_hidden, d_out, seed, ctypes.byref(self._h)))
        a, b, c, n = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong()
        check(self._lib.heomgb_mlp_sizes(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), ctypes.byref(n)))
        self.d_in, self.d_hidden, self.d_out, self.n_params = a.value, b.value, c.value, n.value

    def get_params(self) -> np.ndarray:
        out = np.zeros(self.n_params, dtype=np.float32)
        check(self._lib.heomgb_mlp_get_params(self._h, out.ctypes.data))
        return out

    def set_params(self, params) -> None:
        arr = np.ascontiguousarray(params, dtype=np.float32)
        if arr.size != self.n_params:
            raise ValueError("wrong parameter count")
        check(self._lib.heomgb_mlp_set_params(self._h, arr.ctypes.data))

    def forward(self, x_dev, y_dev, batch: int) -> None:
        check(self._lib.heomgb_mlp_forward(self._h, ctypes.c_void_p(x_dev), ctypes.c_void_p(y_dev), batch))

    def gradients(self, x_dev, t_dev, batch: int):
        g = np.zeros(self.n_params, dtype=np.float32)
        loss = ctypes.c_float()
        check(self._lib.heomgb_mlp_gradients(self._h, ctypes.c_void_p(x_dev), ctypes.c_void_p(t_dev), batch,
                                             g.ctypes.data, ctypes.byref(loss)))
        return g, loss.value

    def train_step(self, x_dev, t_dev, batch: int, lr: float) -> float:
        loss = ctypes.c_float()
        check(self._lib.heomgb_mlp_train_step(self._h, ctypes.c_void_p(x_dev), ctypes.c_void_p(t_dev), batch, lr,
                                              ctypes.byref(loss)))
        return loss.value

    def close(self) -> None:
        if self._h:
            self._lib.heomgb_mlp_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def dims(p: HeomParams):
    n2 = p.n_level ** 2
    return 4 * n2 + p.n_modes, 2 * n2


def attach(qme, mlp) -> None:
    """Use `mlp` for qme's truncated tier (None: plain truncation)."""
    qme._need()
    for s in list(qme._solvers):
        s.close()
    check(qme._lib.heomgb_qme_set_terminator(qme._h, mlp._h if mlp is not None else None))
    qme._terminator = mlp  # keep it alive while the model uses it


def _mode_constants(p: HeomParams):
    bath_of, s_k, a_k, g_k = [], [], [], []
    for u in range(p.n_noise):
        sv = p.S[u] @ p.phi_0[u]
        av = p.A[u] @ p.phi_0[u]
        for k in range(len(p.sigma[u])):
            bath_of.append(u)
            s_k.append(sv[k])
            a_k.append(av[k])
            g_k.append(p.gamma[u][k, k])
    return np.array(bath_of), np.array(s_k), np.array(a_k), np.array(g_k)


def features(p: HeomParams, n_tab, rho_shallow, first):
    """Input rows (tier-N ADOs l >= first, modes k) and the scales s of the ADOs."""
    n = p.n_level
    n2 = n * n
    K = p.n_modes
    bath_of, s_k, a_k, g_k = _mode_constants(p)
    R = rho_shallow[first:]                                    # (T, n, n)
    T = R.shape[0]
    s = np.sqrt((np.abs(R.astype(np.complex64)) ** 2).reshape(T, -1).max(axis=1)) + 1e-30
    ngd = (n_tab[first:first + T] * g_k[None, :]).sum(axis=1)  # (T,)
    V = np.stack([np.diag(p.V[u]) for u in range(p.n_noise)])  # (U, n)
    va = V[bath_of][:, :, None]                                # (K, n, 1)
    vb = V[bath_of][:, None, :]
    c = -1j * s_k[:, None, None] * (va - vb) + a_k[:, None, None] * (va + vb)   # (K, n, n)
    nk1 = n_tab[first:first + T] + 1.0                         # (T, K)
    denom = ngd[:, None] + g_k[None, :]                        # (T, K)
    A = (nk1 / denom)[:, :, None, None] * c[None] * R[:, None]  # (T, K, n, n)
    Rn = (R / s[:, None, None]).reshape(T, 1, n2)
    An = (A / s[:, None, None, None]).reshape(T, K, n2)
    X = np.concatenate([np.broadcast_to(Rn.real, (T, K, n2)), np.broadcast_to(Rn.imag, (T, K, n2)),
                        np.broadcast_to(np.eye(K), (T, K, K)), An.real, An.imag], axis=2)
    return X.reshape(T * K, 4 * n2 + K).astype(np.float32), s


def sample_spin_boson(rng, depth):
    """Spin-boson parameters over the batched-sweep ranges."""
    from .configs import spin_boson
    lam = math.exp(rng.uniform(math.log(0.05), math.log(5.0)))
    beta = rng.uniform(0.1, 10.0)
    eps = rng.uniform(-2.0, 2.0)
    return spin_boson(eps=eps, lam=lam, beta=beta, depth=depth), (lam, beta, eps)


def deep_trajectories(params, t_samples, dt=0.005, precision="fp64"):
    """Plain-method states of a batch of (deep) instances at t_samples; returns
    a list per instance of arrays (n_t, n_hrchy, n, n) and the stable mask."""
    from .heom import batch_solver, from_params, rk4
    qmes = [from_params(p, precision=precision) for p in params]
    bs = batch_solver(qmes, rk4())
    rho = np.concatenate([p.rho0_ground().ravel() for p in params])
    off = bs.offsets()
    frames = []
    bs.solve(rho, [0.0] + list(t_samples), lambda t: frames.append(rho.copy()), {"dt": dt})
    frames = np.array(frames[1:])
    out, stable = [], []
    for i, p in enumerate(params):
        a = frames[:, off[i]:off[i + 1]].reshape(len(t_samples), p.n_hrchy(), p.n_level, p.n_level)
        ok = bool(np.all(np.isfinite(a)) and np.abs(a[:, 0]).max() <= 2.0)
        out.append(a)
        stable.append(ok)
    bs.close()
    for q in qmes:
        q.close()
    return out, np.array(stable)


def make_dataset(params_deep, shallow_depth, t_samples, dt=0.005):
    """(X, T) rows for training from plain deep trajectories."""
    from .heom import from_params
    p0 = params_deep[0]
    q = from_params(HeomParams(**{**p0.__dict__, "max_depth": shallow_depth}))
    n_sh, _, _ = q.hrchy()
    q.close()
    qd = from_params(p0)
    n_deep, p1_deep, _ = qd.hrchy()
    qd.close()
    nh_sh = n_sh.shape[0]
    K = p0.n_modes
    first = nh_sh - (comb(K + shallow_depth - 1, shallow_depth) if shallow_depth > 0 else 1)
    assert np.array_equal(n_deep[:nh_sh], n_sh)
    traj, stable = deep_trajectories(params_deep, t_samples, dt)
    Xs, Ts = [], []
    n2 = p0.n_level ** 2
    for p, tr, ok in zip(params_deep, traj, stable):
        if not ok:
            continue
        for frame in tr:
            X, s = features(p, n_sh, frame[:nh_sh], first)
            child = p1_deep[first:nh_sh]                      # (T, K)
            tgt = frame[child] / s[:, None, None, None]       # (T, K, n, n)
            tgt = tgt.reshape(-1, n2)
            Xs.append(X)
            Ts.append(np.concatenate([tgt.real, tgt.imag], axis=1).astype(np.float32))
    return np.concatenate(Xs), np.concatenate(Ts), int(stable.sum())


def train(mlp: MLP, X, T, epochs=10, batch=4096, lr=1e-3, seed=0, log=None):
    """Adam on mean squared error with this library's kernels; returns epoch losses."""
    import torch
    dev = torch.device("cuda")
    Xd = torch.from_numpy(np.ascontiguousarray(X)).to(dev)
    Td = torch.from_numpy(np.ascontiguousarray(T)).to(dev)
    g = torch.Generator(device="cpu").manual_seed(seed)
    n = X.shape[0]
    losses = []
    for ep in range(epochs):
        perm = torch.randperm(n, generator=g).to(dev)
        tot, cnt = 0.0, 0
        for i in range(0, n - batch + 1, batch):
            idx = perm[i:i + batch]
            xb = Xd.index_select(0, idx).contiguous()
            tb = Td.index_select(0, idx).contiguous()
            torch.cuda.synchronize()
            loss = mlp.train_step(xb.data_ptr(), tb.data_ptr(), batch, lr)
            tot += loss
            cnt += 1
        losses.append(tot / max(cnt, 1))
        if log:
            log(ep, losses[-1])
    return losses


def population_errors(params_shallow, params_deep, mlp, t_list, dt=0.005):
    """Max |rho_00(t) - rho_00^deep(t)| of plain truncation and of the learned
    terminator, per instance (both at the shallow depth)."""
    from .heom import from_params, qme_solver, rk4
    out = []
    for ps, pd in zip(params_shallow, params_deep):
        ref = []
        qd = from_params(pd)
        sd = qme_solver(qd, rk4())
        r = pd.rho0_ground()
        sd.solve(r, t_list, lambda t: ref.append(r[0, 0, 0].real), {"dt": dt})
        res = []
        for use in (False, True):
            q = from_params(ps)
            if use:
                attach(q, mlp)
            s = qme_solver(q, rk4())
            r = ps.rho0_ground()
            pops = []
            s.solve(r, t_list, lambda t: pops.append(r[0, 0, 0].real), {"dt": dt})
            res.append(float(np.max(np.abs(np.array(pops) - np.array(ref)))))
            s.close()
            q.close()
        out.append(res)
        sd.close()
        qd.close()
    return np.array(out)
