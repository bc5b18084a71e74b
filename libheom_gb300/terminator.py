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

Output: an elementwise gain C with rho_{n+1_k} ~ C rho_n / sigma_k, whose
imaginary part is constrained (C = y - i sign(v_a - v_b) softplus(z)) so that
the closure term only damps the tier-N ADOs.  Unconstrained regressions of
rho_{n+1_k} (and the adiabatic estimate itself) made the truncated hierarchy
blow up at low temperature, where the Matsubara coefficients are negative.
The loss is relative per row, so weak-coupling rows, where plain truncation
is already accurate, weigh as much as strong-coupling ones.

Applicability and fallback.  A damping-only closure cannot stand in for the
anti-damping that large negative Matsubara coefficients bring at low
temperature, so the closure is used (and trained) only where a bath's
expansion is dominated by its positive terms: cancel_log10 =
max_u log10(sum_k |s_k| / |sum_k s_k|) <= 0.2, the quantity the mixed form's
range guard reports (heomgb_qme_get_precision).  Elsewhere the model keeps
plain truncation.  `propagate` also checks rho_0 at every output time (finite,
populations in [-0.05, 1.05]) and reruns with plain truncation if the closure
failed.

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

    def set_loss(self, kind: int, n2: int = 0) -> None:
        """0: mean squared error; 1: the terminator's closure loss (heomgb_mlp_set_loss)."""
        check(self._lib.heomgb_mlp_set_loss(self._h, kind, n2))

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
    bath_of, s_k, a_k, g_k, sig = [], [], [], [], []
    for u in range(p.n_noise):
        sv = p.S[u] @ p.phi_0[u]
        av = p.A[u] @ p.phi_0[u]
        for k in range(len(p.sigma[u])):
            bath_of.append(u)
            s_k.append(sv[k])
            a_k.append(av[k])
            g_k.append(p.gamma[u][k, k])
            sig.append(p.sigma[u][k])
    return np.array(bath_of), np.array(s_k), np.array(a_k), np.array(g_k), np.array(sig)


def gain_signs(p: HeomParams):
    """(K, n2) sign(Re(v_a - v_b)) of every mode's bath (0 where the +1 term vanishes)."""
    bath_of = _mode_constants(p)[0]
    V = np.stack([np.diag(p.V[u]).real for u in range(p.n_noise)])
    dv = (V[:, :, None] - V[:, None, :]).reshape(p.n_noise, -1)
    return np.sign(dv[bath_of])


def features(p: HeomParams, n_tab, rho_shallow, first):
    """Input rows (tier-N ADOs l >= first, modes k) and the scales s of the ADOs."""
    n = p.n_level
    n2 = n * n
    K = p.n_modes
    bath_of, s_k, a_k, g_k, _ = _mode_constants(p)
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


def sample_exciton7(rng, depth):
    """7-site aggregates around the measured workload: a seeded Hamiltonian
    (site energies ~N(0, 100 cm^-1), couplings ~U(-100, 100) cm^-1), the
    reorganisation energy log-uniform in [15, 80] cm^-1 and the temperature
    uniform in [200, 400] K (gamma_c = 1/50 fs)."""
    from .configs import exciton_7site
    seed = int(rng.integers(1, 1 << 30))
    lam = math.exp(rng.uniform(math.log(15.0), math.log(80.0)))
    temp = rng.uniform(200.0, 400.0)
    return exciton_7site(seed=seed, depth=depth, lam_cm=lam, temp_k=temp), (seed, lam, temp)


def sample_spin_boson(rng, depth):
    """Spin-boson parameters over the batched-sweep ranges."""
    from .configs import spin_boson
    lam = math.exp(rng.uniform(math.log(0.05), math.log(5.0)))
    beta = rng.uniform(0.1, 10.0)
    eps = rng.uniform(-2.0, 2.0)
    return spin_boson(eps=eps, lam=lam, beta=beta, depth=depth), (lam, beta, eps)


CANCEL_MAX = 0.2


def admits(qme) -> bool:
    """True where the closure applies (see the module docstring)."""
    return qme.get_precision()["cancel_log10"] <= CANCEL_MAX


def deep_trajectories(params, t_samples, dt=0.005, precision="fp64", keep=None):
    """Plain-method states of a batch of (deep) instances at t_samples; returns
    a list per instance of arrays (n_t, n_keep, n, n) and the mask of the
    instances that stay bounded and that the closure applies to.  keep: only
    the first `keep` ADOs of every frame are kept (the tiers a shallower model
    and its closure need), so deep batches need not be stored whole."""
    from .heom import batch_solver, from_params, rk4
    qmes = [from_params(p, precision=precision) for p in params]
    gate = [admits(q) for q in qmes]
    bs = batch_solver(qmes, rk4())
    rho = np.concatenate([p.rho0_ground().ravel() for p in params])
    off = bs.offsets()
    frames = [[] for _ in params]
    seen = [0]

    def grab(t):
        seen[0] += 1
        if seen[0] == 1:  # the initial state
            return
        for i, p in enumerate(params):
            n2 = p.n_level ** 2
            nk = p.n_hrchy() if keep is None else min(keep, p.n_hrchy())
            frames[i].append(rho[off[i]:off[i] + nk * n2].copy())

    bs.solve(rho, [0.0] + list(t_samples), grab, {"dt": dt})
    out, stable = [], []
    for i, p in enumerate(params):
        nk = p.n_hrchy() if keep is None else min(keep, p.n_hrchy())
        a = np.array(frames[i]).reshape(len(t_samples), nk, p.n_level, p.n_level)
        ok = bool(gate[i] and np.all(np.isfinite(a)) and np.abs(a[:, 0]).max() <= 2.0)
        out.append(a)
        stable.append(ok)
    bs.close()
    for q in qmes:
        q.close()
    return out, np.array(stable)


def make_dataset(params_deep, shallow_depth, t_samples, dt=0.005):
    """(X, T) rows for the closure loss from plain deep trajectories: T rows are
    [Re t, Im t, Re r, Im r, sg] with t = rho_{n+1_k}/s, r = rho_n/(s sigma_k)."""
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
    # the tiers up to N + 1 (the targets' tier) of the deep frames
    keep = comb(K + shallow_depth + 1, shallow_depth + 1)
    traj, stable = deep_trajectories(params_deep, t_samples, dt, keep=keep)
    Xs, Ts = [], []
    n2 = p0.n_level ** 2
    for p, tr, ok in zip(params_deep, traj, stable):
        if not ok:
            continue
        sig = _mode_constants(p)[4]
        sg = gain_signs(p)                                    # (K, n2)
        for frame in tr:
            X, s = features(p, n_sh, frame[:nh_sh], first)
            T = s.shape[0]
            child = p1_deep[first:nh_sh]                      # (T, K)
            tgt = (frame[child] / s[:, None, None, None]).reshape(-1, n2)
            r = (frame[first:nh_sh].reshape(T, 1, n2) / s[:, None, None] / sig[None, :, None]).reshape(-1, n2)
            sgr = np.broadcast_to(sg[None], (T,) + sg.shape).reshape(-1, n2)
            Xs.append(X)
            Ts.append(np.concatenate([tgt.real, tgt.imag, r.real, r.imag, sgr], axis=1).astype(np.float32))
    return np.concatenate(Xs), np.concatenate(Ts), int(stable.sum())


def train(mlp: MLP, X, T, epochs=10, batch=4096, lr=1e-3, seed=0, log=None, cosine=False):
    """Adam with this library's kernels on the MLP's loss (set_loss); returns
    epoch losses.  cosine: decay the step size to zero over the epochs."""
    import torch
    dev = torch.device("cuda")
    Xd = torch.from_numpy(np.ascontiguousarray(X)).to(dev)
    Td = torch.from_numpy(np.ascontiguousarray(T)).to(dev)
    g = torch.Generator(device="cpu").manual_seed(seed)
    n = X.shape[0]
    losses = []
    for ep in range(epochs):
        lr_ep = 0.5 * lr * (1.0 + math.cos(math.pi * ep / epochs)) if cosine else lr
        perm = torch.randperm(n, generator=g).to(dev)
        tot, cnt = 0.0, 0
        for i in range(0, n - batch + 1, batch):
            idx = perm[i:i + batch]
            xb = Xd.index_select(0, idx).contiguous()
            tb = Td.index_select(0, idx).contiguous()
            torch.cuda.synchronize()
            loss = mlp.train_step(xb.data_ptr(), tb.data_ptr(), batch, lr_ep)
            tot += loss
            cnt += 1
        losses.append(tot / max(cnt, 1))
        if log:
            log(ep, losses[-1])
    return losses


def physical(rho0, tol=0.05) -> bool:
    """rho_0 finite with populations in [-tol, 1 + tol]."""
    if not np.all(np.isfinite(rho0)):
        return False
    pops = np.real(np.diagonal(rho0))
    return bool(pops.min() >= -tol and pops.max() <= 1.0 + tol)


def propagate(p: HeomParams, mlp, t_list, dt=0.005, observe=None):
    """Propagate p (truncated at its depth) with the learned closure `mlp` and
    RK4; if rho_0 leaves the physical range at an output time, rerun with plain
    truncation.  Returns (list of rho_0 at t_list, True if the closure was kept)."""
    from .heom import from_params, qme_solver, rk4
    for use in ((True, False) if mlp is not None else (False,)):
        q = from_params(p)
        if use and not admits(q):
            q.close()
            continue
        if use:
            attach(q, mlp)
        s = qme_solver(q, rk4())
        r = p.rho0_ground()
        out = []
        s.solve(r, t_list, lambda t: out.append(r[0].copy()), {"dt": dt})
        s.close()
        q.close()
        if not use or all(physical(x) for x in out):
            return out, use
    raise AssertionError("unreachable")


def population_errors(params_shallow, params_deep, mlp, t_list, dt=0.005):
    """Per instance: [max |rho_00(t) - rho_00^deep(t)| of plain truncation, the
    same with the learned closure (plain-truncation fallback included), 1 if
    the closure was kept], all at the shallow depth."""
    from .heom import from_params, qme_solver, rk4
    out = []
    for ps, pd in zip(params_shallow, params_deep):
        ref = []
        qd = from_params(pd)
        sd = qme_solver(qd, rk4())
        r = pd.rho0_ground()
        sd.solve(r, t_list, lambda t: ref.append(r[0, 0, 0].real), {"dt": dt})
        sd.close()
        qd.close()
        ref = np.array(ref)
        plain, _ = propagate(ps, None, t_list, dt)
        term, kept = propagate(ps, mlp, t_list, dt)
        e_plain = float(np.max(np.abs(np.array([x[0, 0].real for x in plain]) - ref)))
        e_term = float(np.max(np.abs(np.array([x[0, 0].real for x in term]) - ref)))
        out.append([e_plain, e_term, 1.0 if kept else 0.0])
    return np.array(out)
