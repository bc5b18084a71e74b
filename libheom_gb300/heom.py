"""Python mirror of libheom's model / solver interface over the C ABI.

Same class names, public members and call order as the reference:

    qme = heom_hilb(max_depth, n_inner_threads, n_outer_threads)   # heom_hilb.h:41-43
    qme.n_level = n; qme.n_level_2 = n*n; qme.H = H                 # qme_base.h:32-36
    qme.alloc_noises(U)                                             # qme_base.h:47-60
    qme.V[u] = ...; qme.len_gamma[u] = ...; qme.gamma[u] = ...      # qme_base.h:38-45
    qme.phi_0[u], qme.sigma[u], qme.S[u], qme.A[u], qme.s_delta[u]
    qme.set_param()                                                 # heom_hilb.h:57-68
    solver = rk4()        # or lsrk4(), rkdp()
    qs = qme_solver(qme, solver)                                    # qme_solver.h:26-35
    qs.solve(rho, t_list, callback, {"dt": 0.005})                  # qme_solver.h:44-52

The engine argument of the reference (a linalg_engine*) has no counterpart:
the device path is the only path.  Errors raise HeomError (the reference
throws std::out_of_range for a missing kwarg and exits on CUDA errors).
"""
from __future__ import annotations

import ctypes
import weakref
from concurrent.futures import ThreadPoolExecutor
from typing import Callable, Optional

import numpy as np

from . import _lib
from ._lib import CALLBACK, Kwargs, check

_FORMS = {"hilb": 0, "liou": 1, "ado": 2, "redfield_hilb": 3, "redfield_liou": 4}
_PRECISION = {"fp64": 0, "mixed": 1}


def _c128(a, shape=None) -> np.ndarray:
    arr = np.ascontiguousarray(np.asarray(a, dtype=np.complex128))
    if shape is not None:
        arr = arr.reshape(shape)
    return arr


class heom:
    """Common base of heom_hilb / heom_liou / heom_ado (heom.h:21-139)."""

    form = "hilb"

    def __init__(self, max_depth: int, n_inner_threads: int = 1, n_outer_threads: int = 1):
        if int(max_depth) < 0:
            raise ValueError("max_depth must be >= 0")
        self.max_depth = int(max_depth)
        self.n_inner_threads = n_inner_threads
        self.n_outer_threads = n_outer_threads
        self.n_level = 0
        self.n_level_2 = 0
        self.H = None
        self.n_noise = 0
        self.V, self.len_gamma, self.gamma, self.phi_0, self.sigma = [], [], [], [], []
        self.S, self.A, self.s_delta = [], [], []
        self.precision = "fp64"
        # "integer" (the reference's default) or "sqrt" (its LIBHEOM_SQRT_NORMALIZATION build)
        self.normalization = "integer"
        # storage of every ADO in the caller's state arrays: the reference's `order`
        self.order = "row_major"
        # hrchy_filter(index: list[int], depth: int) -> bool, the filter of
        # alloc_hrchy_space (hrchy_space.h:29-36); None: the full hierarchy
        self.hrchy_filter = None
        self.stream = None  # optional cudaStream_t handle (int)
        self._h = ctypes.c_void_p()
        self._lib = _lib.load()
        self._solvers = weakref.WeakSet()

    # -- qme_base ------------------------------------------------------------
    def alloc_noises(self, n_noise: int) -> None:
        n_noise = int(n_noise)
        if n_noise < 0:
            raise ValueError("n_noise must be >= 0")
        self.n_noise = n_noise
        self.V = [None] * n_noise
        self.len_gamma = [0] * n_noise
        self.gamma = [None] * n_noise
        self.phi_0 = [None] * n_noise
        self.sigma = [None] * n_noise
        self.S = [None] * n_noise
        self.A = [None] * n_noise
        self.s_delta = [0j] * n_noise

    def set_param(self, engine=None) -> None:
        lib = self._lib
        self.close()
        n = int(self.n_level)
        if n <= 0 or self.H is None:
            raise ValueError("set n_level and H before set_param")
        if self.n_level_2 and int(self.n_level_2) != n * n:
            raise ValueError("n_level_2 must equal n_level**2")
        h = ctypes.c_void_p()
        check(lib.heomgb_qme_create(_FORMS[self.form], self.max_depth, int(self.n_inner_threads),
                                    int(self.n_outer_threads), ctypes.byref(h)))
        self._h = h
        H = _c128(self.H, (n, n))
        check(lib.heomgb_qme_set_hamiltonian(h, n, H.ctypes.data))
        check(lib.heomgb_qme_alloc_noises(h, self.n_noise))
        for u in range(self.n_noise):
            L = int(self.len_gamma[u])
            V = _c128(self.V[u], (n, n))
            g = _c128(self.gamma[u], (L, L))
            p = _c128(self.phi_0[u], (L,))
            s = _c128(self.sigma[u], (L,))
            Sm = _c128(self.S[u], (L, L))
            Am = _c128(self.A[u], (L, L))
            sd = _c128([self.s_delta[u]])
            check(lib.heomgb_qme_set_noise(h, u, V.ctypes.data, L, g.ctypes.data, p.ctypes.data, s.ctypes.data,
                                           Sm.ctypes.data, Am.ctypes.data, sd.ctypes.data))
        check(lib.heomgb_qme_set_precision(h, _PRECISION[self.precision]))
        check(lib.heomgb_qme_set_normalization(h, {"integer": 0, "sqrt": 1}[self.normalization]))
        check(lib.heomgb_qme_set_order(h, {"row_major": 0, "col_major": 1}[self.order]))
        if self.hrchy_filter is not None:
            fn = self.hrchy_filter
            self._filter_cb = _lib.HRCHY_FILTER(lambda idx, k, depth, _u: 1 if fn([idx[i] for i in range(k)], depth)
                                                else 0)
            check(lib.heomgb_qme_set_hrchy_filter(h, self._filter_cb, None))
        if self.stream:
            check(lib.heomgb_qme_set_stream(h, ctypes.c_void_p(int(self.stream))))
        check(lib.heomgb_qme_set_param(h))

    def _need(self):
        if not self._h:
            raise RuntimeError("set_param has not been called")

    def get_precision(self) -> dict:
        """Requested / effective precision and the range-guard inputs
        (heomgb_qme_get_precision): a MIXED model runs in FP64 when
        cancel_log10 > 0.8, growth_log10 > 7.5, or both growth_log10 > 2 and
        cancel_log10 > 0.2."""
        self._need()
        r, e, g, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_double(), ctypes.c_double()
        check(self._lib.heomgb_qme_get_precision(self._h, ctypes.byref(r), ctypes.byref(e), ctypes.byref(g),
                                                 ctypes.byref(c)))
        names = {0: "fp64", 1: "mixed"}
        return dict(requested=names[r.value], effective=names[e.value], growth_log10=g.value, cancel_log10=c.value)

    def get_n_hrchy(self) -> int:
        self._need()
        v = ctypes.c_int()
        check(self._lib.heomgb_qme_get_n_hrchy(self._h, ctypes.byref(v)))
        return v.value

    def get_n_dim(self) -> int:
        self._need()
        v = ctypes.c_int()
        check(self._lib.heomgb_qme_get_n_dim(self._h, ctypes.byref(v)))
        return v.value

    def main_size(self) -> int:
        self._need()
        v = ctypes.c_longlong()
        check(self._lib.heomgb_qme_main_size(self._h, ctypes.byref(v)))
        return v.value

    def hrchy(self):
        """(n, ptr_p1, ptr_m1) tables of hs (hrchy_space.h:18-27), from the device."""
        nh, K = self.get_n_hrchy(), self.get_n_dim()
        n = np.zeros((nh, K), dtype=np.int32)
        p1 = np.zeros((nh + 1, K), dtype=np.int32)
        m1 = np.zeros((nh + 1, K), dtype=np.int32)
        check(self._lib.heomgb_qme_get_hrchy(self._h, n.ctypes.data, p1.ctypes.data, m1.ctypes.data))
        return n, p1, m1

    def calc_diff_impl(self, drho_dt: np.ndarray, rho: np.ndarray, alpha=1.0, beta=0.0) -> None:
        """drho_dt = beta*drho_dt - alpha*D(rho), in place (heom_hilb.h:70-215)."""
        self._need()
        if not (isinstance(drho_dt, np.ndarray) and drho_dt.dtype == np.complex128 and drho_dt.flags.c_contiguous):
            raise TypeError("drho_dt must be a C-contiguous complex128 array")
        rho = _c128(rho)
        if rho.size != self.main_size() or drho_dt.size != self.main_size():
            raise ValueError("rho / drho_dt must hold main_size() elements")
        a = np.array([complex(alpha).real, complex(alpha).imag])
        b = np.array([complex(beta).real, complex(beta).imag])
        check(self._lib.heomgb_qme_calc_diff(self._h, drho_dt.ctypes.data, rho.ctypes.data, a.ctypes.data,
                                             b.ctypes.data))

    def calc_diff(self, rho, alpha=1.0, beta=0.0, drho=None) -> np.ndarray:
        out = np.zeros(np.shape(rho), dtype=np.complex128) if drho is None else np.array(drho, np.complex128)
        self.calc_diff_impl(out, rho, alpha, beta)
        return out

    def close(self) -> None:
        for s in list(self._solvers):
            s.close()
        if self._h:
            check(self._lib.heomgb_qme_destroy(self._h))
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class heom_hilb(heom):
    """Hilbert-space HEOM (heom_hilb.h:18-216)."""
    form = "hilb"


class heom_liou(heom):
    """Liouville-space HEOM with per-ADO superoperators (heom_liou.h:18-259)."""
    form = "liou"


class heom_ado(heom):
    """ADO-space HEOM: one global block-sparse generator (heom_ado.h:18-204)."""
    form = "ado"


class _redfield(heom):
    """Redfield models (redfield.h:21-173): the same H and noise members, no
    hierarchy; the state is one n x n matrix.  The constructor takes no depth
    (redfield_hilb() in the reference); thread-count arguments are accepted."""

    def __init__(self, *args, **kwargs):
        super().__init__(0)


class redfield_hilb(_redfield):
    """Hilbert-space Redfield (redfield_hilb.h:18-91)."""
    form = "redfield_hilb"


class redfield_liou(_redfield):
    """Liouville-space Redfield (redfield_liou.h:18-104)."""
    form = "redfield_liou"


class solver_base:
    kind = -1

    def __init__(self):
        self._h = ctypes.c_void_p()
        lib = _lib.load()
        check(lib.heomgb_solver_create(self.kind, ctypes.byref(self._h)))
        self._lib = lib

    def __del__(self):
        try:
            if self._h:
                self._lib.heomgb_solver_destroy(self._h)
        except Exception:
            pass


class rk4(solver_base):
    """Classic RK4 (solver/rk4.h:15-66)."""
    kind = 0


class lsrk4(solver_base):
    """2N-storage RK4 (solver/lsrk4.h:15-48)."""
    kind = 1


class rkdp(solver_base):
    """Dormand-Prince 5(4) with error control (solver/rkdp.h:15-180)."""
    kind = 2


def _kwargs(kw: Optional[dict]) -> Kwargs:
    k = Kwargs()
    kw = kw or {}
    for key in ("dt", "atol", "rtol"):
        if key in kw:
            v = kw[key]
            if not isinstance(v, (float, int, np.floating, np.integer)) or isinstance(v, bool):
                raise TypeError(f"kwarg {key!r} must be a real number")
            setattr(k, key, float(v))
            setattr(k, "has_" + key, 1)
    return k


class qme_solver:
    """Facade wiring a model and an integrator (qme_solver.h:18-53)."""

    def __init__(self, qme: heom, solver: solver_base, engine=None):
        qme._need()
        self.qme, self.solver = qme, solver
        self._lib = qme._lib
        self._h = ctypes.c_void_p()
        check(self._lib.heomgb_qme_solver_create(qme._h, solver._h, ctypes.byref(self._h)))
        qme._solvers.add(self)

    def _need(self):
        if not self._h:
            raise RuntimeError("this qme_solver was closed (its model was set up again or closed)")

    def solve(self, rho: np.ndarray, t_list, callback: Optional[Callable[[float], None]] = None,
              kwargs: Optional[dict] = None) -> None:
        """Propagate the host array rho in place through t_list (qme_solver.h:44-52)."""
        self._need()
        if not (isinstance(rho, np.ndarray) and rho.dtype == np.complex128 and rho.flags.c_contiguous):
            raise TypeError("rho must be a C-contiguous complex128 array")
        if rho.size != self.main_size():
            raise ValueError("rho must hold main_size() elements")
        t = np.ascontiguousarray(t_list, dtype=np.float64)
        cb = CALLBACK(lambda tt, _u: callback(tt)) if callback else CALLBACK()
        kw = _kwargs(kwargs)
        check(self._lib.heomgb_qme_solver_solve(self._h, rho.ctypes.data, t.ctypes.data, len(t), cb, None,
                                                ctypes.byref(kw)))

    def solve_device(self, rho_ptr: int, t_list, callback=None, kwargs: Optional[dict] = None) -> None:
        """Same as solve with rho a device pointer (double2 array of main_size())."""
        self._need()
        t = np.ascontiguousarray(t_list, dtype=np.float64)
        cb = CALLBACK(lambda tt, _u: callback(tt)) if callback else CALLBACK()
        kw = _kwargs(kwargs)
        check(self._lib.heomgb_qme_solver_solve_device(self._h, ctypes.c_void_p(int(rho_ptr)), t.ctypes.data,
                                                       len(t), cb, None, ctypes.byref(kw)))

    def main_size(self) -> int:
        v = ctypes.c_longlong()
        check(self._lib.heomgb_qme_solver_main_size(self._h, ctypes.byref(v)))
        return v.value

    def tuning(self) -> dict:
        """Tile shape the autotuner picked (diagonal-coupling kernel)."""
        b, e, t, m = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(self._lib.heomgb_qme_solver_tuning(self._h, ctypes.byref(b), ctypes.byref(e), ctypes.byref(t),
                                                 ctypes.byref(m)))
        tc, rs, rg, ra = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(self._lib.heomgb_qme_solver_tensor_cores(self._h, ctypes.byref(tc)))
        check(self._lib.heomgb_qme_solver_resident(self._h, ctypes.byref(rs), ctypes.byref(rg), ctypes.byref(ra)))
        lo, lb, lk = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(self._lib.heomgb_qme_solver_local(self._h, ctypes.byref(lo), ctypes.byref(lb), ctypes.byref(lk)))
        si, st = ctypes.c_int(), ctypes.c_int()
        check(self._lib.heomgb_qme_solver_site_kernel(self._h, ctypes.byref(si), ctypes.byref(st)))
        out = dict(block=b.value, elems_per_thread=e.value, n_tiles=t.value, min_blocks=m.value,
                   tensor_cores=bool(tc.value), resident=bool(rs.value), local=bool(lo.value),
                   sites=bool(si.value))
        if si.value:
            out.update(sites_ados_per_tile=st.value)
        if rs.value:
            out.update(resident_grid=rg.value, resident_ados_per_cta=ra.value)
        if lo.value:
            out.update(local_bins=lb.value, local_block=lk.value)
        return out

    def stats(self) -> dict:
        r, a, c = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_longlong()
        d = ctypes.c_double()
        check(self._lib.heomgb_qme_solver_stats(self._h, ctypes.byref(r), ctypes.byref(a), ctypes.byref(c),
                                                ctypes.byref(d)))
        nh = sum(q.get_n_hrchy() for q in getattr(self, "qmes", [self.qme]))
        return dict(rhs=r.value, attempts=a.value, accepted=c.value, dt_save=d.value, ado_updates=r.value * nh)

    def timing(self) -> dict:
        """Device time of the last solve inside stage-kernel graph replays."""
        ms, k = ctypes.c_double(), ctypes.c_longlong()
        check(self._lib.heomgb_qme_solver_timing(self._h, ctypes.byref(ms), ctypes.byref(k)))
        return dict(busy_ms=ms.value, kernels=k.value)

    def close(self) -> None:
        if self._h:
            self._lib.heomgb_qme_solver_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _batch_part(qme_solver):
    """One C-level batch solver over models that share an effective precision."""

    def __init__(self, qmes, solver):
        self.qme, self.qmes, self.solver = qmes[0], qmes, solver
        self._lib = qmes[0]._lib
        self._h = ctypes.c_void_p()
        arr = (ctypes.c_void_p * len(qmes))(*[q._h.value for q in qmes])
        check(self._lib.heomgb_batch_solver_create(arr, len(qmes), solver._h, ctypes.byref(self._h)))
        for q in qmes:
            q._solvers.add(self)


class batch_solver:
    """Many uneven instances stepped together, every stage in one launch.

    The state is the concatenation of the models' states in order
    (`offsets()` gives each instance's first element).  Models whose effective
    precision differs (a MIXED request kept in FP64 by the range
    guard, heomgb_qme_get_precision) run in a second sub-batch; each output
    interval then steps both sub-batches concurrently: each sub-batch solver
    runs on its own stream from its own host thread (the library's calls
    release the interpreter lock), so the FP64 sub-batch's FP64-pipe work
    overlaps the mixed sub-batch's memory-bound stages."""

    def __init__(self, qmes, solver: solver_base, engine=None):
        qmes = list(qmes)
        if not qmes:
            raise ValueError("empty batch")
        for q in qmes:
            q._need()
        self.qmes, self.solver = qmes, solver
        sizes = [q.main_size() for q in qmes]
        self._off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        groups = {}
        for i, q in enumerate(qmes):
            groups.setdefault(q.get_precision()["effective"], []).append(i)
        self._parts = []
        for _, idx in sorted(groups.items()):
            part = _batch_part([qmes[i] for i in idx], solver)
            ranges = [(int(self._off[i]), int(self._off[i + 1])) for i in idx]
            contiguous = all(ranges[j][1] == ranges[j + 1][0] for j in range(len(ranges) - 1))
            self._parts.append((part, idx, ranges, contiguous))

    def offsets(self):
        return self._off.copy()

    def main_size(self) -> int:
        return int(self._off[-1])

    def parts(self):
        """[(instance indices, effective precision)] of the sub-batches."""
        return [(idx, p.qme.get_precision()["effective"]) for p, idx, _, _ in self._parts]

    def _gather(self, rho, ranges):
        return np.concatenate([rho[a:b] for a, b in ranges]) if len(ranges) > 1 else rho[ranges[0][0]:ranges[0][1]].copy()

    def _scatter(self, rho, ranges, sub):
        o = 0
        for a, b in ranges:
            rho[a:b] = sub[o:o + b - a]
            o += b - a

    def solve(self, rho: np.ndarray, t_list, callback=None, kwargs=None) -> None:
        if not (isinstance(rho, np.ndarray) and rho.dtype == np.complex128 and rho.flags.c_contiguous):
            raise TypeError("rho must be a C-contiguous complex128 array")
        if rho.size != self.main_size():
            raise ValueError("rho must hold main_size() elements")
        flat = rho.reshape(-1)
        if len(self._parts) == 1:
            self._parts[0][0].solve(flat, t_list, callback, kwargs)
            return
        t = [float(x) for x in t_list]
        self._counts = [dict(rhs=0, attempts=0, accepted=0) for _ in self._parts]
        with ThreadPoolExecutor(len(self._parts)) as pool:  # sub-batches run concurrently (own streams)
            for i in range(len(t) - 1):
                if callback:
                    callback(t[i])
                subs = [self._gather(flat, ranges) for _, _, ranges, _ in self._parts]
                futs = [pool.submit(part.solve, sub, [t[i], t[i + 1]], None, kwargs)
                        for (part, _, _, _), sub in zip(self._parts, subs)]
                for f in futs:
                    f.result()
                for (_, _, ranges, _), sub in zip(self._parts, subs):
                    self._scatter(flat, ranges, sub)
                self._count_interval()
        if callback and t:
            callback(t[-1])

    def _count_interval(self):
        # each sub-batch solve covers one interval: its counters restart every interval
        for c, (part, _, _, _) in zip(self._counts, self._parts):
            st = part.stats()
            for k in c:
                c[k] += st[k]

    def solve_device(self, rho_ptr: int, t_list, callback=None, kwargs=None) -> None:
        """rho_ptr: device pointer to the concatenated state (complex128)."""
        if len(self._parts) == 1:
            self._parts[0][0].solve_device(rho_ptr, t_list, callback, kwargs)
            return
        if not all(c for _, _, _, c in self._parts):
            raise ValueError("sub-batches must be contiguous in the state for device solves; order the models "
                             "by effective precision")
        t = [float(x) for x in t_list]
        self._counts = [dict(rhs=0, attempts=0, accepted=0) for _ in self._parts]
        with ThreadPoolExecutor(len(self._parts)) as pool:  # sub-batches run concurrently (own streams)
            for i in range(len(t) - 1):
                if callback:
                    callback(t[i])
                futs = [pool.submit(part.solve_device, int(rho_ptr) + 16 * ranges[0][0], [t[i], t[i + 1]], None,
                                    kwargs) for part, _, ranges, _ in self._parts]
                for f in futs:
                    f.result()
                self._count_interval()
        if callback and t:
            callback(t[-1])

    def stats(self) -> dict:
        out = dict(rhs=0, attempts=0, accepted=0, ado_updates=0, dt_save=-1.0)
        counts = getattr(self, "_counts", None) if len(self._parts) > 1 else None
        for j, (part, idx, _, _) in enumerate(self._parts):
            st = counts[j] if counts else part.stats()
            nh = sum(self.qmes[i].get_n_hrchy() for i in idx)
            out["rhs"] = max(out["rhs"], st["rhs"])
            out["attempts"] = max(out["attempts"], st["attempts"])
            out["accepted"] = max(out["accepted"], st["accepted"])
            out["ado_updates"] += st["rhs"] * nh
        return out

    def timing(self) -> dict:
        """Busy time and stage kernels of the last solve, in total and per sub-batch
        (the sub-batches run concurrently: the total busy time is the longest one's)."""
        ms, k, parts = 0.0, 0, []
        for part, idx, ranges, _ in self._parts:
            t = part.timing()
            ms = max(ms, t["busy_ms"])
            k += t["kernels"]
            parts.append(dict(t, precision=part.qme.get_precision()["effective"], instances=len(idx),
                              elements=sum(b - a for a, b in ranges), rhs=part.stats()["rhs"]))
        return dict(busy_ms=ms, kernels=k, parts=parts)

    def tuning(self) -> dict:
        return {"parts": [p.tuning() for p, _, _, _ in self._parts]} if len(self._parts) > 1 else \
            self._parts[0][0].tuning()

    def close(self) -> None:
        for part, _, _, _ in self._parts:
            part.close()


def from_params(p, form: str = "hilb", precision: str = "fp64", stream=None) -> heom:
    """Build and set up a model from a HeomParams."""
    cls = {"hilb": heom_hilb, "liou": heom_liou, "ado": heom_ado, "redfield_hilb": redfield_hilb,
           "redfield_liou": redfield_liou}[form]
    q = cls(p.max_depth, 1, 1)
    q.n_level = p.n_level
    q.n_level_2 = p.n_level ** 2
    q.H = p.H
    q.alloc_noises(p.n_noise)
    for u in range(p.n_noise):
        q.V[u] = p.V[u]
        q.len_gamma[u] = p.len_gamma[u]
        q.gamma[u] = p.gamma[u]
        q.phi_0[u] = p.phi_0[u]
        q.sigma[u] = p.sigma[u]
        q.S[u] = p.S[u]
        q.A[u] = p.A[u]
        q.s_delta[u] = p.s_delta[u]
    q.precision = precision
    q.normalization = p.normalization
    q.order = p.order
    q.hrchy_filter = p.hrchy_filter
    q.stream = stream
    q.set_param()
    return q


SOLVERS = {"rk4": rk4, "lsrk4": lsrk4, "rkdp": rkdp}
