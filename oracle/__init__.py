"""Test infrastructure: ctypes front end of the two CPU oracles.

THE ORACLE IS NOT THE PRODUCT.  Only tests/, ``__graft_entry__.smoke()`` and
bench.py's CPU-baseline arm import this module, as the checker or as the timed
CPU baseline.  The product (``libheom_gb300``) never imports it.

* ``port``: oracle/heom_oracle.cpp, the CPU restatement of the reference path
  (built anywhere by ``make -C oracle port``).
* ``ref``:  the reference's own model/hierarchy/integrator sources compiled with
  a plain-loop engine (``make -C oracle ref``; needs the reference tree, so it is
  available only where golden fixtures are generated).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_lib", "libheom_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libheomref.so")
REF_SQRT_SO = os.path.join(HERE, "_ref", "libheomref_sqrt.so")
# where the reference source tree lies (only the fixture generator and the
# reference-code oracle read it); LIBHEOM_REFERENCE overrides the default
REF_TREE = os.environ.get("LIBHEOM_REFERENCE", "/root/reference")

FORMS = {"hilb": 0, "liou": 1, "ado": 2, "redfield_hilb": 3, "redfield_liou": 4}
SOLVERS = {"rk4": 0, "lsrk4": 1, "rkdp": 2}


class _Case(ctypes.Structure):
    _fields_ = [("n_level", ctypes.c_int), ("n_noise", ctypes.c_int), ("max_depth", ctypes.c_int),
                ("H", ctypes.c_void_p), ("V", ctypes.c_void_p), ("len_gamma", ctypes.c_void_p),
                ("gamma", ctypes.c_void_p), ("phi_0", ctypes.c_void_p), ("sigma", ctypes.c_void_p),
                ("S", ctypes.c_void_p), ("A", ctypes.c_void_p), ("s_delta", ctypes.c_void_p),
                ("sqrt_normalization", ctypes.c_int), ("col_major", ctypes.c_int),
                ("hrchy_filter", ctypes.c_void_p), ("filter_user", ctypes.c_void_p)]

# int filter(const int* index, int n_dim, int depth, void* user): nonzero keeps
FILTER = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_int, ctypes.c_void_p)


def make_filter(fn):
    """ctypes callback of fn(index: list[int], depth: int) -> bool (None: no filter)."""
    if fn is None:
        return None
    return FILTER(lambda idx, n_dim, depth, _u: 1 if fn([idx[i] for i in range(n_dim)], depth) else 0)


class PackedCase:
    """Keeps the flat arrays alive for as long as the ctypes struct is used."""

    def __init__(self, p):
        cat = lambda xs: np.ascontiguousarray(np.concatenate([np.ravel(x) for x in xs]) if xs else
                                              np.zeros(0), dtype=np.complex128)
        self.H = np.ascontiguousarray(p.H, dtype=np.complex128)
        self.V = cat(p.V)
        self.len_gamma = np.ascontiguousarray(p.len_gamma, dtype=np.int32)
        self.gamma = cat(p.gamma)
        self.phi_0 = cat(p.phi_0)
        self.sigma = cat(p.sigma)
        self.S = cat(p.S)
        self.A = cat(p.A)
        self.s_delta = np.ascontiguousarray(p.s_delta, dtype=np.complex128)
        ptr = lambda a: a.ctypes.data if a.size else None
        self.struct = _Case(p.n_level, p.n_noise, p.max_depth, ptr(self.H), ptr(self.V), ptr(self.len_gamma),
                            ptr(self.gamma), ptr(self.phi_0), ptr(self.sigma), ptr(self.S), ptr(self.A),
                            ptr(self.s_delta), 1 if getattr(p, "normalization", "integer") == "sqrt" else 0,
                            1 if getattr(p, "order", "row_major") == "col_major" else 0)
        self.filter = make_filter(getattr(p, "hrchy_filter", None))  # kept alive with the struct
        if self.filter is not None:
            self.struct.hrchy_filter = ctypes.cast(self.filter, ctypes.c_void_p)


def build(which: str = "port") -> None:
    target = {"port": PORT_SO, "ref": REF_SO, "ref_sqrt": REF_SQRT_SO}[which]
    if which.startswith("ref") and not os.path.isdir(REF_TREE):
        raise FileNotFoundError("reference tree not present; the reference oracle cannot be built here")
    subprocess.run(["make", "-s", "-C", HERE, "port" if which == "port" else "ref"], check=True)
    if not os.path.exists(target):
        raise RuntimeError(f"oracle build produced no {target}")


class Oracle:
    """which: "port", "ref" (the reference's build) or "ref_sqrt" (its
    LIBHEOM_SQRT_NORMALIZATION build; models must then carry
    normalization="sqrt")."""

    def __init__(self, which: str = "port"):
        path = {"port": PORT_SO, "ref": REF_SO, "ref_sqrt": REF_SQRT_SO}[which]
        if not os.path.exists(path):
            build(which)
        self.which = which
        self.lib = ctypes.CDLL(path)
        pre = "oracle_" if which == "port" else "heomref_"
        self._pre = pre
        L = self.lib
        c_int_p = ctypes.POINTER(ctypes.c_int)
        self._hrchy = getattr(L, pre + "hrchy")
        self._hrchy.argtypes = [ctypes.c_int, ctypes.c_int, c_int_p, ctypes.c_void_p, ctypes.c_void_p,
                                ctypes.c_void_p]
        self._n_hrchy = getattr(L, pre + "n_hrchy")
        self._n_hrchy.argtypes = [ctypes.c_void_p, c_int_p]
        self._calc = getattr(L, pre + "calc_diff")
        self._calc.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                               ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        self._solve = getattr(L, pre + "solve")
        argt = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_void_p, ctypes.c_int]
        if which == "port":
            argt.append(ctypes.c_void_p)
        self._solve.argtypes = argt
        err = getattr(L, pre + "last_error")
        err.restype = ctypes.c_char_p
        self._err = err

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(f"oracle ({self.which}) failed: {self._err().decode()}")

    def hrchy(self, n_dim: int, max_depth: int, hrchy_filter=None):
        """Hierarchy tables (n, ptr_p1, ptr_m1); hrchy_filter(index, depth) -> bool
        enables the reference's filter_flag."""
        cnt = ctypes.c_int(0)
        if hrchy_filter is None:
            call = lambda *tabs: self._hrchy(n_dim, max_depth, ctypes.byref(cnt), *tabs)
        else:
            f = make_filter(hrchy_filter)
            fn = getattr(self.lib, self._pre + "hrchy_filtered")
            fn.argtypes = [ctypes.c_int, ctypes.c_int, FILTER, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int),
                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
            call = lambda *tabs: fn(n_dim, max_depth, f, None, ctypes.byref(cnt), *tabs)
        self._check(call(None, None, None))
        c = cnt.value
        n = np.zeros((c, n_dim), dtype=np.int32)
        p1 = np.zeros((c + 1, n_dim), dtype=np.int32)
        m1 = np.zeros((c + 1, n_dim), dtype=np.int32)
        self._check(call(n.ctypes.data, p1.ctypes.data, m1.ctypes.data))
        return n, p1, m1

    def calc_diff(self, params, rho, drho=None, alpha=1.0, beta=0.0, form="hilb", threads=0):
        pc = PackedCase(params)
        rho = np.ascontiguousarray(rho, dtype=np.complex128)
        out = np.zeros_like(rho) if drho is None else np.array(drho, dtype=np.complex128, copy=True)
        a = np.array([complex(alpha).real, complex(alpha).imag])
        b = np.array([complex(beta).real, complex(beta).imag])
        self._check(self._calc(ctypes.byref(pc.struct), FORMS[form], rho.ctypes.data, out.ctypes.data,
                               a.ctypes.data, b.ctypes.data, threads or os.cpu_count()))
        return out

    def solve(self, params, rho0, t_list, solver="rk4", dt=0.005, atol=1e-8, rtol=1e-8, form="hilb",
              threads=0, with_stats=False):
        """Returns the states at every output time, shape (n_t, n_hrchy, n, n)."""
        pc = PackedCase(params)
        rho = np.array(rho0, dtype=np.complex128, copy=True, order="C")
        t = np.ascontiguousarray(t_list, dtype=np.float64)
        rho_t = np.zeros((len(t),) + rho.shape, dtype=np.complex128)
        args = [ctypes.byref(pc.struct), FORMS[form], SOLVERS[solver], rho.ctypes.data, t.ctypes.data, len(t),
                float(dt), float(atol), float(rtol), rho_t.ctypes.data, threads or os.cpu_count()]
        stats = np.zeros(3, dtype=np.int64)
        if self.which == "port":
            args.append(stats.ctypes.data)
        self._check(self._solve(*args))
        if with_stats:
            return rho_t, dict(rhs=int(stats[0]), attempts=int(stats[1]), accepted=int(stats[2]))
        return rho_t
