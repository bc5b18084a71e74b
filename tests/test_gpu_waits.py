"""Bounded device waits that run out.

The resident interval kernels separate stages with a grid barrier whose wait
is bounded (a spin limit of polls).  Here one CTA is made to skip its
arrivals (host-side fault injection through HEOMGB_FAULT_SKIP_ARRIVAL, with
the spin limit shortened by HEOMGB_FAULT_SPIN_LIMIT), so every other CTA's wait
runs out: the kernel must return, the solve must report HEOMGB_ERR_CUDA with
its message within a second, and the same solver must then run a normal
solve that gives the same bits as a fresh solver.  Nothing here faults the
GPU: the missing arrival only makes bounded waits give up.  The reference
calls std::exit(1) on a device error instead (utility_gpu.h:14-36)."""
import time

import numpy as np
import pytest

import libheom_gb300 as lh
from libheom_gb300 import configs

pytestmark = pytest.mark.gpu

CASES = {
    "rkdp": (lh.rkdp, [0.0, 5.0], dict(dt=0.1, atol=1e-8, rtol=1e-8), "mixed"),
    "rk4": (lh.rk4, [0.0, 2.0], dict(dt=0.1), "mixed"),
    "rk4_fp64": (lh.rk4, [0.0, 2.0], dict(dt=0.1), "fp64"),
    "lsrk4": (lh.lsrk4, [0.0, 2.0], dict(dt=0.1), "mixed"),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_missing_arrival_makes_the_wait_run_out(name, monkeypatch):
    solver, t, kw, prec = CASES[name]
    p = configs.exciton_7site(depth=3)
    monkeypatch.setenv("HEOMGB_RESIDENT", "1")
    monkeypatch.setenv("HEOMGB_LOCAL", "0")
    qs = lh.qme_solver(lh.from_params(p, precision=prec), solver())
    assert qs.tuning()["resident"]
    monkeypatch.setenv("HEOMGB_FAULT_SKIP_ARRIVAL", "0")
    monkeypatch.setenv("HEOMGB_FAULT_SPIN_LIMIT", "4096")
    rho = p.rho0_ground()
    t0 = time.perf_counter()
    with pytest.raises(lh.HeomError) as err:
        qs.solve(rho, t, None, dict(kw))
    assert time.perf_counter() - t0 < 1.0
    assert err.value.status == 3  # HEOMGB_ERR_CUDA
    assert "grid barrier wait ran out" in str(err.value)
    monkeypatch.delenv("HEOMGB_FAULT_SKIP_ARRIVAL")
    monkeypatch.delenv("HEOMGB_FAULT_SPIN_LIMIT")
    # the same solver recovers: a normal solve gives the bits of a fresh solver
    rho = p.rho0_ground()
    qs.solve(rho, t, None, dict(kw))
    fresh = lh.qme_solver(lh.from_params(p, precision=prec), solver())
    assert fresh.tuning()["resident"]
    ref = p.rho0_ground()
    fresh.solve(ref, t, None, dict(kw))
    assert np.all(np.isfinite(rho))
    if name != "rkdp":  # fixed steps: the same launches, the same bits
        assert np.array_equal(rho, ref)
    else:  # tuned shapes may differ between the two solvers (the error norm's sum order)
        assert np.abs(rho - ref).max() <= 1e-6
