"""Instance-resident fixed-step intervals (k_fixed_local: every instance of a batch
inside one CTA, its stage inputs in shared memory, one launch per output
interval with no grid-wide synchronisation) against the per-stage kernels on
the same batches.  The per-element arithmetic is the stage kernels', in the
same order, so every ADO agrees bit for bit in both forms, after many steps
and a clamped last step; the FP64 form also stays within 1e-10 of the oracle
port per instance."""
import dataclasses

import numpy as np
import pytest

import libheom_gb300 as lh
import oracle
from libheom_gb300 import configs

pytestmark = pytest.mark.gpu
DT = 0.005
T = [0.0, 37 * DT + 0.3 * DT, 60 * DT]  # the first interval ends with a shorter step


def instances(k_sb=10, k_chain=4):
    full = configs.batched_sweep()
    return full[:k_sb] + full[768:768 + k_chain]


def parts(tune):
    return tune["parts"] if "parts" in tune else [tune]


def go(ps, precision, local, monkeypatch, t=T, solver="rk4"):
    monkeypatch.setenv("HEOMGB_LOCAL", "1" if local else "0")
    qmes = [lh.from_params(p, precision=precision) for p in ps]
    bs = lh.batch_solver(qmes, lh.SOLVERS[solver]())
    rho = np.concatenate([p.rho0_ground().ravel() for p in ps])
    bs.solve(rho, list(t), None, {"dt": DT})
    monkeypatch.delenv("HEOMGB_LOCAL")
    return rho, bs


@pytest.mark.parametrize("solver", ["rk4", "lsrk4"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_local_bit_identical_to_stage_kernels(precision, solver, monkeypatch):
    ps = instances()
    loc, bs_l = go(ps, precision, True, monkeypatch, solver=solver)
    stg, bs_s = go(ps, precision, False, monkeypatch, solver=solver)
    assert all(p["local"] and p["local_bins"] >= 1 for p in parts(bs_l.tuning()))
    assert not any(p["local"] for p in parts(bs_s.tuning()))
    assert bs_l.stats()["rhs"] == bs_s.stats()["rhs"] == 4 * 61
    assert np.array_equal(loc, stg)
    if precision == "mixed":
        assert len(bs_l.parts()) == 2  # the range guard keeps some instances in FP64


def test_local_fp64_matches_oracle(monkeypatch):
    ps = instances(4, 2)
    rho, _ = go(ps, "fp64", True, monkeypatch, t=[0.0, 0.25])
    off = np.cumsum([0] + [p.n_hrchy() * p.n_level ** 2 for p in ps])
    port = oracle.Oracle("port")
    for i, p in enumerate(ps):
        ref = port.solve(p, p.rho0_ground(), [0.0, 0.25], solver="rk4", dt=DT)[-1]
        got = rho[off[i]:off[i + 1]].reshape(ref.shape)
        scale = np.abs(ref).max(axis=(1, 2), keepdims=True) + 1e-300
        assert (np.abs(got - ref) / scale).max() <= 1e-10


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_local_complex_h_sqrt_filter_col_major(precision, monkeypatch):
    """Complex H, sqrt normalisation, a filtered hierarchy (sentinel
    neighbours) and column-major ADOs at the boundary, in one batch."""
    rng = np.random.default_rng(5)
    base = [configs.spin_boson(depth=d) for d in (4, 6, 9)] + [configs.batched_sweep()[770]]
    ps = []
    for i, p in enumerate(base):
        n = p.n_level
        X = rng.uniform(-0.2, 0.2, (n, n))
        q = dataclasses.replace(p, H=p.H + 1j * (X - X.T), normalization="sqrt", order="col_major")
        if i == 1:
            q = dataclasses.replace(q, hrchy_filter=lambda idx, depth: idx[0] <= 3)
        ps.append(q)
    assert ps[1].n_hrchy() < configs.spin_boson(depth=6).n_hrchy()
    loc, bs_l = go(ps, precision, True, monkeypatch)
    stg, _ = go(ps, precision, False, monkeypatch)
    assert all(p["local"] for p in parts(bs_l.tuning()))
    assert np.all(np.isfinite(loc))
    assert np.array_equal(loc, stg)


def test_local_single_model(monkeypatch):
    """One FP64 model in one bin."""
    p = configs.spin_boson(depth=10)

    def run(local):
        monkeypatch.setenv("HEOMGB_LOCAL", "1" if local else "0")
        monkeypatch.setenv("HEOMGB_RESIDENT", "0")  # against the stage kernels
        qs = lh.qme_solver(lh.from_params(p, precision="fp64"), lh.rk4())
        rho = p.rho0_ground()
        qs.solve(rho, T, None, {"dt": DT})
        monkeypatch.delenv("HEOMGB_LOCAL")
        return rho, qs.tuning()

    loc, tune = run(True)
    stg, _ = run(False)
    assert tune["local"] and tune["local_bins"] == 1
    assert np.array_equal(loc, stg)


def test_local_not_for_adaptive_steps(monkeypatch):
    monkeypatch.setenv("HEOMGB_LOCAL", "1")
    p = configs.spin_boson(depth=6)
    qs = lh.qme_solver(lh.from_params(p, precision="fp64"), lh.rkdp())
    assert not qs.tuning()["local"]
