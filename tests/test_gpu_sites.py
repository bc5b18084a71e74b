"""The stage kernel for site-local baths (k_rhs_sites: per-ADO lists of
occupied modes, 4 x 4 register blocks of the commutator, compile-time stage
epilogues, cp.async-staged tiles) against the general diagonal-coupling stage
kernel (k_rhs_diag) on the same models and solvers.

Both do the same per-element arithmetic in the same order, so the states
must agree bit for bit (the new kernel skips terms without a neighbour that
the other adds as 0 * 0, which can only change the sign of a zero).  The
resident and instance-resident interval kernels are switched off so that
both runs use per-stage launches."""
import dataclasses

import numpy as np
import pytest

import libheom_gb300 as lh
import oracle
from libheom_gb300 import configs

pytestmark = pytest.mark.gpu


def run(p, solver, t, kw, monkeypatch, sites, shape="256x2x2"):
    monkeypatch.setenv("HEOMGB_RESIDENT", "0")
    monkeypatch.setenv("HEOMGB_LOCAL", "0")
    if sites:
        monkeypatch.setenv("HEOMGB_TILE", "sites:" + shape)
        monkeypatch.delenv("HEOMGB_SITES", raising=False)
    else:
        monkeypatch.delenv("HEOMGB_TILE", raising=False)
        monkeypatch.setenv("HEOMGB_SITES", "0")
    qs = lh.qme_solver(lh.from_params(p, precision="mixed"), lh.SOLVERS[solver]())
    tune = qs.tuning()
    rho = p.rho0_ground()
    qs.solve(rho, list(t), None, dict(kw))
    for k in ("HEOMGB_RESIDENT", "HEOMGB_LOCAL", "HEOMGB_TILE", "HEOMGB_SITES"):
        monkeypatch.delenv(k, raising=False)
    return rho, qs.stats(), tune


def complex_h(p):
    rng = np.random.default_rng(11)
    n = p.n_level
    X = rng.standard_normal((n, n)) * 0.002
    return dataclasses.replace(p, H=p.H + 1j * (X - X.T))


CASES = {
    "agg8_depth4": lambda: configs.aggregate_24site(n_sites=8, depth=4),
    "agg12_sqrt": lambda: dataclasses.replace(configs.aggregate_24site(n_sites=12, depth=3), normalization="sqrt"),
    "agg8_filtered": lambda: dataclasses.replace(configs.aggregate_24site(n_sites=8, depth=4),
                                                 hrchy_filter=lambda idx, d: idx[0] <= 1 and d <= 3 + (idx[1] == 0)),
    # n > 32: the bath-term pass's lanes cover a row or column in two rounds
    "agg36_depth2": lambda: configs.aggregate_24site(n_sites=36, depth=2),
    # the smallest hierarchies: one ADO (no bath terms), and one tier below it
    "agg8_depth0": lambda: configs.aggregate_24site(n_sites=8, depth=0),
    "agg8_depth1": lambda: configs.aggregate_24site(n_sites=8, depth=1),
}
SOLVES = {
    "rk4": ([0.0, 2.0, 4.0], dict(dt=0.5)),
    "lsrk4": ([0.0, 2.0, 4.0], dict(dt=0.5)),
    "rkdp": ([0.0, 5.0, 10.0], dict(dt=0.1, atol=1e-8, rtol=1e-8)),
}


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("solver", sorted(SOLVES))
def test_sites_kernel_bit_identical_to_stage_kernel(case, solver, monkeypatch):
    p = CASES[case]()
    t, kw = SOLVES[solver]
    got, st_s, tune_s = run(p, solver, t, kw, monkeypatch, True)
    ref, st_r, tune_r = run(p, solver, t, kw, monkeypatch, False)
    assert tune_s["sites"] and tune_s["sites_ados_per_tile"] == 2
    assert not tune_r["sites"]
    assert st_s["rhs"] == st_r["rhs"]
    assert np.all(np.isfinite(got))
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("shape", ["128x1x2", "256x3x3", "128x4x3", "256x8x2", "288x8x2", "64x5x2", "256x4x4", "256x2x2x4"])
def test_sites_kernel_tile_shapes(shape, monkeypatch):
    """Every tile shape gives the same bits (the tile only moves work between CTAs)."""
    p = configs.aggregate_24site(n_sites=8, depth=4)
    t, kw = SOLVES["lsrk4"]
    got, _, tune = run(p, "lsrk4", t, kw, monkeypatch, True, shape=shape)
    ref, _, _ = run(p, "lsrk4", t, kw, monkeypatch, False)
    assert tune["sites"]
    assert np.array_equal(got, ref)


def test_complex_hamiltonian_keeps_the_general_kernel(monkeypatch):
    """The site-local-bath kernel takes real H only; pinning it for a complex H
    is refused and the autotuner leaves it out."""
    p = complex_h(configs.aggregate_24site(n_sites=8, depth=3))
    monkeypatch.setenv("HEOMGB_TILE", "sites:256x2x2")
    with pytest.raises(lh.HeomError):
        lh.qme_solver(lh.from_params(p, precision="mixed"), lh.lsrk4())
    monkeypatch.delenv("HEOMGB_TILE")
    assert not lh.qme_solver(lh.from_params(p, precision="mixed"), lh.lsrk4()).tuning()["sites"]


def test_sites_kernel_24site_vs_oracle(monkeypatch):
    """The 24-site aggregate (20825 ADOs x 576 elements) through the new
    kernel, three LSRK4 steps, against the CPU oracle: 1e-6 absolute."""
    p = configs.aggregate_24site()
    t = [0.0, 1.5]
    got, _, tune = run(p, "lsrk4", t, dict(dt=0.5), monkeypatch, True)
    assert tune["sites"]
    ref = oracle.Oracle("port").solve(p, p.rho0_ground(), t, solver="lsrk4", dt=0.5)[-1]
    assert np.abs(got - ref).max() <= 1e-6
