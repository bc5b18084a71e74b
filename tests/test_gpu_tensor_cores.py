"""Tensor-core commutators of the mixed form (3xTF32 tcgen05 MMAs, FP32
accumulation in tensor memory) against the CUDA-core FP32 kernel and the FP64
drop-in on the same seeded aggregates.

The commutator is the only term that changes; the mixed form's budget holds
for both variants: the system block within 1e-6 of FP64 relative to its
largest element, and the tensor-core error no worse than a small multiple of
the CUDA-core one."""
import numpy as np
import pytest

import libheom_gb300 as lh
from libheom_gb300 import configs

pytestmark = pytest.mark.gpu


def solve(p, precision, tile, monkeypatch, solver="rk4", t=(0.0, 10.0), dt=0.5):
    if tile is None:
        monkeypatch.delenv("HEOMGB_TILE", raising=False)
    else:
        monkeypatch.setenv("HEOMGB_TILE", tile)
    q = lh.from_params(p, precision=precision)
    qs = lh.qme_solver(q, lh.SOLVERS[solver]())
    rho = p.rho0_ground()
    kw = {"dt": dt}
    if solver == "rkdp":
        kw.update(atol=1e-10, rtol=1e-10)
    qs.solve(rho, list(t), None, kw)
    monkeypatch.delenv("HEOMGB_TILE", raising=False)
    return rho.reshape(p.n_hrchy(), p.n_level, p.n_level), qs.tuning(), q


@pytest.mark.parametrize("n_sites", [8, 12, 16, 24, 32])
def test_tensor_core_commutator_matches_cuda_cores(n_sites, monkeypatch):
    p = configs.aggregate_24site(n_sites=n_sites, depth=2)
    ref, _, _ = solve(p, "fp64", None, monkeypatch)
    cc, tune_cc, _ = solve(p, "mixed", "256x1", monkeypatch)
    tc, tune_tc, q = solve(p, "mixed", "tc", monkeypatch)
    assert q.get_precision()["effective"] == "mixed"
    assert tune_tc["tensor_cores"] and not tune_cc["tensor_cores"]
    assert np.all(np.isfinite(tc))
    scale = np.abs(ref[0]).max()
    err_cc = np.abs(cc[0] - ref[0]).max() / scale
    err_tc = np.abs(tc[0] - ref[0]).max() / scale
    assert err_tc <= 1e-6, (err_tc, err_cc)
    assert err_tc <= max(4.0 * err_cc, 1e-7), (err_tc, err_cc)
    # every ADO, not only the system block: relative to the ADO's largest element
    for l in range(0, p.n_hrchy(), max(1, p.n_hrchy() // 17)):
        s = np.abs(ref[l]).max() + 1e-300
        assert np.abs(tc[l] - ref[l]).max() / s <= 1e-4


@pytest.mark.parametrize("solver,dt", [("lsrk4", 0.5), ("rkdp", 0.25)])
def test_tensor_core_commutator_other_integrators(solver, dt, monkeypatch):
    p = configs.aggregate_24site(n_sites=24, depth=2)
    ref, _, _ = solve(p, "fp64", None, monkeypatch, solver=solver, dt=dt)
    tc, tune, _ = solve(p, "mixed", "tc", monkeypatch, solver=solver, dt=dt)
    assert tune["tensor_cores"]
    scale = np.abs(ref[0]).max()
    assert np.abs(tc[0] - ref[0]).max() / scale <= 1e-6


def test_tensor_core_batch_of_uneven_aggregates(monkeypatch):
    ps = [configs.aggregate_24site(seed=s, n_sites=n, depth=2) for s, n in ((3, 8), (4, 24), (5, 12), (6, 8))]
    monkeypatch.setenv("HEOMGB_TILE", "tc")
    qmes = [lh.from_params(p, precision="mixed") for p in ps]
    bs = lh.batch_solver(qmes, lh.rk4())
    rho = np.concatenate([p.rho0_ground().ravel() for p in ps])
    bs.solve(rho, [0.0, 10.0], None, {"dt": 0.5})
    monkeypatch.delenv("HEOMGB_TILE")
    assert bs.tuning()["tensor_cores"]
    off = bs.offsets()
    for i, p in enumerate(ps):
        ref, _, _ = solve(p, "fp64", None, monkeypatch)
        got = rho[off[i]:off[i + 1]].reshape(p.n_hrchy(), p.n_level, p.n_level)
        assert np.abs(got[0] - ref[0]).max() / np.abs(ref[0]).max() <= 1e-6


def test_tensor_core_pin_rejected_where_it_does_not_apply(monkeypatch):
    p = configs.exciton_7site(depth=2)  # n_state 7: not a micro-tiled size
    monkeypatch.setenv("HEOMGB_TILE", "tc")
    q = lh.from_params(p, precision="mixed")
    with pytest.raises(lh.HeomError):
        qs = lh.qme_solver(q, lh.rk4())
        rho = p.rho0_ground()
        qs.solve(rho, [0.0, 1.0], None, {"dt": 0.5})
    q64 = lh.from_params(configs.aggregate_24site(n_sites=8, depth=2), precision="fp64")
    with pytest.raises(lh.HeomError):  # FP64 has no tensor-core variant
        qs = lh.qme_solver(q64, lh.rk4())
        rho = np.zeros(qs.main_size(), dtype=np.complex128)
        qs.solve(rho, [0.0, 1.0], None, {"dt": 0.5})
