"""Resident Dormand-Prince interval (one cooperative launch per output
interval, every CTA holding its ADOs' state in shared memory between stages)
against the per-stage kernels and the FP64 path on the same models.

Both mixed-form variants do the same per-element arithmetic in the same order;
they can differ only through the order of the error norm's sum over
elements, which moves step sizes by rounding.  Budget: the system block
within 1e-6 of FP64 (relative to its largest element), the two variants
within 1e-6 of each other per ADO, attempt counts within two."""
import dataclasses

import numpy as np
import pytest

import libheom_gb300 as lh
from libheom_gb300 import configs

pytestmark = pytest.mark.gpu
KW = dict(dt=0.1, atol=1e-8, rtol=1e-8)


def run(p, t, monkeypatch, resident, precision="mixed", kw=KW):
    monkeypatch.setenv("HEOMGB_RESIDENT", "1" if resident else "0")
    q = lh.from_params(p, precision=precision)
    qs = lh.qme_solver(q, lh.rkdp())
    rho = p.rho0_ground()
    seen = []
    qs.solve(rho, list(t), lambda tt: seen.append(tt), dict(kw))
    monkeypatch.delenv("HEOMGB_RESIDENT")
    assert seen == list(t)
    return rho.reshape(p.n_hrchy(), p.n_level, p.n_level), qs.stats(), qs.tuning()


def ado_rel(a, b):
    scale = np.abs(b).max(axis=(1, 2), keepdims=True) + 1e-300
    return float((np.abs(a - b) / scale).max())


def compare(p, t, monkeypatch, kw=KW):
    res, st_r, tune_r = run(p, t, monkeypatch, True, kw=kw)
    stg, st_s, tune_s = run(p, t, monkeypatch, False, kw=kw)
    ref, _, _ = run(p, t, monkeypatch, False, precision="fp64", kw=kw)
    assert tune_r["resident"] and tune_r["resident_grid"] >= 1
    assert not tune_s["resident"]
    assert np.all(np.isfinite(res))
    assert abs(st_r["attempts"] - st_s["attempts"]) <= 2
    assert st_r["rhs"] == 7 * st_r["attempts"]
    scale = np.abs(ref[0]).max()
    assert np.abs(res[0] - ref[0]).max() / scale <= 1e-6
    assert ado_rel(res, stg) <= 1e-6
    return st_r


def test_resident_exciton7_matches_stage_kernels(monkeypatch):
    st = compare(configs.exciton_7site(), [0.0, 5.0, 10.0, 20.0], monkeypatch)
    assert st["accepted"] >= 1


def test_resident_complex_hamiltonian_sqrt_normalisation(monkeypatch):
    p = configs.exciton_7site(depth=3)
    rng = np.random.default_rng(11)
    X = rng.uniform(-0.05, 0.05, (7, 7))
    p = dataclasses.replace(p, H=p.H + 1j * (X - X.T), normalization="sqrt")
    compare(p, [0.0, 4.0, 8.0], monkeypatch)


def test_resident_filtered_hierarchy_col_major(monkeypatch):
    """A filtered hierarchy (missing neighbours are sentinels in the term
    table) with column-major ADOs at the boundary."""
    p = configs.exciton_7site(depth=4)

    def keep(idx, depth):  # drop the Matsubara modes' second excitations
        return all(idx[k] <= 1 for k in range(1, len(idx), 2))

    p = dataclasses.replace(p, hrchy_filter=keep, order="col_major")
    assert p.n_hrchy() < configs.exciton_7site(depth=4).n_hrchy()
    compare(p, [0.0, 5.0, 10.0], monkeypatch)


def test_resident_spin_boson(monkeypatch):
    p = configs.spin_boson(depth=8)
    compare(p, [0.0, 2.0, 4.0], monkeypatch, kw=dict(dt=0.01, atol=1e-9, rtol=1e-9))


@pytest.mark.parametrize("ept", ["1", "2"])
def test_resident_first_attempt_bit_identical(ept, monkeypatch):
    """One accepted attempt: the per-element arithmetic is the stage kernels',
    so the state agrees bit for bit; the step size may differ in the last bit
    (the error norm's sum runs in another order)."""
    p = configs.spin_boson(depth=8)
    kw = dict(dt=0.01, atol=1e-9, rtol=1e-9)
    monkeypatch.setenv("HEOMGB_RESIDENT_EPT", ept)
    res, st_r, tune = run(p, [0.0, 0.01], monkeypatch, True, kw=kw)
    monkeypatch.delenv("HEOMGB_RESIDENT_EPT")
    stg, st_s, _ = run(p, [0.0, 0.01], monkeypatch, False, kw=kw)
    assert tune["resident"]
    assert st_r["attempts"] == st_s["attempts"] == 1
    assert np.array_equal(res, stg)
    assert abs(st_r["dt_save"] - st_s["dt_save"]) <= 1e-12 * abs(st_s["dt_save"])


def test_resident_only_where_it_applies(monkeypatch):
    p = configs.spin_boson(depth=4)  # V = sigma_z: not a site-local bath
    _, _, tune = run(p, [0.0, 0.1], monkeypatch, True, precision="fp64", kw=dict(dt=0.01, atol=1e-9, rtol=1e-9))
    assert not tune["resident"]  # Dormand-Prince in the FP64 form keeps the stage kernels there
    p7 = configs.exciton_7site(depth=2)
    _, _, tune7 = run(p7, [0.0, 1.0], monkeypatch, True, precision="fp64")
    assert tune7["resident"]  # site-local baths: the FP64 resident interval
    monkeypatch.setenv("HEOMGB_RESIDENT", "1")
    qs = lh.qme_solver(lh.from_params(p7, precision="fp64"), lh.lsrk4())
    assert not qs.tuning()["resident"]  # LSRK4 in the FP64 form keeps the stage kernels


@pytest.mark.parametrize("ept", ["1", "2"])
def test_fp64_resident_dp_first_attempt_bit_identical(ept, monkeypatch):
    """The FP64 form's resident Dormand-Prince interval (site-local baths):
    one accepted attempt gives the stage kernels' state bit for bit."""
    p = configs.exciton_7site(depth=3)
    monkeypatch.setenv("HEOMGB_RESIDENT_EPT", ept)
    res, st_r, tune = run(p, [0.0, 0.1], monkeypatch, True, precision="fp64")
    monkeypatch.delenv("HEOMGB_RESIDENT_EPT")
    stg, st_s, _ = run(p, [0.0, 0.1], monkeypatch, False, precision="fp64")
    assert tune["resident"]
    assert st_r["attempts"] == st_s["attempts"] == 1
    assert np.array_equal(res, stg)
    assert abs(st_r["dt_save"] - st_s["dt_save"]) <= 1e-12 * abs(st_s["dt_save"])


FP64_CASES = {
    "exciton7_depth4": lambda: configs.exciton_7site(),
    "complex_h_sqrt": lambda: dataclasses.replace(
        configs.exciton_7site(depth=3), normalization="sqrt",
        H=configs.exciton_7site(depth=3).H + 1j * 0.02 * (np.triu(np.ones((7, 7)), 1) - np.tril(np.ones((7, 7)), -1))),
    "filtered_col_major": lambda: dataclasses.replace(
        configs.exciton_7site(depth=4), order="col_major",
        hrchy_filter=lambda idx, d: all(idx[k] <= 1 for k in range(1, len(idx), 2))),
}


@pytest.mark.parametrize("case", sorted(FP64_CASES))
def test_fp64_resident_dp_matches_stage_kernels(case, monkeypatch):
    """Several output intervals: the same per-element arithmetic as the stage
    kernels; only the error norm's sum order differs (step sizes may move in
    the last bits), so 1e-10 of the state's largest element and attempts within two."""
    p = FP64_CASES[case]()
    t = [0.0, 5.0, 10.0, 20.0]
    res, st_r, tune = run(p, t, monkeypatch, True, precision="fp64")
    stg, st_s, _ = run(p, t, monkeypatch, False, precision="fp64")
    assert tune["resident"]
    assert abs(st_r["attempts"] - st_s["attempts"]) <= 2
    assert st_r["rhs"] == 7 * st_r["attempts"]
    assert np.abs(res - stg).max() <= 1e-10 * np.abs(stg).max()


@pytest.mark.parametrize("form", ["mixed", "rk4_fp64"])
@pytest.mark.parametrize("solver", ["rk4", "lsrk4"])
@pytest.mark.parametrize("ept", ["1", "2"])
@pytest.mark.parametrize("maker", ["spin_boson", "exciton"])
def test_resident_fixed_step_bit_identical(maker, ept, solver, form, monkeypatch):
    """Fixed-step RK4 / LSRK4 in one resident launch per interval: the same
    per-element arithmetic as the stage kernels and no step control, so every
    ADO agrees bit for bit after many steps, the clamped last step included."""
    if form == "rk4_fp64" and solver != "rk4":
        pytest.skip("the FP64 form has a resident kernel for RK4 only")
    precision = "fp64" if form == "rk4_fp64" else "mixed"
    p = configs.spin_boson(depth=10) if maker == "spin_boson" else configs.exciton_7site(depth=3)
    dt = 0.005 if maker == "spin_boson" else 0.5
    t = [0.0, 37 * dt + 0.3 * dt, 60 * dt]  # the first interval ends with a shorter step

    def go(resident):
        monkeypatch.setenv("HEOMGB_RESIDENT", "1" if resident else "0")
        monkeypatch.setenv("HEOMGB_RESIDENT_EPT", ept)
        monkeypatch.setenv("HEOMGB_LOCAL", "0")  # the cooperative kernel under test, not the one-CTA plan
        q = lh.from_params(p, precision=precision)
        qs = lh.qme_solver(q, lh.SOLVERS[solver]())
        rho = p.rho0_ground()
        qs.solve(rho, t, None, {"dt": dt})
        return rho, qs.stats(), qs.tuning()

    res, st_r, tune = go(True)
    stg, st_s, _ = go(False)
    assert tune["resident"]
    assert st_r["rhs"] == st_s["rhs"]
    assert np.array_equal(res, stg)


@pytest.mark.parametrize("solver", ["lsrk4", "rk4"])
@pytest.mark.parametrize("ept,per_sm", [("1", "1"), ("1", "3"), ("1", "6"), ("2", "2"), ("2", "4")])
def test_resident_fixed_step_bit_identical_every_shape(solver, ept, per_sm, monkeypatch):
    """The resident fixed-step intervals give the stage kernels' bits at every
    grid shape (a shape changes which CTA owns which ADOs and how the threads
    of a CTA interleave; the LSRK4 kernel once lost a CTA barrier on its first
    stage and differed only at some shapes)."""
    p = configs.exciton_7site(depth=3)
    dt = 0.5
    t = [0.0, 37 * dt + 0.3 * dt, 60 * dt]

    def go(resident):
        monkeypatch.setenv("HEOMGB_RESIDENT", "1" if resident else "0")
        monkeypatch.setenv("HEOMGB_RESIDENT_EPT", ept)
        monkeypatch.setenv("HEOMGB_RESIDENT_PER_SM", per_sm)
        monkeypatch.setenv("HEOMGB_LOCAL", "0")
        qs = lh.qme_solver(lh.from_params(p, precision="mixed"), lh.SOLVERS[solver]())
        rho = p.rho0_ground()
        qs.solve(rho, t, None, {"dt": dt})
        return rho, qs.tuning()

    res, tune = go(True)
    stg, _ = go(False)
    assert tune["resident"]
    assert np.array_equal(res, stg)
