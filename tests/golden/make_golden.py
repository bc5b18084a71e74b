"""Generate the golden fixtures of tests/golden/ from the reference's own code.

Runs the reference's unmodified hierarchy / model / integrator sources, built
by `make -C oracle ref` from the reference tree with the plain-loop harness
engine, on small seeded cases and stores inputs and outputs as .npz files.
Needs the reference tree, so it runs where that tree exists; the fixtures it
writes are committed and are all the tests need elsewhere.

    python tests/golden/make_golden.py            # every fixture
    python tests/golden/make_golden.py horizon    # only the 1 ps horizon fixture
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from libheom_gb300 import configs  # noqa: E402
from libheom_gb300.params import HeomParams  # noqa: E402

sys.path.insert(0, os.path.dirname(HERE))
from _cases import FILTERS, generic_case, projector_case, params_to_dict  # noqa: E402


def hrchy_fixture(ref: oracle.Oracle):
    out = {}
    for K, N in [(3, 10), (14, 4), (5, 3), (4, 6), (1, 5), (2, 0), (6, 5), (7, 2)]:
        n, p1, m1 = ref.hrchy(K, N)
        out[f"n_{K}_{N}"] = n
        out[f"p1_{K}_{N}"] = p1
        out[f"m1_{K}_{N}"] = m1
    for K, N in [(48, 3), (14, 6)]:
        n, p1, m1 = ref.hrchy(K, N)
        h = hashlib.sha256()
        for a in (n, p1, m1):
            h.update(np.ascontiguousarray(a, dtype="<i4").tobytes())
        out[f"sha_{K}_{N}"] = np.frombuffer(h.digest(), dtype=np.uint8)
        out[f"count_{K}_{N}"] = np.array(n.shape[0])
    np.savez_compressed(os.path.join(HERE, "hrchy.npz"), **out)


def diff_fixture(ref, name, p: HeomParams, seed, forms=("hilb", "liou", "ado")):
    rng = np.random.default_rng(seed)
    shape = (p.n_hrchy(), p.n_level, p.n_level)
    rho = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    drho = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    alpha, beta = 0.7 - 0.2j, 0.3 + 0.1j
    out = dict(params_to_dict(p), rho=rho, drho=drho, alpha=np.array(alpha), beta=np.array(beta))
    for form in forms:
        out[f"out_{form}"] = ref.calc_diff(p, rho, drho, alpha, beta, form=form, threads=4)
        out[f"out0_{form}"] = ref.calc_diff(p, rho, None, 1.0, 0.0, form=form, threads=4)
    np.savez_compressed(os.path.join(HERE, f"diff_{name}.npz"), **out)


def solve_fixture(ref, name, p: HeomParams, solver, t_list, dt, atol=1e-8, rtol=1e-8, forms=("hilb",), rho0=None):
    rho0 = p.rho0_ground() if rho0 is None else rho0
    out = dict(params_to_dict(p), rho0=rho0, t_list=np.asarray(t_list, float), dt=np.array(dt),
               atol=np.array(atol), rtol=np.array(rtol), solver=np.array(solver))
    for form in forms:
        out[f"rho_t_{form}"] = ref.solve(p, rho0, t_list, solver=solver, dt=dt, atol=atol, rtol=rtol, form=form,
                                         threads=4)
    np.savez_compressed(os.path.join(HERE, f"solve_{name}.npz"), **out)


def sqrt_fixtures():
    """The reference built with LIBHEOM_SQRT_NORMALIZATION on the same cases."""
    import dataclasses
    ref = oracle.Oracle("ref_sqrt")
    sq = lambda p: dataclasses.replace(p, normalization="sqrt")
    diff_fixture(ref, "generic_sqrt", sq(generic_case()), 31)
    diff_fixture(ref, "spin_boson_sqrt", sq(configs.spin_boson(depth=4)), 33)
    solve_fixture(ref, "spin_boson_rk4_sqrt", sq(configs.spin_boson()), "rk4", [0.0, 0.25, 0.5], 0.005,
                  forms=("hilb", "liou", "ado"))
    solve_fixture(ref, "exciton7_rkdp_sqrt", sq(configs.exciton_7site(depth=2)), "rkdp", [0.0, 10.0, 20.0], 0.1,
                  atol=1e-8, rtol=1e-8)


def col_major_fixtures(ref):
    """heom_hilb instantiated with the reference's col_major order (ADOs stored
    column-major); the harness provides that order's set-up algebra for
    heom_hilb only."""
    import dataclasses
    cm = lambda p: dataclasses.replace(p, order="col_major")
    diff_fixture(ref, "generic_colmajor", cm(generic_case()), 41, forms=("hilb",))
    diff_fixture(ref, "spin_boson_colmajor", cm(configs.spin_boson(depth=4)), 43, forms=("hilb",))
    solve_fixture(ref, "spin_boson_rkdp_colmajor", cm(configs.spin_boson(eps=0.4)), "rkdp", [0.0, 0.5, 1.0], 0.01,
                  atol=1e-8, rtol=1e-6)
    g = cm(generic_case())
    rng = np.random.default_rng(22)
    r0 = np.zeros((g.n_hrchy(), g.n_level, g.n_level), complex)
    v = rng.standard_normal(g.n_level) + 1j * rng.standard_normal(g.n_level)
    r0[0] = np.outer(v, v.conj()).T / np.vdot(v, v).real   # column-major storage of |v><v|
    solve_fixture(ref, "generic_rk4_colmajor", g, "rk4", [0.0, 0.1, 0.2], 0.01, rho0=r0)


def redfield_fixtures(ref):
    """The reference's redfield_hilb / redfield_liou (no hierarchy: one n x n state)."""
    import dataclasses
    forms = ("redfield_hilb", "redfield_liou")
    for name, p, seed in [("spin_boson", configs.spin_boson(eps=0.4, depth=0), 51),
                          ("exciton7", configs.exciton_7site(depth=0), 52),
                          ("generic", dataclasses.replace(generic_case(), max_depth=0), 53)]:
        rng = np.random.default_rng(seed)
        n = p.n_level
        rho = rng.standard_normal((1, n, n)) + 1j * rng.standard_normal((1, n, n))
        drho = rng.standard_normal((1, n, n)) + 1j * rng.standard_normal((1, n, n))
        alpha, beta = 0.7 - 0.2j, 0.3 + 0.1j
        out = dict(params_to_dict(p), rho=rho, drho=drho, alpha=np.array(alpha), beta=np.array(beta))
        for form in forms:
            out[f"out_{form}"] = ref.calc_diff(p, rho, drho, alpha, beta, form=form, threads=1)
        np.savez_compressed(os.path.join(HERE, f"redfield_diff_{name}.npz"), **out)
    for name, p, solver, t_list, dt in [
            ("spin_boson_rk4", configs.spin_boson(eps=0.4, depth=0), "rk4", [0.0, 1.0, 2.0], 0.005),
            ("exciton7_rkdp", configs.exciton_7site(depth=0), "rkdp", [0.0, 50.0, 100.0], 0.1)]:
        rho0 = p.rho0_ground()
        out = dict(params_to_dict(p), rho0=rho0, t_list=np.asarray(t_list, float), dt=np.array(dt),
                   atol=np.array(1e-8), rtol=np.array(1e-8), solver=np.array(solver))
        for form in forms:
            out[f"rho_t_{form}"] = ref.solve(p, rho0, t_list, solver=solver, dt=dt, atol=1e-8, rtol=1e-8, form=form,
                                             threads=1)
        np.savez_compressed(os.path.join(HERE, f"redfield_solve_{name}.npz"), **out)


def filter_fixture(ref):
    """alloc_hrchy_space with the filters of tests/_cases.py (filter_flag on)."""
    out = {}
    for name, (K, N, f) in FILTERS.items():
        n, p1, m1 = ref.hrchy(K, N, f)
        out[f"n_{name}"], out[f"p1_{name}"], out[f"m1_{name}"] = n, p1, m1
    np.savez_compressed(os.path.join(HERE, "hrchy_filtered.npz"), **out)


def horizon_fixture(ref):
    """The default measured workload at its own size and horizon: the 7-site
    aggregate (depth 4, 3060 ADOs), Dormand-Prince atol=rtol=1e-8 to 1 ps.
    Stored: the ADOs of tiers 0 and 1, every 17th ADO and the largest |rho|
    of every tier, so that the fixture stays small."""
    p = configs.exciton_7site()
    kw = dict(dt=0.1, atol=1e-8, rtol=1e-8)
    rho_t = ref.solve(p, p.rho0_ground(), [0.0, 1000.0], solver="rkdp", **kw)
    final = rho_t[-1]
    n, _, _ = ref.hrchy(p.n_modes, p.max_depth)
    tiers = n.sum(axis=1)
    idx = np.union1d(np.arange(0, 1 + p.n_modes), np.arange(0, p.n_hrchy(), 17))
    out = dict(t_final=np.array(1000.0), dt=np.array(kw["dt"]), atol=np.array(kw["atol"]),
               rtol=np.array(kw["rtol"]), ado_index=idx, ados=final[idx],
               tier_max=np.array([np.abs(final[tiers == d]).max() for d in range(p.max_depth + 1)]))
    np.savez_compressed(os.path.join(HERE, "horizon_exciton7_rkdp_1ps.npz"), **out)


def main():
    oracle.build("ref")
    ref = oracle.Oracle("ref")
    if sys.argv[1:] == ["horizon"]:  # only the horizon fixture (the others are unchanged)
        horizon_fixture(ref)
        return
    horizon_fixture(ref)
    hrchy_fixture(ref)
    diff_fixture(ref, "generic", generic_case(), 11)
    diff_fixture(ref, "projector", projector_case(), 12)
    diff_fixture(ref, "spin_boson", configs.spin_boson(depth=4), 13)
    sb = configs.spin_boson()
    solve_fixture(ref, "spin_boson_rk4", sb, "rk4", [0.0, 0.25, 0.5], 0.005, forms=("hilb", "liou", "ado"))
    solve_fixture(ref, "spin_boson_lsrk4", sb, "lsrk4", [0.0, 0.25, 0.5], 0.005)
    solve_fixture(ref, "spin_boson_rkdp", sb, "rkdp", [0.0, 0.5, 1.0], 0.01, atol=1e-8, rtol=1e-6)
    sbx = configs.spin_boson(eps=0.5, coupling="x", depth=6)
    solve_fixture(ref, "spin_boson_x_rk4", sbx, "rk4", [0.0, 0.2, 0.4], 0.01, forms=("hilb", "liou"))
    ex = configs.exciton_7site(depth=2)
    solve_fixture(ref, "exciton7_rkdp", ex, "rkdp", [0.0, 10.0, 20.0], 0.1, atol=1e-8, rtol=1e-8)
    g = generic_case()
    rng = np.random.default_rng(21)
    r0 = np.zeros((g.n_hrchy(), g.n_level, g.n_level), complex)
    v = rng.standard_normal(g.n_level) + 1j * rng.standard_normal(g.n_level)
    r0[0] = np.outer(v, v.conj()) / np.vdot(v, v).real
    solve_fixture(ref, "generic_rk4", g, "rk4", [0.0, 0.1, 0.2], 0.01, forms=("hilb", "liou", "ado"), rho0=r0)
    solve_fixture(ref, "generic_rkdp", g, "rkdp", [0.0, 0.2, 0.4], 0.02, atol=1e-9, rtol=1e-7, rho0=r0)
    solve_fixture(ref, "generic_lsrk4", g, "lsrk4", [0.0, 0.1, 0.2], 0.01, rho0=r0)
    sqrt_fixtures()
    col_major_fixtures(ref)
    redfield_fixtures(ref)
    filter_fixture(ref)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
