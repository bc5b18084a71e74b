"""Parity of the CUDA path (through the C ABI) with the reference's own code
(golden fixtures) and with the CPU restatement on larger cases.

Tolerances: FP64 results agree to 1e-12 relative for one right-hand side and
to 1e-10 (relative to the largest element of each ADO) for trajectories; the
mixed-precision form (FP32 bulk products, FP64 state) to 2e-5 for one
right-hand side."""
import glob
import os

import numpy as np
import pytest

import libheom_gb300 as lh
import oracle
from _cases import generic_case, params_from_npz, projector_case
from libheom_gb300 import configs
from libheom_gb300.noise import drude_lorentz_terms, noise_members
from libheom_gb300.params import HeomParams

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def port():
    return oracle.Oracle("port")


def k_mode_params(K, N, U=1):
    """n=2 system with K modes split over U baths."""
    nu, c = drude_lorentz_terms(0.5, 1.0, 1.0, K - 1)
    per = np.array_split(np.arange(K), U)
    gam, phi, sig, S, A = [], [], [], [], []
    for idx in per:
        g, p, s, Sm, Am, _ = noise_members(nu[idx], c[idx])
        gam.append(g); phi.append(p); sig.append(s); S.append(Sm); A.append(Am)
    V = [np.diag([1.0, -1.0]).astype(complex)] * U
    return HeomParams(H=np.array([[0, 1], [1, 0]], complex), V=V, gamma=gam, phi_0=phi, sigma=sig, S=S, A=A,
                      s_delta=[0j] * U, max_depth=N)


def rel_err(got, ref):
    return np.abs(got - ref).max() / np.abs(ref).max()


def ado_rel_err(got, ref):
    scale = np.abs(ref).max(axis=(-2, -1), keepdims=True) + 1e-300
    return (np.abs(got - ref) / scale).max()


@pytest.mark.parametrize("K,N,U", [(3, 10, 1), (14, 4, 7), (5, 3, 2), (4, 6, 1), (1, 5, 1), (2, 0, 1), (6, 5, 3),
                                   (48, 3, 24)])
def test_device_hierarchy_bit_exact(port, K, N, U):
    q = lh.from_params(k_mode_params(K, N, U))
    n, p1, m1 = q.hrchy()
    rn, rp1, rm1 = port.hrchy(K, N)
    assert np.array_equal(n, rn) and np.array_equal(p1, rp1) and np.array_equal(m1, rm1)


def test_device_hierarchy_matches_reference_fixture():
    z = np.load(os.path.join(GOLD, "hrchy.npz"))
    for key in z.files:
        if key.startswith("n_"):
            _, K, N = key.split("_")
            q = lh.from_params(k_mode_params(int(K), int(N)))
            n, p1, m1 = q.hrchy()
            assert np.array_equal(n, z[key]) and np.array_equal(p1, z[f"p1_{K}_{N}"])
            assert np.array_equal(m1, z[f"m1_{K}_{N}"])


def _ref_key(z, key, form):
    """Fixture output of `form`; col_major fixtures hold heom_hilb only, and the
    Liouville forms apply the same operator, so they are checked against it."""
    return z[f"{key}_{form}"] if f"{key}_{form}" in z.files else z[f"{key}_hilb"]


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLD, "diff_*.npz"))))
@pytest.mark.parametrize("form", ["hilb", "liou", "ado"])
def test_calc_diff_fp64_vs_reference(path, form):
    z = np.load(path)
    q = lh.from_params(params_from_npz(z), form=form)
    got = q.calc_diff(z["rho"], complex(z["alpha"]), complex(z["beta"]), drho=z["drho"])
    assert rel_err(got, _ref_key(z, "out", form)) <= 1e-12
    got0 = q.calc_diff(z["rho"])
    assert rel_err(got0, _ref_key(z, "out0", form)) <= 1e-12


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLD, "diff_*.npz"))))
@pytest.mark.parametrize("form", ["hilb", "liou"])
def test_calc_diff_mixed_vs_reference(path, form):
    z = np.load(path)
    q = lh.from_params(params_from_npz(z), form=form, precision="mixed")
    got = q.calc_diff(z["rho"], complex(z["alpha"]), complex(z["beta"]), drho=z["drho"])
    assert rel_err(got, _ref_key(z, "out", form)) <= 2e-5


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLD, "solve_*.npz"))))
def test_solve_fp64_vs_reference(path):
    z = np.load(path)
    p = params_from_npz(z)
    solver = str(z["solver"])
    for key in z.files:
        if not key.startswith("rho_t_"):
            continue
        form = key[len("rho_t_"):]
        q = lh.from_params(p, form=form)
        qs = lh.qme_solver(q, lh.SOLVERS[solver]())
        rho = np.array(z["rho0"], dtype=np.complex128, copy=True)
        seen = []
        qs.solve(rho, z["t_list"], lambda t: seen.append((t, rho.copy())),
                 {"dt": float(z["dt"]), "atol": float(z["atol"]), "rtol": float(z["rtol"])})
        got = np.array([s[1] for s in seen])
        assert [s[0] for s in seen] == list(z["t_list"])
        assert ado_rel_err(got, z[key]) <= 1e-10, form


def test_generic_rhs_larger_depth_vs_port(port):
    p = generic_case()
    p.max_depth = 6
    rng = np.random.default_rng(3)
    shape = (p.n_hrchy(), 3, 3)
    rho = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    ref = port.calc_diff(p, rho)
    for form in ("hilb", "liou", "ado"):
        assert rel_err(lh.from_params(p, form=form).calc_diff(rho), ref) <= 1e-12


def test_aggregate24_full_size_rhs_vs_port(port):
    p = configs.aggregate_24site()
    rng = np.random.default_rng(4)
    shape = (p.n_hrchy(), 24, 24)
    rho = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) * 0.01
    ref = port.calc_diff(p, rho)
    got = lh.from_params(p).calc_diff(rho)
    assert rel_err(got, ref) <= 1e-12
    gotm = lh.from_params(p, precision="mixed").calc_diff(rho)
    assert rel_err(gotm, ref) <= 2e-5


def test_exciton7_full_depth_dp_vs_port(port):
    p = configs.exciton_7site()
    t = [0.0, 5.0, 10.0]
    kw = dict(dt=0.1, atol=1e-8, rtol=1e-8)
    ref, st = port.solve(p, p.rho0_ground(), t, solver="rkdp", with_stats=True, **kw)
    q = lh.from_params(p)
    qs = lh.qme_solver(q, lh.rkdp())
    rho = p.rho0_ground()
    qs.solve(rho, t, None, kw)
    assert ado_rel_err(rho, ref[-1]) <= 1e-10
    assert qs.stats()["attempts"] == st["attempts"]


def test_spin_boson_full_rk4_vs_port(port):
    p = configs.spin_boson()
    t = [0.0, 10.0]
    ref = port.solve(p, p.rho0_ground(), t, solver="rk4", dt=0.005)
    q = lh.from_params(p)
    qs = lh.qme_solver(q, lh.rk4())
    rho = p.rho0_ground()
    qs.solve(rho, t, None, {"dt": 0.005})
    assert ado_rel_err(rho, ref[-1]) <= 1e-10
    assert qs.stats()["rhs"] == 4 * 2000


def test_projector_lsrk4_liou_vs_port(port):
    p = projector_case(depth=4)
    t = [0.0, 0.5, 1.0]
    ref = port.solve(p, p.rho0_ground(), t, solver="lsrk4", dt=0.01)
    for form in ("hilb", "liou", "ado"):
        qs = lh.qme_solver(lh.from_params(p, form=form), lh.lsrk4())
        rho = p.rho0_ground()
        qs.solve(rho, t, None, {"dt": 0.01})
        assert ado_rel_err(rho, ref[-1]) <= 1e-10, form


def test_missing_kwarg_is_an_error():
    p = configs.spin_boson(depth=3)
    qs = lh.qme_solver(lh.from_params(p), lh.rkdp())
    rho = p.rho0_ground()
    with pytest.raises(lh.HeomError):
        qs.solve(rho, [0.0, 1.0], None, {"dt": 0.01, "atol": 1e-8})   # rtol missing
