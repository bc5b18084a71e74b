"""Hierarchy filter (alloc_hrchy_space's hrchy_filter, filter_flag on) on the
device: the compacted tables against the reference's filtered build, and the
filtered model's right-hand side and propagation against the oracle port."""
import dataclasses
import os

import numpy as np
import pytest

import libheom_gb300 as lh
import oracle
from _cases import FILTERS, generic_case
from libheom_gb300 import configs
from libheom_gb300.params import HeomParams

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _model_for(K, N, f):
    """A model with K modes: 7-site-like baths (2 modes each) or, for odd K, a
    3-mode bath plus 2-mode baths."""
    p = configs.exciton_7site(depth=N)
    n_baths = K // 2
    V = p.V[:n_baths]
    gam, phi, sig, S, A = (list(x[:n_baths]) for x in (p.gamma, p.phi_0, p.sigma, p.S, p.A))
    if K % 2:
        sb = configs.spin_boson()  # one 3-mode bath on site 0
        gam[0], phi[0], sig[0], S[0], A[0] = sb.gamma[0], sb.phi_0[0], sb.sigma[0], sb.S[0], sb.A[0]
    return HeomParams(H=p.H, V=V, gamma=gam, phi_0=phi, sigma=sig, S=S, A=A, s_delta=[0j] * n_baths,
                      max_depth=N, hrchy_filter=f)


@pytest.fixture(scope="module")
def port():
    return oracle.Oracle("port")


@pytest.mark.parametrize("name", sorted(FILTERS))
def test_filtered_tables_match_reference(name):
    z = np.load(os.path.join(GOLD, "hrchy_filtered.npz"))
    K, N, f = FILTERS[name]
    p = _model_for(K, N, f)
    assert p.n_modes == K
    q = lh.from_params(p)
    n, p1, m1 = q.hrchy()
    assert q.get_n_hrchy() == z[f"n_{name}"].shape[0] == p.n_hrchy()
    assert np.array_equal(n, z[f"n_{name}"])
    assert np.array_equal(p1, z[f"p1_{name}"])
    assert np.array_equal(m1, z[f"m1_{name}"])


@pytest.mark.parametrize("name", sorted(FILTERS))
@pytest.mark.parametrize("form", ["hilb", "liou"])
def test_filtered_rhs_vs_port(port, name, form):
    K, N, f = FILTERS[name]
    p = _model_for(K, N, f)
    rng = np.random.default_rng(3)
    shape = (p.n_hrchy(), p.n_level, p.n_level)
    rho = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    ref = port.calc_diff(p, rho)
    got = lh.from_params(p, form=form).calc_diff(rho)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
    got32 = lh.from_params(p, form=form, precision="mixed").calc_diff(rho)
    assert np.abs(got32 - ref).max() <= 2e-5 * np.abs(ref).max()


def test_filtered_solve_vs_port(port):
    K, N, f = FILTERS["weighted"]
    p = _model_for(K, N, f)
    ref = port.solve(p, p.rho0_ground(), [0.0, 20.0, 40.0], solver="rkdp", dt=0.1, atol=1e-8, rtol=1e-8)
    qs = lh.qme_solver(lh.from_params(p), lh.rkdp())
    rho = p.rho0_ground()
    seen = []
    qs.solve(rho, [0.0, 20.0, 40.0], lambda t: seen.append(rho.copy()), {"dt": 0.1, "atol": 1e-8, "rtol": 1e-8})
    got = np.array(seen)
    scale = np.abs(ref).max(axis=(2, 3), keepdims=True) + 1e-300
    assert (np.abs(got - ref) / scale).max() <= 1e-10


def test_filter_not_with_terminator():
    K, N, f = FILTERS["weighted"]
    p = _model_for(K, N, f)
    from libheom_gb300 import terminator as T
    din, dout = T.dims(p)
    q = lh.from_params(p)
    with pytest.raises(lh.HeomError):
        T.attach(q, T.MLP(din, 32, dout))
