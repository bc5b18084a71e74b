"""Redfield models on the GPU against the reference's own redfield_hilb /
redfield_liou (golden fixtures): one right-hand side and propagations."""
import glob
import os

import numpy as np
import pytest

import libheom_gb300 as lh
from _cases import params_from_npz

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
FORMS = ("redfield_hilb", "redfield_liou")


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLD, "redfield_diff_*.npz"))))
@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 2e-5)])
def test_redfield_rhs_vs_reference(path, form, precision, tol):
    z = np.load(path)
    q = lh.from_params(params_from_npz(z), form=form, precision=precision)
    assert q.get_n_hrchy() == 1 and q.main_size() == z["rho"].size
    got = q.calc_diff(z["rho"], complex(z["alpha"]), complex(z["beta"]), drho=z["drho"])
    ref = z[f"out_{form}"]
    assert np.abs(got - ref).max() <= tol * np.abs(ref).max()


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLD, "redfield_solve_*.npz"))))
@pytest.mark.parametrize("form", FORMS)
def test_redfield_solve_vs_reference(path, form):
    z = np.load(path)
    p = params_from_npz(z)
    solver = str(z["solver"])
    q = lh.from_params(p, form=form)
    qs = lh.qme_solver(q, lh.SOLVERS[solver]())
    rho = np.array(z["rho0"], dtype=np.complex128, copy=True)
    seen = []
    qs.solve(rho, z["t_list"], lambda t: seen.append(rho.copy()),
             {"dt": float(z["dt"]), "atol": float(z["atol"]), "rtol": float(z["rtol"])})
    ref = z[f"rho_t_{form}"]
    assert np.abs(np.array(seen) - ref).max() <= 1e-10 * np.abs(ref).max()
    # trace and hermiticity of the Redfield state are kept
    assert abs(np.trace(rho[0]) - 1.0) <= 1e-10
    assert np.abs(rho[0] - rho[0].conj().T).max() <= 1e-10


def test_redfield_rejects_non_hermitian_h():
    z = np.load(os.path.join(GOLD, "redfield_diff_spin_boson.npz"))
    p = params_from_npz(z)
    p.H = p.H + np.array([[0, 0.1], [0, 0]])
    with pytest.raises(lh.HeomError):
        lh.from_params(p, form="redfield_hilb")
