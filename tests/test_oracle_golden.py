"""The CPU restatement (oracle/heom_oracle.cpp) against the golden fixtures
produced by the reference's own hierarchy/model/integrator code."""
import glob
import hashlib
import os

import numpy as np
import pytest

import oracle
from _cases import FILTERS, params_from_npz
from libheom_gb300 import configs

GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def port():
    return oracle.Oracle("port")


def test_hierarchy_tables_bit_exact(port):
    z = np.load(os.path.join(GOLD, "hrchy.npz"))
    for key in z.files:
        if not key.startswith("n_"):
            continue
        _, K, N = key.split("_")
        n, p1, m1 = port.hrchy(int(K), int(N))
        assert np.array_equal(n, z[f"n_{K}_{N}"])
        assert np.array_equal(p1, z[f"p1_{K}_{N}"])
        assert np.array_equal(m1, z[f"m1_{K}_{N}"])


def test_hierarchy_large_digest(port):
    z = np.load(os.path.join(GOLD, "hrchy.npz"))
    for key in z.files:
        if not key.startswith("sha_"):
            continue
        _, K, N = key.split("_")
        n, p1, m1 = port.hrchy(int(K), int(N))
        assert n.shape[0] == int(z[f"count_{K}_{N}"])
        h = hashlib.sha256()
        for a in (n, p1, m1):
            h.update(np.ascontiguousarray(a, dtype="<i4").tobytes())
        assert np.frombuffer(h.digest(), dtype=np.uint8).tobytes() == z[key].tobytes()


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLD, "diff_*.npz"))))
def test_calc_diff_matches_reference(port, path):
    z = np.load(path)
    p = params_from_npz(z)
    for form in ("hilb", "liou", "ado"):
        if f"out_{form}" not in z.files:   # col_major fixtures hold heom_hilb only
            continue
        got = port.calc_diff(p, z["rho"], z["drho"], complex(z["alpha"]), complex(z["beta"]), form=form)
        ref = z[f"out_{form}"]
        scale = np.abs(ref).max()
        assert np.abs(got - ref).max() <= 1e-12 * scale, form
        got0 = port.calc_diff(p, z["rho"], None, 1.0, 0.0, form=form)
        assert np.abs(got0 - z[f"out0_{form}"]).max() <= 1e-12 * np.abs(z[f"out0_{form}"]).max()


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLD, "solve_*.npz"))))
def test_solve_matches_reference(port, path):
    z = np.load(path)
    p = params_from_npz(z)
    solver = str(z["solver"])
    for key in z.files:
        if not key.startswith("rho_t_"):
            continue
        form = key[len("rho_t_"):]
        got = port.solve(p, z["rho0"], z["t_list"], solver=solver, dt=float(z["dt"]), atol=float(z["atol"]),
                         rtol=float(z["rtol"]), form=form)
        ref = z[key]
        # relative to the largest element of each ADO (deep tiers are tiny)
        scale = np.abs(ref).max(axis=(2, 3), keepdims=True) + 1e-300
        assert (np.abs(got - ref) / scale).max() <= 1e-10, form


@pytest.mark.parametrize("name", sorted(FILTERS))
def test_filtered_hierarchy_matches_reference(port, name):
    """The port's breadth-first build with a hierarchy filter against the
    reference's alloc_hrchy_space with filter_flag on."""
    z = np.load(os.path.join(GOLD, "hrchy_filtered.npz"))
    K, N, f = FILTERS[name]
    n, p1, m1 = port.hrchy(K, N, f)
    assert np.array_equal(n, z[f"n_{name}"])
    assert np.array_equal(p1, z[f"p1_{name}"])
    assert np.array_equal(m1, z[f"m1_{name}"])
    from libheom_gb300.params import hierarchy_indices
    assert [tuple(r) for r in n] == hierarchy_indices(K, N, f)


def test_port_vs_reference_at_1ps_horizon():
    """The CPU restatement against the reference's own code on the default
    measured workload at its full horizon (7-site, Dormand-Prince to 1 ps):
    identical attempt sequence, 1e-12 of the state's largest element."""
    z = np.load(os.path.join(GOLD, "horizon_exciton7_rkdp_1ps.npz"))
    p = configs.exciton_7site()
    rho = oracle.Oracle("port").solve(p, p.rho0_ground(), [0.0, float(z["t_final"])], solver="rkdp",
                                      dt=float(z["dt"]), atol=float(z["atol"]), rtol=float(z["rtol"]))[-1]
    got = rho[z["ado_index"]]
    assert np.abs(got - z["ados"]).max() / z["tier_max"].max() <= 1e-12
    n, _, _ = oracle.Oracle("port").hrchy(p.n_modes, p.max_depth)
    tiers = n.sum(axis=1)
    assert np.allclose([np.abs(rho[tiers == d]).max() for d in range(p.max_depth + 1)], z["tier_max"], rtol=1e-9)
