"""The numpy restatement of the Redfield models against the golden fixtures
written by the reference's own redfield_hilb / redfield_liou (CPU only)."""
import glob
import os

import numpy as np
import pytest

from _cases import params_from_npz
from oracle import redfield_oracle

GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLD, "redfield_diff_*.npz"))))
def test_redfield_rhs_restatement_matches_reference(path):
    z = np.load(path)
    p = params_from_npz(z)
    got = redfield_oracle.calc_diff(p, z["rho"], z["drho"], complex(z["alpha"]), complex(z["beta"]))
    for form in ("redfield_hilb", "redfield_liou"):
        ref = z[f"out_{form}"]
        assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max(), form
