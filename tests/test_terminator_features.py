"""Terminator input features: the package's vectorised numpy version (used to
build training data) against the oracle's per-ADO restatement (CPU only)."""
import numpy as np

import oracle
from libheom_gb300 import configs
from libheom_gb300 import terminator as T
from oracle import mlp_oracle


def test_terminator_features_match_numpy():
    p = configs.exciton_7site(depth=2)
    rng = np.random.default_rng(9)
    rho = (rng.standard_normal((p.n_hrchy(), 7, 7)) + 1j * rng.standard_normal((p.n_hrchy(), 7, 7)))
    n_tab, _, _ = oracle.Oracle("port").hrchy(p.n_modes, p.max_depth)
    first = int(np.argmax(n_tab.sum(1) == p.max_depth))
    X1, s1 = mlp_oracle.term_features(p, n_tab, rho, first)
    X2, s2 = T.features(p, n_tab, rho, first)
    assert np.abs(X1 - X2).max() <= 1e-5 * np.abs(X1).max()
    assert np.allclose(s1, s2, rtol=1e-6)
