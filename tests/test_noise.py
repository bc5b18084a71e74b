"""Noise decomposition and workload definitions."""
import math

import numpy as np
import pytest
from scipy import integrate

from libheom_gb300 import configs
from libheom_gb300.noise import drude_lorentz_terms, noise_members


def corr_numeric(t, lam, gc, beta):
    J = lambda w: 2 * lam * gc * w / (w * w + gc * gc)
    # Fourier-weighted quadrature (QAWF) for the oscillatory tails
    re = integrate.quad(lambda w: J(w) / math.tanh(beta * w / 2) / math.pi if w > 0 else 4 * lam / (beta * gc * math.pi),
                        0, np.inf, weight="cos", wvar=t)[0]
    im = -integrate.quad(lambda w: J(w) / math.pi, 0, np.inf, weight="sin", wvar=t)[0]
    return re + 1j * im


@pytest.mark.parametrize("t", [0.5, 1.0, 2.0])
def test_drude_lorentz_series_reproduces_correlation(t):
    lam, gc, beta = 0.5, 1.0, 1.0
    nu, c = drude_lorentz_terms(lam, gc, beta, 4000)
    series = np.sum(c * np.exp(-nu * t))
    assert abs(series - corr_numeric(t, lam, gc, beta)) < 2e-4


def test_noise_member_mapping():
    nu, c = drude_lorentz_terms(0.5, 1.0, 1.0, 2)
    g, phi, sig, S, A, sd = noise_members(nu, c)
    assert np.allclose(np.diag(g), nu) and np.allclose(phi, 1) and np.allclose(sig, 1)
    assert np.allclose(S @ phi, c.real) and np.allclose(A @ phi, c.imag) and sd == 0


def test_workload_sizes():
    assert configs.spin_boson().n_hrchy() == 286
    assert configs.exciton_7site().n_hrchy() == 3060
    assert configs.aggregate_24site().n_hrchy() == 20825
    ex = configs.exciton_7site()
    assert ex.n_modes == 14 and ex.n_noise == 7
    assert np.allclose(ex.H, ex.H.conj().T)
    sweep = configs.batched_sweep()
    counts = [p.n_hrchy() for p in sweep]
    assert len(sweep) == 1024 and min(counts) >= 15 and max(counts) <= 680
