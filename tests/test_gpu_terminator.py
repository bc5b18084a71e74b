"""Learned terminator: the CUDA MLP kernels against the numpy oracle, and the
terminator's inference feeding the right-hand side."""
import numpy as np
import pytest

import libheom_gb300 as lh
import oracle
from libheom_gb300 import configs
from libheom_gb300 import terminator as T
from oracle import mlp_oracle

pytestmark = pytest.mark.gpu


def _dev(a):
    torch = pytest.importorskip("torch")
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()


@pytest.mark.parametrize("din,h,dout,B", [(19, 256, 8, 300), (210, 256, 98, 70), (5, 48, 3, 1)])
def test_forward_and_gradients_match_numpy(din, h, dout, B):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(din)
    mlp = T.MLP(din, h, dout, seed=din)
    x = rng.standard_normal((B, din)).astype(np.float32)
    t = rng.standard_normal((B, dout)).astype(np.float32)
    xd, td = _dev(x), _dev(t)
    y = torch.empty((B, dout), dtype=torch.float32, device="cuda")
    mlp.forward(xd.data_ptr(), y.data_ptr(), B)
    params = mlp.get_params()
    yref, _ = mlp_oracle.forward(params, x.astype(np.float64), din, h, dout)
    assert np.abs(y.cpu().numpy() - yref).max() <= 1e-4 * (1 + np.abs(yref).max())
    g, loss = mlp.gradients(xd.data_ptr(), td.data_ptr(), B)
    gref, lref = mlp_oracle.gradients(params, x.astype(np.float64), t.astype(np.float64), din, h, dout)
    assert abs(loss - lref) <= 1e-4 * abs(lref)
    assert np.abs(g - gref).max() <= 1e-3 * np.abs(gref).max()


def test_adam_training_reduces_loss():
    rng = np.random.default_rng(5)
    W = rng.standard_normal((8, 19)) * 0.3
    x = rng.standard_normal((8192, 19)).astype(np.float32)
    t = (x @ W.T).astype(np.float32)
    mlp = T.MLP(19, 256, 8, seed=1)
    losses = T.train(mlp, x, t, epochs=15, batch=1024, lr=2e-3)
    assert losses[-1] < 0.05 * losses[0]


def test_terminator_feeds_rhs_like_numpy():
    p = configs.spin_boson(eps=0.3, lam=0.4, beta=1.5, depth=3)
    din, dout = T.dims(p)
    mlp = T.MLP(din, 256, dout, seed=7)
    q = lh.from_params(p)
    rng = np.random.default_rng(2)
    rho = (rng.standard_normal((p.n_hrchy(), 2, 2)) + 1j * rng.standard_normal((p.n_hrchy(), 2, 2))) * 0.3
    plain = q.calc_diff(rho)
    T.attach(q, mlp)
    got = q.calc_diff(rho)
    # numpy: plain RHS plus the +1 terms of the predicted tier-(N+1) ADOs
    n_tab, p1, _ = oracle.Oracle("port").hrchy(p.n_modes, p.max_depth)
    nh = p.n_hrchy()
    first = int(np.argmax(n_tab.sum(1) == p.max_depth))
    X, s = mlp_oracle.term_features(p, n_tab, rho, first)
    Y, _ = mlp_oracle.forward(mlp.get_params(), X, din, 256, dout)
    v = np.diag(p.V[0])
    cphi = 1j * (v[:, None] - v[None, :])
    expect = plain.copy()
    K = p.n_modes
    for j, l in enumerate(range(first, nh)):
        for k in range(K):
            y = Y[j * K + k]
            pred = s[j] * (y[:4] + 1j * y[4:]).reshape(2, 2)
            expect[l] -= cphi * p.sigma[0][k] * pred
    scale = np.abs(plain).max()
    assert np.abs(got - expect).max() <= 1e-5 * scale
    assert np.abs(got - plain).max() > 1e-8 * scale  # the terminator does contribute
