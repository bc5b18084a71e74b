"""Test infrastructure: numpy restatement of the learned terminator.

THE ORACLE, NOT THE PRODUCT: tests use it to check the CUDA forward,
backward and inference kernels of the terminator (libheom_gb300/csrc/mlp.cu).

* MLP: x -> Linear(h) -> GELU -> Linear(h) -> GELU -> Linear(d_out).  Every
  product is a BF16 GEMM on the device (both operands rounded to BF16, round to
  nearest even, FP32 accumulation): here the weight matrices and each GEMM's
  other operand (the layer input, or the back-propagated gradient) are
  rounded to BF16 the same way, biases and bias gradients stay unrounded, and
  the arithmetic is float64.
* Terminator features of a tier-N ADO rho_n and mode k:
  [Re rho/s, Im rho/s, onehot(k), Re A/s, Im A/s], s = max |rho_n|,
  A = (n_k+1) (-i s_k (v_a - v_b) + a_k (v_a + v_b)) rho_ab / (ngamma_n + gamma_kk).
* Gain head and closure loss: outputs (y | z) of a row give
  C = y - i sign(v_a - v_b) softplus(z) and the prediction C rho_n / sigma_k;
  the loss is each row's squared error relative to its own size.
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf


def bf16(x):
    """Round float32 values to bfloat16 (nearest even) and back to float32."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    rounding = ((u >> 16) & 1) + 0x7FFF
    u = ((u + rounding) >> 16) << 16
    return u.astype(np.uint32).view(np.float32)


def q(x):
    """A GEMM operand as the device stages it: float32, then BF16 (float64 out)."""
    return bf16(np.asarray(x, dtype=np.float64).astype(np.float32)).astype(np.float64)


def unpack(params, din, h, dout):
    sizes = [h * din, h, h * h, h, dout * h, dout]
    out, o = [], 0
    for s in sizes:
        out.append(np.asarray(params[o:o + s], dtype=np.float64))
        o += s
    W1, b1, W2, b2, W3, b3 = out
    return (bf16(W1.astype(np.float32)).astype(np.float64).reshape(h, din), b1,
            bf16(W2.astype(np.float32)).astype(np.float64).reshape(h, h), b2,
            bf16(W3.astype(np.float32)).astype(np.float64).reshape(dout, h), b3)


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)


def forward(params, x, din, h, dout):
    W1, b1, W2, b2, W3, b3 = unpack(params, din, h, dout)
    z1 = q(x) @ W1.T + b1
    a1 = gelu(z1)
    z2 = q(a1) @ W2.T + b2
    a2 = gelu(z2)
    return q(a2) @ W3.T + b3, (z1, a1, z2, a2)


def softplus(z):
    return np.maximum(z, 0.0) + np.log1p(np.exp(-np.abs(z)))


def gain_head(y, sg):
    """C_e = y_e - i sg_e softplus(z_e) from the outputs (y | z) of a row."""
    n2 = sg.shape[-1]
    return y[..., :n2] - 1j * sg * softplus(y[..., n2:])


def gain_loss(y, t):
    """Closure loss of rows y (B, 2 n2) against t (B, 5 n2) and its gradient d/dy."""
    n2 = y.shape[1] // 2
    tt = t[:, :n2] + 1j * t[:, n2:2 * n2]
    r = t[:, 2 * n2:3 * n2] + 1j * t[:, 3 * n2:4 * n2]
    sg = t[:, 4 * n2:]
    m = np.abs(sg)
    C = gain_head(y, sg)
    d = C * r - tt
    den = (m * (np.abs(tt) ** 2 + 1e-2 * np.abs(r) ** 2)).sum(1) + 1e-6
    B = y.shape[0]
    loss = float(np.mean((m * np.abs(d) ** 2).sum(1) / den))
    w = (2.0 / (B * den))[:, None]
    cr = np.conj(d) * r
    z = y[:, n2:]
    dy = np.concatenate([w * m * cr.real, w * m * sg * (1.0 / (1.0 + np.exp(-z))) * cr.imag], axis=1)
    return loss, dy


def gradients(params, x, t, din, h, dout, loss_kind=0):
    """Gradient of the loss (0: mean((y - t)^2); 1: gain_loss) with respect to
    the packed parameters."""
    W1, b1, W2, b2, W3, b3 = unpack(params, din, h, dout)
    y, (z1, a1, z2, a2) = forward(params, x, din, h, dout)
    if loss_kind == 1:
        loss, dy = gain_loss(y, t)
    else:
        dy = 2.0 * (y - t) / y.size
        loss = float(np.mean((y - t) ** 2))
    gW3 = q(dy).T @ q(a2)
    gb3 = dy.sum(0)
    d2 = (q(dy) @ W3) * gelu_grad(z2)
    gW2 = q(d2).T @ q(a1)
    gb2 = d2.sum(0)
    d1 = (q(d2) @ W2) * gelu_grad(z1)
    gW1 = q(d1).T @ q(x)
    gb1 = d1.sum(0)
    return np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3]), loss


def term_features(p, n_tab, rho, first):
    """Feature rows and scales of the tier-N ADOs l >= first (rows l-major, then k)."""
    n = p.n_level
    K = p.n_modes
    bath_of, s_k, a_k, g_k = [], [], [], []
    for u in range(p.n_noise):
        sv = p.S[u] @ p.phi_0[u]
        av = p.A[u] @ p.phi_0[u]
        for k in range(len(p.sigma[u])):
            bath_of.append(u)
            s_k.append(sv[k])
            a_k.append(av[k])
            g_k.append(p.gamma[u][k, k])
    nh = rho.shape[0]
    rows, scales = [], []
    for l in range(first, nh):
        r = rho[l]
        s = np.sqrt(np.max(np.abs(r.astype(np.complex64)) ** 2)) + 1e-30
        ngd = np.sum(n_tab[l] * np.array(g_k))
        scales.append(s)
        for k in range(K):
            v = np.diag(p.V[bath_of[k]])
            va, vb = v[:, None], v[None, :]
            c = -1j * s_k[k] * (va - vb) + a_k[k] * (va + vb)
            A = (n_tab[l, k] + 1) * c * r / (ngd + g_k[k])
            onehot = np.zeros(K)
            onehot[k] = 1
            rows.append(np.concatenate([r.real.ravel() / s, r.imag.ravel() / s, onehot, A.real.ravel() / s,
                                        A.imag.ravel() / s]))
    return np.array(rows), np.array(scales)
