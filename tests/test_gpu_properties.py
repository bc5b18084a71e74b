"""Size-independent properties of the CUDA path at full workload sizes."""
import numpy as np
import pytest

import libheom_gb300 as lh
from libheom_gb300 import configs

pytestmark = pytest.mark.gpu


def test_trace_and_hermiticity_exciton7_dp():
    p = configs.exciton_7site()
    qs = lh.qme_solver(lh.from_params(p), lh.rkdp())
    rho = p.rho0_ground()
    qs.solve(rho, [0.0, 100.0], None, dict(dt=0.1, atol=1e-8, rtol=1e-8))
    r0 = rho[0]
    assert abs(np.trace(r0) - 1.0) < 1e-10
    assert np.abs(r0 - r0.conj().T).max() < 1e-10
    assert np.all(np.linalg.eigvalsh((r0 + r0.conj().T) / 2) > -1e-6)


def test_zero_coupling_is_unitary():
    p = configs.spin_boson(lam=0.0, depth=4)
    qs = lh.qme_solver(lh.from_params(p), lh.rk4())
    rho = p.rho0_ground()
    out = []
    t = np.linspace(0, 2.0, 5)
    qs.solve(rho, t, lambda tt: out.append(rho[0, 0, 0].real), {"dt": 0.005})
    assert np.allclose(out, np.cos(t) ** 2, atol=1e-9)
    assert np.abs(rho[1:]).max() == 0.0


def test_mixed_precision_error_budget_exciton7():
    """FP32 bulk / FP64 state stays within 1e-6 of the FP64 path."""
    p = configs.exciton_7site()
    kw = dict(dt=0.1, atol=1e-8, rtol=1e-8)
    out = {}
    for prec in ("fp64", "mixed"):
        qs = lh.qme_solver(lh.from_params(p, precision=prec), lh.rkdp())
        rho = p.rho0_ground()
        qs.solve(rho, [0.0, 200.0], None, kw)
        out[prec] = rho
    assert np.abs(out["mixed"] - out["fp64"]).max() <= 1e-6


def test_device_solve_matches_host_solve():
    import ctypes
    p = configs.spin_boson(depth=6)
    q = lh.from_params(p)
    qs = lh.qme_solver(q, lh.lsrk4())
    rho_h = p.rho0_ground()
    qs.solve(rho_h, [0.0, 1.0], None, {"dt": 0.01})
    import torch
    rho_d = torch.from_numpy(p.rho0_ground()).cuda()
    torch.cuda.synchronize()
    qs.solve_device(rho_d.data_ptr(), [0.0, 1.0], None, {"dt": 0.01})
    torch.cuda.synchronize()
    assert np.array_equal(rho_d.cpu().numpy(), rho_h)
