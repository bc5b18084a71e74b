"""The allocation-free hierarchy build (heomgb_hrchy_build_noalloc).

Callers that cannot call cudaMalloc -- code running inside a framework that
owns the device heap, or a plugin whose allocations are audited -- hand in
device buffers they already own; the entry point keeps its own scratch in a
fixed device array.  Its tables must equal those of the regular path
(heomgb_qme_set_param + heomgb_qme_get_hrchy) exactly, on repeated calls that
reuse the shared scratch.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

import libheom_gb300 as lh
from libheom_gb300 import _lib
from libheom_gb300.noise import drude_lorentz_terms, noise_members
from libheom_gb300.params import HeomParams

pytestmark = pytest.mark.gpu


def regular_tables(K, N, U):
    nu, c = drude_lorentz_terms(0.5, 1.0, 1.0, K - 1)
    per = np.array_split(np.arange(K), U)
    gam, phi, sig, S, A = [], [], [], [], []
    for idx in per:
        g, p, s, Sm, Am, _ = noise_members(nu[idx], c[idx])
        gam.append(g); phi.append(p); sig.append(s); S.append(Sm); A.append(Am)
    p = HeomParams(H=np.array([[0, 1], [1, 0]], complex), V=[np.diag([1.0, -1.0]).astype(complex)] * U,
                   gamma=gam, phi_0=phi, sigma=sig, S=S, A=A, s_delta=[0j] * U, max_depth=N)
    return lh.from_params(p).hrchy()


def noalloc_tables(K, N, torch):
    from math import comb
    count = comb(K + N, N)
    n = torch.full((count * K,), -7, dtype=torch.int32, device="cuda")
    p1 = torch.full(((count + 1) * K,), -7, dtype=torch.int32, device="cuda")
    m1 = torch.full(((count + 1) * K,), -7, dtype=torch.int32, device="cuda")
    got = ctypes.c_int(0)
    torch.cuda.synchronize()
    _lib.check(_lib.load().heomgb_hrchy_build_noalloc(K, N, n.data_ptr(), p1.data_ptr(), m1.data_ptr(),
                                                       ctypes.byref(got), None))
    torch.cuda.synchronize()
    assert got.value == count
    return (n.cpu().numpy().reshape(count, K), p1.cpu().numpy().reshape(count + 1, K),
            m1.cpu().numpy().reshape(count + 1, K))


@pytest.mark.parametrize("K,N,U", [(3, 10, 1), (14, 4, 7), (48, 3, 24), (5, 3, 2)])
def test_noalloc_matches_regular_path_twice(K, N, U):
    torch = pytest.importorskip("torch")
    ref = regular_tables(K, N, U)
    for _ in range(2):  # the second call reuses the shared scratch left by the first
        got = noalloc_tables(K, N, torch)
        for a, b in zip(got, ref):
            assert np.array_equal(a, b)


def test_noalloc_rejects_sizes_beyond_scratch():
    lib = _lib.load()
    got = ctypes.c_int(0)
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    st = lib.heomgb_hrchy_build_noalloc(80, 20, dummy, dummy, dummy, ctypes.byref(got), None)
    assert st == 7  # HEOMGB_ERR_CAPACITY
    assert b"exceeds the fixed scratch maximum" in lib.heomgb_last_error()
