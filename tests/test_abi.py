"""The C-ABI library builds, loads and exports every entry point the header
declares; argument errors come back as status codes (no GPU needed)."""
import ctypes
import os
import re

import pytest

import libheom_gb300 as lh
from libheom_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "heomgb.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(heomgb_[a-z0-9_]+)\s*\(", text)
    return sorted(set(n for n in names if n != "heomgb_callback"))


def test_every_declared_symbol_is_exported():
    lib = _lib.load()
    names = declared_functions()
    assert len(names) >= 25
    for name in names:
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, f"{name} has no ctypes signature"


def test_library_is_in_tree():
    assert os.path.dirname(lh.library_path()).startswith(os.path.join(ROOT, "libheom_gb300"))
    assert os.path.exists(lh.library_path())


def test_version_and_errors_without_gpu():
    lib = _lib.load()
    assert lib.heomgb_abi_version() == 1
    assert lib.heomgb_version().decode()
    h = ctypes.c_void_p()
    assert lib.heomgb_solver_create(7, ctypes.byref(h)) == 1          # unknown solver
    assert b"unknown solver" in lib.heomgb_last_error()
    assert lib.heomgb_qme_create(9, 3, 1, 1, ctypes.byref(h)) == 1    # unknown form
    assert lib.heomgb_qme_create(0, -1, 1, 1, ctypes.byref(h)) == 1   # negative depth
    assert lib.heomgb_qme_set_param(None) == 1
    assert lib.heomgb_qme_destroy(None) == 0
    assert lib.heomgb_errnrm1_scratch(10**6) > 2


@pytest.mark.parametrize("n_dim,max_depth", [(80, 20), (2**31 - 1, 0), (0x7ffffff0, 0x7ffffff0), (1, 2**31 - 1)])
def test_noalloc_capacity_check_without_gpu(n_dim, max_depth):
    # the size check runs before any CUDA call, so no kernel is launched here;
    # sums that would wrap a 32-bit int must still be rejected
    lib = _lib.load()
    got = ctypes.c_int(0)
    dummy = ctypes.c_void_p(16)  # never dereferenced
    st = lib.heomgb_hrchy_build_noalloc(n_dim, max_depth, dummy, dummy, dummy, ctypes.byref(got), None)
    assert st == 7  # HEOMGB_ERR_CAPACITY
    assert b"exceeds the fixed scratch maximum" in lib.heomgb_last_error()
    assert got.value == 0


def test_python_mirror_validation():
    q = lh.heom_hilb(3)
    q.alloc_noises(2)
    assert len(q.V) == 2 and q.len_gamma == [0, 0]
    with pytest.raises(ValueError):
        lh.heom_hilb(-1)
    with pytest.raises(RuntimeError):
        q.get_n_hrchy()          # before set_param
    with pytest.raises(ValueError):
        q.set_param()            # H not set
    from libheom_gb300.heom import _kwargs
    with pytest.raises(TypeError):
        _kwargs({"dt": "0.1"})
    k = _kwargs({"dt": 0.5})
    assert k.has_dt == 1 and k.has_atol == 0
