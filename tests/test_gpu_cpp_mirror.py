"""The C++ mirror header drives the engine like a libheom C++ caller."""
import os
import subprocess

import numpy as np
import pytest

import libheom_gb300 as lh
import oracle
from libheom_gb300 import configs

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_mirror_spin_boson(tmp_path):
    lib = lh.library_path()
    lh.load()
    exe = tmp_path / "mirror"
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "spin_boson_mirror.cpp"), "-L", os.path.dirname(lib),
                    "-lheomgb", f"-Wl,-rpath,{os.path.dirname(lib)}", "-o", str(exe)], check=True)
    out = tmp_path / "rho.bin"
    r = subprocess.run([str(exe), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    p = configs.spin_boson(depth=6)
    got = np.fromfile(out, dtype=np.complex128).reshape(p.n_hrchy(), 2, 2)
    ref = oracle.Oracle("port").solve(p, p.rho0_ground(), [0.0, 0.5], solver="rk4", dt=0.005)[-1]
    assert np.abs(got - ref).max() < 1e-12
