"""The mixed form's integer-assembled FP32 <-> FP64 conversions
(libheom_gb300/csrc/fpconv.cuh) give the IEEE conversions' bits: the header
compiled for the host with g++ and checked against the compiler's own
conversions (tests/fpconv_check.cpp)."""
import pathlib
import shutil
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parent


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_fpconv_matches_ieee_conversions(tmp_path):
    exe = tmp_path / "fpconv_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-o", str(exe), str(ROOT / "fpconv_check.cpp")], check=True)
    # every 31st float bit pattern (all exponents, ties included); the full
    # sweep (argument 1, every float) passes too and takes a few minutes
    out = subprocess.run([str(exe), "31"], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout
