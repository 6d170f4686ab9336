"""The float-float pairs (scisim_gb300/csrc/ffloat.hpp) that carry the FP64-precision disc sweeps
on the FP32 pipe (k_gs_ff1, k_gs_patch_ff): a host test compiled with g++ from the same header
the kernels include checks that a split keeps 48 bits, that hi + lo is exact in FP64, and that
sums, products and a 20,000-step accumulation stay within 2^-44 of their operands' magnitudes
against long double arithmetic."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_float_float_accuracy(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "ffloat_test")
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "scisim_gb300", "csrc"),
           os.path.join(ROOT, "tests", "cpp", "ffloat_test.cpp"), "-o", exe]
    p = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-3000:]
    p = subprocess.run([exe, "1000000"], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stdout + p.stderr
    assert p.stdout.strip().endswith("0 checks failed")
