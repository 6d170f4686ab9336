"""The pair scans answer the disc-disc CCD test with ccd_hits (scisim_gb300/csrc/ccd2d.hpp), which
skips the square root and the divisions of the reference's ballBallCCDCollisionHappens
(CollisionDetectionUtilities.cpp:3-126) where signs decide.  Host test: compiled with g++ from the
same header the kernels include, the two answers agree on several million inputs (pile-like disc
pairs, quadratics with roots at a hair's breadth from 0 and 1, random bit patterns, special
values)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_ccd_hits_matches_ccd_happens(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "ccd_hits_test")
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "scisim_gb300", "csrc"),
           os.path.join(ROOT, "tests", "cpp", "ccd_hits_test.cpp"), "-o", exe]
    p = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-3000:]
    p = subprocess.run([exe, "2000000"], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stdout + p.stderr
    assert " 0 mismatches" in p.stdout
