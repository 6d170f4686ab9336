"""The allocation-free solve's per-context scratch-address cache (scisim_gb300/csrc/na_cache.hpp),
compiled with g++ into a test program and run on the CPU (tests/cpp/na_cache_test.cpp): the address
is looked up again after the context changes (as after cudaDeviceReset), served from the cache while
it does not, kept per device, never cached without a context identity, and consistent across
threads."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_noalloc_address_cache(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "na_cache_test")
    src = os.path.join(ROOT, "tests", "cpp", "na_cache_test.cpp")
    p = subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-pthread", src, "-o", exe],
                       capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
