"""The C ABI library loads and exports every symbol include/scisim_gpu.h declares.

No compute call is made here (no GPU needed); the library is built in-tree if it
has not been built yet.
"""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "scisim_gpu.h")


def declared_symbols():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"SG_API\s+[\w\s\*]*?\b(sg_\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def built_lib():
    from scisim_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "sg_step" in syms and "sg_sobogus_solve_2d" in syms and "sg_broadphase_2d" in syms
    assert len(syms) >= 14


def test_library_exports_every_declared_symbol(built_lib):
    missing = [s for s in declared_symbols() if not hasattr(built_lib, s)]
    assert not missing, missing


def test_python_binding_covers_header():
    from scisim_gb300 import _lib
    assert sorted(_lib.SIGNATURES) == declared_symbols()


def test_library_is_sm103a_only():
    from scisim_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
    assert "-fmad=false" in build.NVCC_FLAGS


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    from scisim_gb300 import _lib
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "absent.so"))
    monkeypatch.setattr(_lib, "_lib", None)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _lib.lib()
