"""The C-ABI library loads and exports every entry point include/gbcomb.h
declares (no GPU calls)."""
import ctypes
import os
import re

from conftest import ROOT


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "gbcomb.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|int64_t|const char \*)\s*(gbc_[a-z0-9_]+)\s*\(", src, re.M)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "gbc_spgemm" in syms and "gbc_context_create" in syms


def test_library_exports_every_declared_symbol():
    from combblas_gb300 import _lib

    lib = _lib.lib()
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_covers_header():
    from combblas_gb300 import _lib

    assert set(declared_symbols()) <= set(_lib.exported_symbols())


def test_library_has_no_torch_dependency():
    # the C ABI stands alone: loaded into a fresh interpreter that never
    # imports torch, it maps no torch library (its dependencies are the CUDA
    # runtime and the C++ runtime)
    import subprocess
    import sys

    from combblas_gb300 import _lib

    code = ("import ctypes, sys; ctypes.CDLL(sys.argv[1]); "
            "print(open('/proc/self/maps').read())")
    r = subprocess.run([sys.executable, "-c", code, _lib.LIB_PATH], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert "libgbcomb.so" in r.stdout
    assert "libtorch" not in r.stdout and "libc10" not in r.stdout


def test_product_code_does_not_use_the_oracle():
    # the package (host side and CUDA sources) never imports, links or loads
    # the oracle: only tests, smoke() and bench.py's CPU arms do
    pkg = os.path.join(ROOT, "combblas_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if not f.endswith((".py", ".cu", ".cuh", ".h", ".hpp")):
                continue
            src = open(os.path.join(dirpath, f)).read()
            assert not re.search(r"^\s*(import|from)\s+oracle\b", src, re.M), f
            assert "libgbc_oracle" not in src and "libcombblas_ref" not in src, f
    for f in ("gbcomb.h", os.path.join("gbcomb", "combblas_shim.hpp")):
        src = open(os.path.join(ROOT, "include", f)).read()
        assert "oracle" not in src, f


def test_missing_library_fails_loudly(monkeypatch):
    # no CPU fallback: without the CUDA library every entry point raises
    import pytest

    from combblas_gb300 import _lib

    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib, "LIB_PATH", os.path.join(ROOT, "combblas_gb300", "no-such-libgbcomb.so"))
    with pytest.raises(ImportError):
        _lib.lib()
