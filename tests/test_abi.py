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
    # the C ABI stands alone: the shared object links the CUDA runtime only
    from combblas_gb300 import _lib

    data = open(_lib.LIB_PATH, "rb").read()
    assert b"libtorch" not in data and b"libc10" not in data
