"""The native library loads without a GPU and exports every entry point
include/tmrg.h declares (no compute calls here)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "tmrg.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tmrg_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from tmr_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    names = declared_functions()
    assert "tmrg_forest_create" in names and "tmrg_interp_mult" in names
    assert len(names) >= 40


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from tmr_gb300 import _lib
    missing = [n for n in declared_functions() if n not in _lib._SIGS]
    assert not missing, missing


def test_cpu_only_calls(lib):
    lib.tmrg_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.tmrg_version()
    lib.tmrg_last_error.restype = ctypes.c_char_p
    assert lib.tmrg_last_error() == b""
    # argument validation happens before any device work
    assert lib.tmrg_forest_create(2, 7, None, None) == 1
    lib.tmrg_last_error.restype = ctypes.c_char_p
    assert lib.tmrg_last_error() != b""
