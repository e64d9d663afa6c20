"""The C-ABI library builds for sm_103a, loads, and exports every symbol
include/t9gb.h declares (no compute calls: this runs without a GPU)."""
import ctypes
import importlib
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "t9gb.h")).read()
    return sorted(set(re.findall(r"\b(t9gb_\w+)\s*\(", src)))


def test_header_lists_all_exports():
    abi = importlib.import_module("tinker-gpu_gb300.abi")
    assert sorted(abi.EXPORTS) == declared_symbols()


def test_library_exports_declared_symbols():
    b = importlib.import_module("tinker-gpu_gb300.build")
    lib_path, _ = b.build()
    lib = ctypes.CDLL(lib_path)
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_status_strings_without_device():
    b = importlib.import_module("tinker-gpu_gb300.build")
    lib = ctypes.CDLL(b.build()[0])
    lib.t9gb_status_string.restype = ctypes.c_char_p
    assert lib.t9gb_status_string(1) == b"induced dipoles are not converged"
