"""The C-ABI library: loads and exports every symbol include/fhg.h declares. CPU only (no
compute call is made here)."""
import ctypes
import os
import re

import pytest

import importlib

B = importlib.import_module("fhhos4_gb300.build")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    syms = set()
    for name in os.listdir(os.path.join(ROOT, "include")):
        if name.endswith(".h"):
            text = open(os.path.join(ROOT, "include", name)).read()
            syms |= set(re.findall(r"^\s*(?:[A-Za-z_][\w\s\*]*?\s\**)(fhg_\w+)\s*\(", text, re.M))
    return sorted(syms)


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(B.LIB):
        B.build()
    return ctypes.CDLL(B.LIB)


def test_header_declares_the_solver_entry_points():
    syms = header_symbols()
    for s in ("fhg_create", "fhg_set_level", "fhg_set_prolongation", "fhg_setup", "fhg_solve", "fhg_destroy",
              "fhg_last_error"):
        assert s in syms


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in header_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_lists_every_declared_symbol():
    from fhhos4_gb300 import _native as N
    assert sorted(N.EXPORTS) == header_symbols()


def test_build_targets_sm_103a_only():
    assert B.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
