"""The C-ABI library: loads and exports every symbol include/fhg.h declares. CPU only (no
compute call is made here)."""
import ctypes
import os
import re
import shutil
import subprocess

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


def _c_layout(header: str, include_dir: str, struct: str, fields):
    """sizeof and offsetof of a C struct as gcc lays it out (compiled into the git-ignored _build)."""
    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("gcc not available")
    out_dir = os.path.join(ROOT, "fhhos4_gb300", "_build")
    os.makedirs(out_dir, exist_ok=True)
    src = os.path.join(out_dir, f"layout_{struct}.c")
    exe = os.path.join(out_dir, f"layout_{struct}")
    body = "".join(f'printf(" %zu", offsetof({struct}, {f}));' for f in fields)
    with open(src, "w") as f:
        f.write(f'#include <stddef.h>\n#include <stdio.h>\n#include "{header}"\n'
                f'int main(void) {{ printf("%zu", sizeof({struct})); {body} return 0; }}\n')
    subprocess.run([gcc, "-std=c11", "-I", include_dir, src, "-o", exe], check=True)
    vals = [int(v) for v in subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()]
    return vals[0], vals[1:]


def _ctypes_layout(cls):
    return ctypes.sizeof(cls), [getattr(cls, name).offset for name, _ in cls._fields_]


def test_python_structs_match_the_c_header():
    """fhg_options and fhg_solve_info as ctypes mirror them: same size, every field at its offset."""
    from fhhos4_gb300 import _native as N
    for cls, struct in ((N.Options, "fhg_options"), (N.SolveInfo, "fhg_solve_info")):
        fields = [name for name, _ in cls._fields_]
        assert _c_layout("fhg.h", os.path.join(ROOT, "include"), struct, fields) == _ctypes_layout(cls), struct


def test_oracle_options_match_its_header():
    import sys
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    fields = [name for name, _ in O._Opts._fields_]
    assert _c_layout("fcgmg_oracle.h", os.path.join(ROOT, "oracle"), "orc_options", fields) == _ctypes_layout(O._Opts)


def test_default_options():
    """fhg_default_options (host only): the reference's defaults, one smoothing count for every
    level (-1 for the coarse counts) and the autotuner's GS layout."""
    from fhhos4_gb300 import _native as N
    o = N.default_options()
    assert (o.pre_iterations, o.post_iterations, o.w_loops, o.galerkin) == (1, 1, 1, 0)
    assert (o.coarse_pre_iterations, o.coarse_post_iterations) == (-1, -1)
    assert o.gs_layout == N.GS_LAYOUT["auto"] == 0
    assert o.tolerance == 1e-8 and o.max_iterations == 200
