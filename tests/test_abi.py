"""The C-ABI library loads on any machine and exports every function that
include/mandoct_gb300.h declares (no compute calls: no GPU needed)."""
import ctypes
import os
import re

from conftest import ROOT
from reconstruction_program_taichi_gb300 import _lib


def _declared():
    src = open(os.path.join(ROOT, "include", "mandoct_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mct_\w+)\s*\(", src)))


def test_header_declares_the_bound_symbols():
    declared = _declared()
    assert set(_lib.SIGNATURES) == set(declared), set(declared) ^ set(_lib.SIGNATURES)


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    for name in _declared():
        assert hasattr(lib, name), name
    assert lib.mct_version().startswith(b"mandoct-gb300")
    assert lib.mct_reduce_scratch_size() > 0


def test_invalid_geometry_is_rejected_without_a_gpu():
    lib = _lib.load()
    g = _lib.Geom()  # all zeros: invalid
    rc = lib.mct_filter(ctypes.byref(g), None, None, None, None)
    assert rc == -1
    assert b"bad detector size" in lib.mct_last_error_string()
