"""The C-ABI library builds for sm_103a, loads, and exports every entry
point declared in include/parphom_gpu.h (no compute calls: no GPU needed)."""
import ctypes
import os
import re

from parphom_gb300 import api, build

HDR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "parphom_gpu.h")


def declared_symbols():
    txt = open(HDR).read()
    return sorted(set(re.findall(r"PP_API\s+[\w\s\*]*?\b(pp_\w+)\s*\(", txt)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "pp_ctx_create" in syms and "pp_solve_batch" in syms
    assert set(api.EXPORTED) <= set(syms)


def test_library_exports_all_declared():
    path = build.build()
    lib = ctypes.CDLL(path)
    for s in declared_symbols():
        assert hasattr(lib, s), s


def test_strerror_and_version():
    L = api.load()
    assert L.pp_version() >= 100
    assert b"memory" in L.pp_strerror(1002)
    assert L.pp_strerror(-3).startswith(b"illegal")
