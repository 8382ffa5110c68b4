"""The C-ABI library builds, loads and exports every entry point of include/wbem.h."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols(header=None):
    names = [header] if header else sorted(f for f in os.listdir(os.path.join(ROOT, "include"))
                                           if f.endswith(".h"))
    out = set()
    for n in names:
        txt = open(os.path.join(ROOT, "include", n)).read()
        out |= set(re.findall(r"\b(wbem_[a-z0-9_]+)\s*\(", txt))
    return sorted(out)


def test_header_lists_match_wrapper():
    from wavebem_gb300.bem_problem import EXPORTS
    assert sorted(EXPORTS) == declared_symbols("wbem.h")


def test_library_exports_every_declared_symbol():
    from wavebem_gb300 import build
    lib = build.LIB
    if not os.path.exists(lib):
        build.build()
    import ctypes
    L = ctypes.CDLL(lib)
    for s in declared_symbols():
        assert hasattr(L, s), s


def test_default_options_match_reference_prm():
    from wavebem_gb300.bem_problem import default_options
    o = default_options()
    assert o.quadrature_order == 4 and o.singular_quadrature_order == 5
    assert o.gmres_restart == 100
