"""The C-ABI library loads and exports every symbol include/fesom_tracer_gb300.h
declares (no GPU needed: no compute call is made)."""
import ctypes
import os
import re

from fesom2_tracer_dwarf_gb300 import _lib

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "fesom_tracer_gb300.h")


def _declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^[A-Za-z_][\w\s\*]*?\b((?:tracer|fgb)_\w+)\s*\(", src, flags=re.M)))


def test_header_lists_reference_interface():
    decl = _declared()
    for name in _lib.REFERENCE_SYMBOLS + _lib.EXTENSION_SYMBOLS + _lib.ENGINE_SYMBOLS:
        assert name in decl, name
    assert len(_lib.REFERENCE_SYMBOLS) == 23


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    missing = [n for n in _declared() if not hasattr(L, n)]
    assert not missing, missing


def test_library_is_in_tree():
    L = _lib.load()
    assert os.path.dirname(L._name).startswith(os.path.dirname(os.path.dirname(HEADER)))
    assert ctypes.c_int(L.fgb_version()).value >= 1
