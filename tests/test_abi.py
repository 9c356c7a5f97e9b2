"""CPU-side checks of the C-ABI library: it loads and exports every symbol
declared in include/broadcast_gb300.h (no GPU compute is called here)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = []
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", f)).read()
            names += re.findall(r"\b(bcg_[a-z0-9_]+)\s*\(", txt)
    return sorted(set(names))


def test_library_builds_and_exports_every_declared_symbol():
    from broadcast_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    names = _declared()
    assert len(names) > 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_table_covers_header():
    from broadcast_gb300 import _lib
    assert set(_declared()) <= set(_lib.SIGNATURES), set(_declared()) - set(_lib.SIGNATURES)
