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


def _declarations():
    """name -> parameter list of every bcg_ function declared in the headers."""
    out = {}
    for f in os.listdir(os.path.join(ROOT, "include")):
        if not f.endswith(".h"):
            continue
        txt = re.sub(r"/\*.*?\*/", " ", open(os.path.join(ROOT, "include", f)).read(), flags=re.S)
        for m in re.finditer(r"\b(?:int|const char\*|void)\s+\*?\s*(bcg_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", txt):
            params = [p.strip() for p in m.group(2).split(",") if p.strip() and p.strip() != "void"]
            out[m.group(1)] = params
    return out


def test_binding_signatures_match_header_arity_and_kinds():
    """Each ctypes signature has one code per declared parameter, and the code
    agrees with the C type: strings 's', other pointers 'p', int 'i', long long
    'L', double 'd', float 'f'."""
    from broadcast_gb300 import _lib
    decl = _declarations()
    assert len(decl) > 30
    bad = []
    for name, params in decl.items():
        sig = _lib.SIGNATURES[name]
        if len(sig) != len(params):
            bad.append((name, len(params), len(sig)))
            continue
        for code, p in zip(sig, params):
            if "char*" in p.replace(" ", ""):
                kind = "s"
            elif "*" in p:
                kind = "p"
            else:
                kind = "L" if "long long" in p else ("d" if p.startswith("double") else
                                                     ("f" if p.startswith("float") else "i"))
            if code != kind:
                bad.append((name, p, code))
    assert not bad, bad
