"""The C-ABI library builds, loads and exports every function include/petrbf_gb300.h
declares (CPU only: no compute calls)."""
import ctypes
import os
import re

from conftest import ROOT


def _declared():
    names = []
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            names += re.findall(r"^\s*(?:[\w*]+\s+)+\**(prbf_\w+)\s*\(", src, re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    from petrbf_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    names = _declared()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    from petrbf_gb300 import _native
    assert set(_declared()) <= set(_native.SIGNATURES)


def test_status_strings_and_defaults():
    from petrbf_gb300 import _native as N
    L = N.lib()
    p = N.Params()
    L.prbf_params_default(ctypes.byref(p))
    assert p.dim == 2 and p.restart == 30 and p.rtol == 1e-13 and p.max_it == 1000
    assert L.prbf_status_string(0) == b"ok"
    assert L.prbf_status_string(N.ERR_STATE) == b"call out of order"
