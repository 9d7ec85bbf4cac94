"""The C-ABI library builds for sm_103a, loads, and exports every symbol the
public header declares (no GPU needed: no compute call is made)."""
import ctypes
import os
import re

from conftest import REPO

HEADER_DIR = os.path.join(REPO, "include")


def declared_symbols():
    names = set()
    for f in os.listdir(HEADER_DIR):
        if f.endswith(".h"):
            src = open(os.path.join(HEADER_DIR, f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(otg_\w+)\s*\(", src))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "otg_sinkhorn_dense" in names and "otg_dense_plan" in names


def test_library_exports_declared_symbols():
    from pot_gb300 import _build, _lib
    path = _build.build()
    lib = ctypes.CDLL(path)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing
    # every declared symbol also has a ctypes signature in the binding
    assert set(declared_symbols()) <= set(_lib.SIGNATURES), set(declared_symbols()) - set(_lib.SIGNATURES)
