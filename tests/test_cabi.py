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


def test_struct_mirrors_match_compiled_layout():
    """Every ctypes mirror in the binding has the size and field offsets of
    the compiled C struct (otg_abi_layout), so no field is read shifted."""
    from pot_gb300 import _build, _lib
    lib = ctypes.CDLL(_build.build())
    fn = lib.otg_abi_layout
    fn.restype, fn.argtypes = _lib.SIGNATURES["otg_abi_layout"][0], _lib.SIGNATURES["otg_abi_layout"][1]
    src = re.sub(r"/\*.*?\*/", "", open(os.path.join(HEADER_DIR, "pot_gb300.h")).read(), flags=re.S)
    structs = re.findall(r"typedef struct (\w+) \{", src)
    assert len(structs) >= 8
    for name in structs:
        mirror = getattr(_lib, name)
        buf = (ctypes.c_int64 * 64)()
        cnt = fn(name.encode(), buf, 64)
        assert cnt == len(mirror._fields_) + 1, (name, cnt, len(mirror._fields_))
        assert buf[0] == ctypes.sizeof(mirror), (name, buf[0], ctypes.sizeof(mirror))
        for k, (field, _) in enumerate(mirror._fields_):
            assert buf[k + 1] == getattr(mirror, field).offset, (name, field)
    assert fn(b"NoSuchStruct", (ctypes.c_int64 * 4)(), 4) == -1  # OTG_ERR_ARG
    assert fn(b"OtgDenseProblem", (ctypes.c_int64 * 4)(), 4) == -1  # cap too small
