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


def test_invalid_arguments_are_rejected_before_any_device_work():
    """The C ABI reports bad arguments with its error codes before touching a
    device (these calls run without a GPU): null problem structs and buffers,
    unknown dtypes, sizes the fused kernels do not cover."""
    from pot_gb300 import _build, _lib
    lib = ctypes.CDLL(_build.build())
    for name, (res, args) in _lib.SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype, fn.argtypes = res, args
    ERR_ARG, ERR_DTYPE, ERR_UNSUPPORTED = -1, -2, -5
    assert lib.otg_sinkhorn_dense(None, None, None) == ERR_ARG
    assert lib.otg_sinkhorn_dense_noalloc(None, None, None, None) == ERR_ARG
    assert lib.otg_sinkhorn_multi(None, None) == ERR_ARG
    assert lib.otg_sinkhorn_pairs(None, None) == ERR_ARG
    assert lib.otg_pairs_max_cost(None, None, None) == ERR_ARG
    assert lib.otg_batched_sqdist(None, 1, None) == ERR_ARG
    assert lib.otg_dense_plan(0, 1, None, 4, 4, 4, None, None, 1.0, None, 0, None, None) == ERR_ARG
    assert lib.otg_gibbs_kernel(0, None, 4, 4, 4, 1.0, None, 4, None) == ERR_ARG
    assert lib.otg_softmin_points(None, None, 1, 8, 4, 16, 128, 64, None, None, 0.0, None, None, 0, None, None,
                                  None) == ERR_ARG
    cl, mx, err = _lib.c_i32(), _lib.c_i32(), _lib.c_i32()
    tile = _lib.c_i64()
    assert lib.otg_multi_tail_config(7, ctypes.byref(cl), ctypes.byref(mx), ctypes.byref(tile),
                                     ctypes.byref(err)) == ERR_DTYPE
    # the fused network kernels cover the shipped sizes only (pointers are not read)
    fake = ctypes.c_void_p(16)
    assert lib.otg_mlp_encode_pool(fake, 1, 1, 5, 32, 32, fake, fake, fake, fake, fake, None) == ERR_UNSUPPORTED
    assert lib.otg_mlp_head(fake, 1, 1, 7, 32, 64, fake, fake, fake, fake, fake, fake, fake, fake, fake,
                            None) == ERR_UNSUPPORTED


def test_greenkhorn_entry_checks_before_device_work():
    """otg_greenkhorn rejects bad arguments (null buffers, ldm < m, a warm
    start for one side only, unknown dtype, short workspace) before it touches
    a device, and sizes its workspace as K + K^T + both violation vectors."""
    from pot_gb300 import _build, _lib
    lib = ctypes.CDLL(_build.build())
    for name in ("otg_greenkhorn", "otg_greenkhorn_workspace_bytes"):
        fn = getattr(lib, name)
        fn.restype, fn.argtypes = _lib.SIGNATURES[name]
    ERR_ARG, ERR_DTYPE, ERR_WORKSPACE = -1, -2, -3
    f = ctypes.c_void_p(256)
    info = ctypes.c_void_p(512)

    def call(dtype=1, M=f, n=4, m=5, ldm=5, wu=None, wv=None, iters=10, ws=f, wsb=1 << 20):
        return lib.otg_greenkhorn(dtype, M, n, m, ldm, f, f, 1.0, wu, wv, iters, 1e-9, f, m, f, f, info, ws, wsb,
                                  None)

    assert call(M=None) == ERR_ARG
    assert call(ldm=4) == ERR_ARG
    assert call(n=0) == ERR_ARG
    assert call(iters=-1) == ERR_ARG
    assert call(wu=f) == ERR_ARG
    assert call(dtype=7) == ERR_DTYPE
    assert call(wsb=16) == ERR_WORKSPACE
    assert call(ws=None) == ERR_WORKSPACE
    assert lib.otg_greenkhorn_workspace_bytes(1, 1024, 1024) == 2 * (8 << 20) + 2 * 8192
    assert lib.otg_greenkhorn_workspace_bytes(0, 3, 5) == 2 * 256 + 256 + 256
    assert lib.otg_greenkhorn_workspace_bytes(1, 0, 5) == 0
