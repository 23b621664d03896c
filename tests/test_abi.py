"""The C ABI: the library loads, exports every function include/kamino_gb300.h
declares, the ctypes structs match the C layouts, and argument errors come
back as status codes with a message (no GPU needed for these paths)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "kamino_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(kamino_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for must in ("kamino_create", "kamino_step", "kamino_advection", "kamino_geometric", "kamino_projection",
                 "kamino_set_state", "kamino_get_state", "kamino_run_frames", "kamino_parse_config",
                 "kamino_last_error"):
        assert must in names


def test_library_exports_every_declared_function(kg):
    missing = [n for n in declared_functions() if not hasattr(kg.lib, n)]
    assert not missing, missing


def test_struct_sizes_match_c(kg):
    sizes = (ctypes.c_size_t * 4)()
    assert kg.lib.kamino_abi_sizes(sizes, 4) == 0
    from kaminogpu_gb300 import _lib
    assert list(sizes) == [ctypes.sizeof(_lib.KaminoConfig), ctypes.sizeof(_lib.KaminoInitSpec),
                           ctypes.sizeof(_lib.KaminoServerConfig), ctypes.sizeof(_lib.KaminoServerStats)]


def test_invalid_sizes_are_rejected_with_a_message(kg):
    for nt in (0, 16, 100, 4096):
        cfg = kg.default_config(n_theta=nt, radius=1.0, dt=0.005)
        h = ctypes.c_void_p()
        rc = kg.lib.kamino_create(ctypes.byref(cfg), ctypes.byref(h))
        assert rc == kg.ERR_INVALID and not h.value
        assert "n_theta" in kg._lib.last_error()
    cfg = kg.default_config(n_theta=64, radius=-1.0, dt=0.005)
    assert kg.lib.kamino_create(ctypes.byref(cfg), ctypes.byref(ctypes.c_void_p())) == kg.ERR_INVALID
    cfg = kg.default_config(n_theta=64, radius=1.0, dt=0.0)
    assert kg.lib.kamino_create(ctypes.byref(cfg), ctypes.byref(ctypes.c_void_p())) == kg.ERR_INVALID
    assert kg.lib.kamino_create(None, None) == kg.ERR_INVALID


def test_null_handles_are_errors_not_crashes(kg):
    assert kg.lib.kamino_step(None, 0.01) == kg.ERR_INVALID
    assert kg.lib.kamino_set_state(None, 0, None, 0) == kg.ERR_INVALID
    assert kg.lib.kamino_destroy(None) == 0
    assert kg.lib.kamino_save_state(None, b"x") == kg.ERR_INVALID
    assert kg.lib.kamino_load_state(None, b"x") == kg.ERR_INVALID
    rc = kg.lib.kamino_projection_noalloc(512, None, None, None, None, None, None)
    assert rc == kg.ERR_INVALID and "n_theta" in kg._lib.last_error()
