"""CPU-only checks of the C-ABI library: it loads and exports every symbol that
include/tgdns.h declares, and the ctypes table matches the header."""
import os
import re

import pytest

from conftest import REPO

HEADER = os.path.join(REPO, "include", "tgdns.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(tg_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_the_abi():
    names = declared_functions()
    for must in ("tg_plan_create", "tg_step", "tg_run", "tg_rhs", "tg_diagnostics", "tg_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol():
    from jax_tg_project_gb300 import _abi, _build
    if not os.path.exists(_build.LIB):
        pytest.skip("libtgdns.so not built (run __graft_entry__.build())")
    lib = _abi.load()
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert set(declared_functions()) == set(_abi.SIGNATURES)
    assert lib.tg_version() >= 100


def test_errors_are_reported_without_a_gpu():
    """Argument validation happens before any CUDA call."""
    import ctypes
    from jax_tg_project_gb300 import _abi, _build
    if not os.path.exists(_build.LIB):
        pytest.skip("libtgdns.so not built")
    lib = _abi.load()
    h = ctypes.c_void_p()
    desc = _abi.TgDesc(100, 1, 0, 0, 0, 0)  # 100 is not a built size
    rc = lib.tg_plan_create(ctypes.byref(h), ctypes.byref(desc))
    assert rc == _abi.TG_E_UNSUPPORTED
    assert b"grid size 100" in lib.tg_last_error()
    desc = _abi.TgDesc(64, 0, 0, 0, 0, 0)
    assert lib.tg_plan_create(ctypes.byref(h), ctypes.byref(desc)) == _abi.TG_E_INVALID
    assert lib.tg_step(None, None, 0.1, 0.01, 0.0, 1) == _abi.TG_E_INVALID


def declared_arity():
    """Parameter count of every tg_* declaration in the header (comments removed)."""
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for m in re.finditer(r"\b(tg_\w+)\s*\(([^;{]*?)\)\s*;", text, flags=re.S):
        params = m.group(2).strip()
        out[m.group(1)] = 0 if params in ("", "void") else params.count(",") + 1
    return out


def test_ctypes_signatures_match_the_header_arity():
    from jax_tg_project_gb300 import _abi
    arity = declared_arity()
    assert set(arity) == set(_abi.SIGNATURES)
    for name, (_, argtypes) in _abi.SIGNATURES.items():
        assert len(argtypes) == arity[name], (name, len(argtypes), arity[name])
