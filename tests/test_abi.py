"""The C-ABI library builds, loads and exports every symbol include/ee_cccs.h
declares; calls that need no GPU behave (errors are status codes, never an
exit)."""
import ctypes as C
import os
import re

import pytest

from endtoend_gb300 import _build, engine

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if not fn.endswith(".h"):
            continue
        txt = open(os.path.join(ROOT, "include", fn)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names |= set(re.findall(r"\b(ee_[a-z0-9_]+)\s*\(", txt))
    return names


def test_library_exports_all_declared_symbols():
    path = _build.build()
    lib = C.CDLL(path)
    declared = _declared_symbols()
    assert declared, "no declarations found"
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, missing
    # the Python binding covers exactly the declared surface
    assert declared == set(engine._SIGS), declared ^ set(engine._SIGS)


def test_abi_version_and_error_paths_without_gpu():
    lib = engine.load_library(build_if_missing=True)
    assert lib.ee_abi_version() == 1
    # null arguments are rejected with a status code and a message
    st = lib.ee_create(0, None)
    assert st == engine.EE_ERR_INVALID_ARG
    assert b"null" in lib.ee_last_error()
    assert lib.ee_destroy(None) == 0
    assert lib.ee_synchronize(None) == engine.EE_ERR_INVALID_ARG


def test_engine_requires_built_library(monkeypatch, tmp_path):
    monkeypatch.setattr(engine, "_LIB", None)
    monkeypatch.setattr(_build, "LIB", str(tmp_path / "missing.so"))
    with pytest.raises(ImportError):
        engine.load_library()
