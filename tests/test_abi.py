"""CPU checks of the drop-in boundary: the C-ABI library builds, loads without a
GPU, and exports every entry point include/phx.h declares."""
import ctypes
import os
import re

import pytest

from photon_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "phx.h")).read()
    return sorted(set(re.findall(r"\b(phx_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return ctypes.CDLL(_lib.lib_path())


def test_every_declared_symbol_is_exported(lib):
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s


def test_python_binding_covers_header():
    assert sorted(_lib.SYMBOLS) == declared_symbols()


def test_abi_version(lib):
    assert lib.phx_abi_version() == 1


def test_field_and_stage_tables_match_header():
    text = open(os.path.join(ROOT, "include", "phx.h")).read()
    fields = re.findall(r"PHX_FIELD_([A-Z0-9]+)", text)
    fields = [f for f in fields if f != "COUNT"]
    seen = []
    for f in fields:
        if f not in seen:
            seen.append(f)
    assert [f.lower() for f in seen] == [f.lower() for f in _lib.FIELDS]
    stages = []
    for s in re.findall(r"PHX_STAGE_([A-Z]+)", text):
        if s != "COUNT" and s not in stages:
            stages.append(s)
    assert [s.lower() for s in stages] == _lib.STAGES


def test_create_rejects_bad_input_without_gpu():
    L = _lib.load()
    h = ctypes.c_void_p()
    assert L.phx_create(None, 0, ctypes.byref(h)) == _lib.PHX_ERR_INVALID
    g = _lib.PhxGrid()
    g.nx = 0
    assert L.phx_create(ctypes.byref(g), 0, ctypes.byref(h)) == _lib.PHX_ERR_INVALID
    assert b"invalid" in L.phx_last_global_error()
    assert L.phx_create(ctypes.byref(g), 7, ctypes.byref(h)) == _lib.PHX_ERR_INVALID
