"""CPU: libyaffgb.so builds, loads, and exports every symbol that
include/yaffgb.h declares (no compute calls: no GPU here)."""
import ctypes
import os
import re

import pytest

from yaff_gb300 import _lib, build

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), 'include', 'yaffgb.h')


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
    return sorted(set(re.findall(r'\b(yg_[a-z0-9_]+)\s*\(', src)))


def test_library_builds_and_exports_all_symbols():
    path = build.build()
    lib = ctypes.CDLL(path)
    syms = declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_signature_table_covers_header():
    assert set(declared_symbols()) == set(_lib.SIGNATURES)


def test_status_strings():
    lib = _lib.load()
    assert lib.yg_status_string(0) == b'ok'
    assert b'density' in lib.yg_status_string(6)


def test_create_rejects_bad_arguments_without_gpu():
    lib = _lib.load()
    h = ctypes.c_void_p()
    assert lib.yg_create(0, 0, None, ctypes.byref(h)) == _lib.YG_ERR_ARG
    assert lib.yg_create(10, 7, None, ctypes.byref(h)) == _lib.YG_ERR_ARG
