"""The C-ABI library builds for sm_103a, loads, and exports every entry point
that include/*.h declares (no compute calls: no GPU here)."""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(st_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from structured_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    names = declared_functions()
    assert "st_create" in names and "st_residual" in names and "st_vjp_device" in names


@pytest.mark.parametrize("name", declared_functions())
def test_symbol_exported(lib, name):
    assert hasattr(lib, name), name


def test_error_path_without_device(lib):
    lib.st_last_error.restype = ctypes.c_char_p
    lib.st_create.restype = ctypes.c_int
    out = ctypes.c_void_p()
    rc = lib.st_create(None, None, None, 0, ctypes.byref(out))
    assert rc == -1
    assert b"null" in lib.st_last_error()
