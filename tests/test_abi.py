"""The C-ABI library loads without a GPU and exports every declared entry point."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")


@pytest.fixture(scope="module")
def lib():
    from timothy_gb300 import build

    path = build.build()
    return ctypes.CDLL(path)


def declared_functions():
    names = set()
    for h in os.listdir(INCLUDE):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(INCLUDE, h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"^\s*(?:extern\s+)?[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\([^;{]*\)\s*;", text, re.M):
            name = m.group(1)
            if name not in ("if", "while", "for", "return", "sizeof"):
                names.add(name)
    return sorted(names)


def test_headers_declare_entry_points():
    names = declared_functions()
    assert "tm_session_create" in names
    assert len(names) >= 15


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_version_and_device_count_callable_without_gpu(lib):
    lib.tm_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.tm_version()
    lib.tm_device_count.restype = ctypes.c_int
    assert lib.tm_device_count() >= 0
