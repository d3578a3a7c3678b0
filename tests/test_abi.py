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


def test_struct_layout_matches_reference_abi():
    """The ctypes mirror and include/timothy_refabi.h keep the reference layout."""
    import ctypes as C

    from timothy_gb300 import refabi as R

    for name, size in R.SIZES.items():
        assert C.sizeof(getattr(R, name)) == size, name
    cd = R.celldata_t
    assert (cd.young.offset, cd.x.offset, cd.size.offset, cd.v.offset, cd.density.offset, cd.mindist.offset,
            cd.ctype.offset) == (36, 48, 72, 80, 88, 96, 104)
    assert (R.celltype_t.h.offset, R.celltype_t.size.offset, R.celltype_t.randommove.offset) == (160, 152, 360)


def test_header_layout_compiles_to_reference_sizes(tmp_path):
    """Compile include/timothy_refabi.h and compare with the reference's own structs when built here."""
    import subprocess

    src = tmp_path / "sz.c"
    src.write_text('#include <stdio.h>\n#include "timothy_refabi.h"\nint main(void){printf("%zu %zu %zu %zu %zu '
                   '%zu %zu %zu %zu %zu %zu\\n", sizeof(celldata_t), sizeof(cellsinfo_t), sizeof(celltype_t), '
                   'sizeof(systeminfo_t), sizeof(settings_t), sizeof(cellcommdata_t), sizeof(grid_t), '
                   'sizeof(patches_t), sizeof(octnode_t), sizeof(environment_t), sizeof(cellenvdata_t));'
                   'return 0;}\n')
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", INCLUDE, str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert got[:6] == [112, 192, 368, 56, 336, 104]
    assert got[9:] == [192, 32]
    from oracle import bindings

    if bindings.available("ref"):
        try:
            lib = bindings.load("ref")
        except OSError:
            return
        ref = [lib.ref_sizeof(k) for k in range(11)]
        assert got == ref
