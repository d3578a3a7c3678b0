"""The link recipe of the reference-signature drop-ins (no GPU needed).

A program keeps the reference's own object files for cells.c, patches.c and
fieldgradient.c (they hold functions the drop-ins do not replace, such as
cellsupdate, which calls updatepositions in the same file).  The recipe:
compile those files with -fPIC, so calls between functions of one file go
through the symbol; weaken the replaced symbols; link the drop-ins as regular
objects (libtimothy_gb300_dropin.a, whole archive), because a definition in a
shared library never replaces one in the program, weak or not.

The stand-in "reference" object below defines updatepositions (marking the
cells it moves) and cellsupdate calling it.  With no cells the drop-in's
updatepositions returns before any device work, so which definition ran is
visible on a machine without a GPU: the reference's would leave its mark.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "timothy_gb300")

REFERENCE_LIKE = r"""
#include <stdint.h>
#include "timothy_refabi.h"
int ref_marker = 0;
void updatepositions(settings_t settings, celltype_t *celltype, cellsinfo_t *cellsinfo, unsigned char *removecell,
                     int64_t *removecount)
{
    (void)settings; (void)celltype; (void)cellsinfo; (void)removecell; (void)removecount;
    ref_marker = 1;                       /* the CPU version ran */
}
void cellsupdate_like(settings_t settings, celltype_t *celltype, cellsinfo_t *cellsinfo)
{
    unsigned char rem[1];
    int64_t count = 0;
    updatepositions(settings, celltype, cellsinfo, rem, &count);   /* same file, as cells.c:538 */
}
"""

MAIN = r"""
#include <stdio.h>
#include <string.h>
#include "timothy_refabi.h"
extern int ref_marker;
void cellsupdate_like(settings_t settings, celltype_t *celltype, cellsinfo_t *cellsinfo);
int main(void)
{
    settings_t st;
    cellsinfo_t ci;
    celltype_t ct;
    unsigned char rem[1];
    int64_t count = 0;
    memset(&st, 0, sizeof st);
    memset(&ci, 0, sizeof ci);
    memset(&ct, 0, sizeof ct);
    st.dimension = 3;
    ci.dimension = 3;                     /* no cells: the drop-in returns at once */
    cellsupdate_like(st, &ct, &ci);
    int via_file = ref_marker;
    ref_marker = 0;
    updatepositions(st, &ct, &ci, rem, &count);
    printf("%d %d\n", via_file, ref_marker);
    return 0;
}
"""


def _have(tool):
    return shutil.which(tool) is not None


@pytest.fixture(scope="module")
def built():
    from timothy_gb300 import build

    build.build()
    assert os.path.exists(build.DROPIN_LIB)
    return build


def _link_and_run(tmp_path, built, *, pic: bool, static_dropins: bool):
    inc = os.path.join(ROOT, "include")
    ref = tmp_path / "cells_like.c"
    ref.write_text(REFERENCE_LIKE)
    main = tmp_path / "main.c"
    main.write_text(MAIN)
    obj = str(tmp_path / "cells_like.o")
    cflags = ["-O2", "-finline-functions", "-I", inc] + (["-fPIC"] if pic else [])
    subprocess.run(["gcc"] + cflags + ["-c", str(ref), "-o", obj], check=True)
    subprocess.run(["objcopy", "--weaken-symbol=updatepositions", obj], check=True)
    mobj = str(tmp_path / "main.o")
    subprocess.run(["gcc", "-O2", "-I", inc, "-c", str(main), "-o", mobj], check=True)
    exe = str(tmp_path / "prog")
    cuda_lib = "/usr/local/cuda/lib64"
    link = ["gcc", mobj, obj]
    if static_dropins:
        link += ["-Wl,--whole-archive", built.DROPIN_LIB, "-Wl,--no-whole-archive"]
    link += ["-L", PKG, "-ltimothy_gb300", f"-Wl,-rpath,{PKG}", "-L", cuda_lib, "-lcudart", f"-Wl,-rpath,{cuda_lib}",
             "-o", exe]
    subprocess.run(link, check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    return int(out[0]), int(out[1])


@pytest.mark.skipif(not (_have("gcc") and _have("objcopy")), reason="needs gcc and objcopy")
def test_recipe_replaces_calls_within_the_file(tmp_path, built):
    via_file, direct = _link_and_run(tmp_path, built, pic=True, static_dropins=True)
    assert (via_file, direct) == (0, 0)          # the drop-in ran both times


@pytest.mark.skipif(not (_have("gcc") and _have("objcopy")), reason="needs gcc and objcopy")
def test_shared_library_alone_does_not_replace(tmp_path, built):
    """Why the recipe needs the archive: the program's own (weak) definition
    wins over the shared library's."""
    via_file, direct = _link_and_run(tmp_path, built, pic=True, static_dropins=False)
    assert (via_file, direct) == (1, 1)


def test_remote_walk_with_imported_cells_stops_the_program():
    """computeremotepotential with imported halo cells (numimp > 0) ends the
    program through the reference's error exit (terminate(), else abort with
    the message), as the GB300 path runs one MPI rank.  Run in a child
    process; nothing touches a GPU before the check."""
    import subprocess
    import sys
    import textwrap

    code = textwrap.dedent(f"""
        import ctypes, sys
        sys.path.insert(0, {ROOT!r})
        from timothy_gb300 import session
        from timothy_gb300 import refabi as R
        lib = R._bind(session.load_library())
        si = R.systeminfo_t(); si.size = 1
        ci = R.cellsinfo_t(); ci.localcount.n = 10
        ct = (R.celltype_t * 1)()
        cc = R.cellcommdata_t(); cc.numimp = 3
        lib.computeremotepotential(si, ctypes.byref(ci), ct, cc)
        print("returned")
    """)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120)
    assert r.returncode != 0
    assert "returned" not in r.stdout
    assert "halo cells" in r.stderr
