"""Pipelined host I/O (tm_colony_upload_async / tm_colony_download_async):
the same results, bit for bit, as the synchronous upload and download, with
step k + 1's upload queued while step k's results travel back; a cell type
outside the table in an asynchronous upload is read as 0 by the kernel's own
check and reported at the next sync."""
import numpy as np
import pytest

from timothy_gb300 import colonies as C

pytestmark = pytest.mark.gpu
FIELDS = ["x", "y", "z", "density", "v", "mindist", "fx", "fy", "fz", "removecell"]


def _colony(n=30_000, seed=4):
    return C.make_colony("clustered", n, seed, C.initial_radius("clustered", n))


def _run(col, steps, pipelined):
    from timothy_gb300.session import Session

    out = []
    with Session(col.types, dim=3, max_slots=col.n + 64, list_capacity=384) as s:
        cid = s.add_colony(col, precision="fp32c", update="dt", dt=0.01, verlet=True)
        s.step(1)
        s.sync()
        res = [{k: np.zeros(col.n, np.uint8 if k == "removecell" else np.float64) for k in FIELDS}
               for _ in range(steps)]
        for k in range(steps):
            if pipelined:
                s.upload_async(cid, col)
                s.step(1)
                s.download_async(cid, FIELDS, res[k])
            else:
                s.upload(cid, col)
                s.step(1)
                s.download(cid, FIELDS, out=res[k])
        s.sync()
        out = res
    return out


def test_pipelined_io_matches_synchronous():
    col = _colony()
    a = _run(col, 4, pipelined=False)
    b = _run(col, 4, pipelined=True)
    for k in range(4):
        for f in FIELDS:
            assert np.array_equal(a[k][f], b[k][f]), (k, f)


def test_async_upload_reports_bad_type():
    from timothy_gb300.session import Session, TimothyError

    col = _colony(5000)
    with Session(col.types, dim=3, max_slots=col.n + 64) as s:
        cid = s.add_colony(col, precision="fp64", update="dt", dt=0.01)
        s.step(1)
        s.sync()
        bad = C.Colony(col.x, col.y, col.z, col.size, col.young, col.ctype.copy(), col.phase, col.types, 3)
        bad.ctype[17] = 5
        s.upload_async(cid, bad)
        with pytest.raises(TimothyError):
            s.sync()
