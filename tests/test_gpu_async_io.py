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


def test_positions_only_upload_matches_full_upload():
    """An asynchronous upload of positions only (size, young, type and phase
    NULL keep their values) gives the same bits as the full upload of the
    same cells; the positions are fed back from the previous step's
    asynchronous download, as a host loop does."""
    from timothy_gb300.session import Session, host_register, host_unregister

    col = _colony(20_000, 6)
    outs = []
    for positions_only in (False, True):
        with Session(col.types, dim=3, max_slots=col.n + 64, list_capacity=384) as s:
            cid = s.add_colony(col, precision="fp32c", update="dt", dt=0.01, verlet=True)
            res = {k: np.zeros(col.n, np.uint8 if k == "removecell" else np.float64) for k in FIELDS}
            res["x"][:], res["y"][:], res["z"][:] = col.x, col.y, col.z
            for a in res.values():
                host_register(a)            # page-locked: the copies run asynchronously
            for _ in range(5):
                if positions_only:
                    s.upload_positions_async(cid, res["x"], res["y"], res["z"])
                else:
                    fed = C.Colony(res["x"], res["y"], res["z"], col.size, col.young, col.ctype, col.phase,
                                   col.types, 3)
                    s.upload_async(cid, fed)
                s.step(1)
                s.download_async(cid, FIELDS, res)
            s.sync()
            outs.append({k: v.copy() for k, v in res.items()})
            for a in res.values():
                host_unregister(a)
    for f in FIELDS:
        assert np.array_equal(outs[0][f], outs[1][f]), f


def test_async_download_of_grid_is_not_overwritten_by_the_next_step():
    """The grid of an asynchronous download is staged: the step queued after
    it clears and re-deposits the session grid while the copy may still run,
    and the host still receives the grid of the step it asked for."""
    from timothy_gb300.session import Session, host_register, host_unregister

    col = _colony(20_000, 8)
    with Session(col.types, dim=3, max_slots=col.n + 64) as s:
        cid = s.add_colony(col, precision="fp64", update="dt", dt=0.05, cic=True)
        s.step(1)
        s.sync()
        want = s.download(cid, ["grid"])["grid"].copy()
        got = {"grid": np.zeros_like(want)}
        host_register(got["grid"])      # page-locked: the copy runs asynchronously
        s.download_async(cid, ["grid"], got)
        s.step(2)                       # clears and deposits the grid again
        s.sync()
        host_unregister(got["grid"])
        after = s.download(cid, ["grid"])["grid"]
    assert np.array_equal(got["grid"], want)
    assert not np.array_equal(after, want)      # the later steps did change it
