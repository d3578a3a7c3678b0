"""The allocation-free CIC deposit (tm_cic_deposit_noalloc).

Callers that cannot call cudaMalloc -- code running during a CUDA graph
capture, hosts with a fixed device-memory budget, real-time loops -- pass
their own device buffers and get the deposit without any allocation; the
entry point's scratch is a fixed device array.  This test calls it through the
C ABI twice in a row and compares each result with the existing drop-in path
(patches_alloc + patches_cells2envinfo) on the same cells.  It runs last so a
failure here does not stop the other GPU tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _entry():
    from timothy_gb300 import session

    lib = session.load_library()
    fn = lib.tm_cic_deposit_noalloc
    P = C.c_void_p
    fn.argtypes = [P, P, P, P, C.c_int64, C.c_int, P, C.c_float, P, P, P, P]
    fn.restype = C.c_int
    return fn


def test_noalloc_deposit_matches_dropin_on_two_calls():
    torch = pytest.importorskip("torch")
    from timothy_gb300 import colonies as col_mod
    from timothy_gb300.refabi import DropinRun, grid_geometry

    fn = _entry()
    dev = torch.device("cuda", 0)
    gsize, lower = grid_geometry(3, 8.0)
    ngrid = gsize[0] * gsize[1] * gsize[2]
    grid = torch.empty(ngrid, dtype=torch.float64, device=dev)
    corners = torch.empty(6, dtype=torch.int64, device=dev)
    lower_h = np.array(lower, np.float64)
    gsize_h = np.array(gsize, np.int64)
    for call, seed in enumerate((41, 42)):
        col = col_mod.make_colony("clustered", 20000, seed, col_mod.initial_radius("clustered", 20000))
        run = DropinRun(col, cic=True)
        run.step(update=False)
        ref_grid = run.deposit.reshape(-1)
        ref_corners = run.patch_corners
        run.shutdown()

        x = torch.tensor(col.x, device=dev)
        y = torch.tensor(col.y, device=dev)
        z = torch.tensor(col.z, device=dev)
        ph = torch.tensor(col.phase, dtype=torch.int32, device=dev)
        grid.fill_(123.0)   # stale contents must not leak into the result
        stream = torch.cuda.current_stream(dev)
        rc = fn(x.data_ptr(), y.data_ptr(), z.data_ptr(), ph.data_ptr(), col.n, 3, lower_h.ctypes.data, 8.0,
                gsize_h.ctypes.data, grid.data_ptr(), corners.data_ptr(), stream.cuda_stream)
        assert rc == 0, f"call {call}: return code {rc}"
        torch.cuda.synchronize(dev)
        got = grid.cpu().numpy()
        scale = max(np.max(np.abs(ref_grid)), 1e-300)
        assert np.max(np.abs(got - ref_grid)) <= 1e-12 * scale, f"call {call}: grid differs"
        assert tuple(int(v) for v in corners.cpu().numpy()) == tuple(int(v) for v in ref_corners), f"call {call}"


def test_noalloc_rejects_oversized_input():
    fn = _entry()
    lower = np.array([-1024.0, -1024.0, -1024.0])
    gsize = np.array([257, 257, 257], np.int64)
    dummy = C.c_void_p(16)   # never dereferenced: the size check comes first
    rc = fn(dummy, dummy, dummy, dummy, (1 << 24) + 1, 3, lower.ctypes.data, 8.0, gsize.ctypes.data, dummy, dummy,
            None)
    assert rc == -1


def _call(fn, dev, x, y, z, ph, n, dim, lower, gsize, gfh=8.0):
    import torch

    grid = torch.full((int(np.prod(gsize)),), 123.0, dtype=torch.float64, device=dev)
    corners = torch.zeros(6, dtype=torch.int64, device=dev)
    lo = np.array(lower, np.float64)
    gs = np.array(gsize, np.int64)
    stream = torch.cuda.current_stream(dev)
    ptrs = [None if a is None else a.data_ptr() for a in (x, y, z, ph)]
    rc = fn(*ptrs, n, dim, lo.ctypes.data, gfh, gs.ctypes.data, grid.data_ptr(), corners.data_ptr(),
            stream.cuda_stream)
    torch.cuda.synchronize(dev)
    return rc, grid.cpu().numpy(), tuple(int(v) for v in corners.cpu().numpy())


def _expected_corners(x, y, z, dim, lower, gsize, gfh):
    """Touched-node box of patches_alloc (patches.c:61-132) computed here."""
    pos = [np.asarray(a, np.float64) for a in (x, y, z)]
    idx = [np.trunc((p - lo) / np.float64(np.float32(gfh))).astype(np.int64) for p, lo in zip(pos, lower)]
    up = [gsize[0] - 1, gsize[1] - 1, gsize[2] - 1 if dim == 3 else 0]
    lo_c, hi_c = [np.iinfo(np.int32).max] * 3, [np.iinfo(np.int32).min] * 3
    for ax in (0, 1):
        for ay in (0, 1):
            for az in (0, 1):
                c = [idx[0] + ax, idx[1] + ay, idx[2] + az]
                ok = np.ones(len(pos[0]), bool)
                for k in range(3):
                    ok &= (c[k] >= 0) & (c[k] <= up[k])
                for k in range(3):
                    if ok.any():
                        lo_c[k] = min(lo_c[k], int(c[k][ok].min()))
                        hi_c[k] = max(hi_c[k], int(c[k][ok].max()))
    if dim != 3:
        lo_c[2] = hi_c[2] = 0
    return tuple(lo_c + hi_c)


@pytest.mark.parametrize("name", ["clustered4k_cic", "uniform2d_2k_cic"])
def test_noalloc_deposit_matches_reference_golden(name):
    """The reference's own deposit (tests/golden, 3-D and a one-layer 2-D grid):
    the golden grid is the deposit of the last of its steps, so the cells are
    advanced to that step on the GPU first (within 1e-12 of the reference's
    positions) and then deposited through the allocation-free entry point."""
    torch = pytest.importorskip("torch")
    import os

    from timothy_gb300 import session
    from timothy_gb300.refabi import grid_geometry

    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", name + ".npz"))
    t = col_types(d)
    from timothy_gb300 import colonies as col_mod

    dim = int(d["dim"])
    col = col_mod.Colony(d["x"], d["y"], d["z"], d["size"], d["young"], d["ctype"], d["phase"], t, dim)
    update = {0: "reference", 1: "dt", 2: "none"}[int(d["update_mode"])]
    out, _ = session.run_colony(col, int(d["steps"]) - 1, precision="fp64", update=update, dt=float(d["dt"]),
                                fields=["x", "y", "z"])
    gfh = float(d["gfh"])
    gsize, lower = grid_geometry(dim, gfh)
    dev = torch.device("cuda", 0)
    xs = [torch.tensor(out[k], device=dev) for k in ("x", "y", "z")]
    ph = torch.tensor(col.phase, dtype=torch.int32, device=dev)
    shape = tuple(int(s) for s in d["strict_grid_shape"])
    want = np.zeros(shape)
    idx = d["strict_grid_idx"]
    if len(idx):
        want[idx[:, 0], idx[:, 1], idx[:, 2]] = d["strict_grid_val"]
    fn = _entry()
    for call in range(2):
        rc, got, corners = _call(fn, dev, *xs, ph, col.n, dim, lower, gsize, gfh)
        assert rc == 0, (name, call, rc)
        scale = max(np.max(np.abs(want)), 1e-300)
        assert np.max(np.abs(got.reshape(shape) - want)) <= 1e-12 * scale, (name, call)
        assert corners == _expected_corners(out["x"], out["y"], out["z"], dim, lower, gsize, gfh), (name, call)


def col_types(d):
    from timothy_gb300 import colonies as col_mod

    return col_mod.CellTypes(d["th"], d["th2"], d["th3"], d["th4"], d["tsize"], d["trandommove"])


@pytest.mark.parametrize("dim", [3, 2])
def test_noalloc_no_cells_gives_zero_grid_and_sentinel_corners(dim):
    """n = 0: a zeroed grid (stale contents cleared) and the corner values
    patches_alloc starts from, INT_MAX / INT_MIN, with z = 0 on a 2-D grid
    (patches.c:64-77)."""
    torch = pytest.importorskip("torch")
    from timothy_gb300.refabi import grid_geometry

    dev = torch.device("cuda", 0)
    gsize, lower = grid_geometry(dim, 8.0)
    imax, imin = np.iinfo(np.int32).max, np.iinfo(np.int32).min
    want = (imax, imax, imax if dim == 3 else 0, imin, imin, imin if dim == 3 else 0)
    fn = _entry()
    for call in range(2):
        rc, got, corners = _call(fn, dev, None, None, None, None, 0, dim, lower, gsize)
        assert rc == 0
        assert not np.any(got), call
        assert corners == want, (call, corners)
