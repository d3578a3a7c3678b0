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
