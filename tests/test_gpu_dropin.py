"""The reference-signature drop-ins, driven as the reference step loop drives them.

Cells are a host array of celldata_t; octbuild / patches_* / computepotential /
computegradient / updatepositions are called through the C ABI and the
results compared with the reference's own outputs (tests/golden).
"""
import ctypes
import glob
import os

import numpy as np
import pytest

from timothy_gb300 import colonies as C

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
               if not os.path.basename(p).startswith(("field_", "chain_")))

pytestmark = pytest.mark.gpu


def load_case(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    t = C.CellTypes(d["th"], d["th2"], d["th3"], d["th4"], d["tsize"], d["trandommove"])
    col = C.Colony(d["x"], d["y"], d["z"], d["size"], d["young"], d["ctype"], d["phase"], t, int(d["dim"]))
    return d, col


def golden_grid(d):
    shape = tuple(int(s) for s in d["strict_grid_shape"])
    g = np.zeros(shape)
    idx = d["strict_grid_idx"]
    if len(idx):
        g[idx[:, 0], idx[:, 1], idx[:, 2]] = d["strict_grid_val"]
    return g


def rel(a, b, floor=1e-300):
    if np.asarray(a).size == 0:
        return 0.0
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor)))


@pytest.mark.parametrize("name", [c for c in CASES])
def test_dropins_match_reference(name):
    from timothy_gb300.refabi import DropinRun

    d, col = load_case(name)
    mode = int(d["update_mode"])
    steps = int(d["steps"]) if mode == 0 else 1
    run = DropinRun(col, cic=bool(d["cic"]), gfh=float(d["gfh"]))
    for k in range(steps):
        run.step(update=(mode == 0))
    out = run.outputs()
    if mode == 0:
        ref = {k: d[f"strict_{k}"] for k in ("x", "y", "z", "density", "v", "mindist", "fx", "fy", "fz",
                                             "removecell")}
        if col.n:
            assert run.octsize == int(d["strict_octsize"])
            assert rel(run.aff, d["strict_aff"], 1.0) <= 1e-13
        assert int(run.removecount.value) == int(d["strict_removecount"])
    else:
        from oracle import bindings

        r = bindings.run(col, 1, which="oracle", update_mode=2, cic=bool(d["cic"]), gfh=float(d["gfh"]))
        ref = {k: getattr(r, k) for k in ("x", "y", "z", "density", "v", "mindist", "fx", "fy", "fz", "removecell")}
    n = col.n
    for k in ("x", "y", "z"):
        assert rel(out[k], ref[k], 1.0) <= 1e-12, k
    if n > 1:
        assert rel(out["density"], ref["density"]) <= 1e-12
        fin = ref["mindist"] < 1e300
        assert np.array_equal(out["mindist"] > 1e300, ref["mindist"] > 1e300)
        assert rel(out["mindist"][fin], ref["mindist"][fin]) <= 1e-12
        vs = max(np.max(np.abs(ref["v"])), 1e-300)
        assert np.max(np.abs(out["v"] - ref["v"])) <= 1e-12 * vs
        fs = max(np.max(np.abs(np.stack([ref["fx"], ref["fy"], ref["fz"]]))), 1e-300)
        for k in ("fx", "fy", "fz"):
            assert np.max(np.abs(out[k] - ref[k])) <= 1e-12 * fs, k
    assert np.array_equal(out["removecell"], ref["removecell"])
    if int(d["cic"]) and mode == 0:
        g = golden_grid(d)
        assert np.max(np.abs(run.deposit - g)) <= 1e-12 * max(np.max(np.abs(g)), 1e-300)
    run.shutdown()


def test_dropin_halo_cells_are_rejected_only_with_imports():
    """computeremote* are no-ops at one rank (numimp <= 0), as in the reference."""
    from timothy_gb300.refabi import DropinRun

    col = C.make_colony("uniform", 500, 3, 8.0)
    run = DropinRun(col)
    run.cc.numimp = 0
    run.step(update=False)
    out = run.outputs()
    assert np.all(np.isfinite(out["density"]))
    run.shutdown()


@pytest.mark.parametrize("lists", [False, True])
def test_dropins_fp32c_within_tolerance(oracle_lib, lists):
    """tm_dropin_set_precision(TM_PREC_FP32C, lists): the reference step loop
    through the drop-ins on the FP32 + compensated path (searching the bins
    every step, or keeping neighbour lists while the host keeps the same
    cells).  One step against the oracle's FP64 step on the same cells:
    density and mindist within 1e-6 relative, forces within 1e-6 of max |F|.
    Then four steps of x += F (the reference's update): every step's force
    error is within 1e-6 of that step's max |F|, so the positions stay within
    4e-6 of max |F| (with a factor 2 for the compounding) of the FP64 run's."""
    from timothy_gb300 import session
    from timothy_gb300.refabi import DropinRun

    lib = session.load_library()
    lib.tm_dropin_set_precision.argtypes = [ctypes.c_int, ctypes.c_int]
    col = C.make_colony("clustered", 20000, 51, C.initial_radius("clustered", 20000))
    steps = 4
    lib.tm_dropin_set_precision(1, 1 if lists else 0)
    try:
        run = DropinRun(col)
        run.step(update=False)
        one = run.outputs()
        run.shutdown()
        run = DropinRun(col)
        for _ in range(steps):
            run.step(update=True)
        out = run.outputs()
        run.shutdown()
    finally:
        lib.tm_dropin_set_precision(0, 0)
    ref1 = oracle_lib.run(col, 1, which="oracle", update_mode=2)
    pos = ref1.density > 0
    assert rel(one["density"][pos], ref1.density[pos]) <= 1e-6
    fin = ref1.mindist < 1e300
    assert rel(one["mindist"][fin], ref1.mindist[fin]) <= 1e-6
    f = np.stack([ref1.fx, ref1.fy, ref1.fz])
    g = np.stack([one["fx"], one["fy"], one["fz"]])
    assert np.max(np.abs(g - f)) <= 1e-6 * np.max(np.abs(f))
    ref = oracle_lib.run(col, steps, which="oracle", update_mode=0)
    fmax = np.max(np.abs(f))
    for k in ("x", "y", "z"):
        assert np.max(np.abs(out[k] - getattr(ref, k))) <= 2 * steps * 1e-6 * fmax, k
    assert np.array_equal(out["removecell"], ref.removecell)


def test_updatepositions_leaves_the_callers_rand_where_rand_calls_would():
    """updatepositions takes 3 values of the host program's rand() per cell
    (cells.c:353-356); generated on the device from the C library's
    generator window, they must equal those calls' values and leave the
    generator at the same place: the next rand() after a step is the value
    after 3 n calls, and the cells moved with randommove > 0 match a second
    run whose draws come from rand() calls on the host."""
    from timothy_gb300.refabi import DropinRun

    libc = ctypes.CDLL(None)
    libc.srand.argtypes = [ctypes.c_uint]
    libc.rand.restype = ctypes.c_int
    n = 5000
    t = C.CellTypes.consistent(randommove=[0.05])
    col = C.make_colony("uniform", n, 61, C.initial_radius("uniform", n), types=t)
    libc.srand(4242)
    run = DropinRun(col)
    run.step(update=True)
    after = libc.rand()
    out = run.outputs()
    run.shutdown()
    libc.srand(4242)
    draws = np.array([libc.rand() for _ in range(3 * n)], np.int64)
    want_next = libc.rand()
    assert after == want_next
    # the move applied: x += F + randommove * (2 * (float)r / RAND_MAX - 1), cell by cell in order
    r = draws.reshape(n, 3).astype(np.float32) / np.float32(2147483647)
    step = np.float64(np.float32(0.05)) * (r.astype(np.float64) * 2.0 - 1.0)
    ref = DropinRun(col)
    ref.step(update=False)
    f = ref.outputs()
    ref.shutdown()
    for k, ax in enumerate(("x", "y", "z")):
        want = (getattr(col, ax) + f["f" + ax]) + step[:, k]
        assert np.max(np.abs(out[ax] - want)) <= 1e-12 * max(1.0, np.max(np.abs(want))), ax
