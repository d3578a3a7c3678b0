"""The reference-signature drop-ins, driven as the reference step loop drives them.

Cells are a host array of celldata_t; octbuild / patches_* / computepotential /
computegradient / updatepositions are called through the C ABI and the
results compared with the reference's own outputs (tests/golden).
"""
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
