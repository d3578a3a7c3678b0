"""Parity of the plain FP64 path at the size of the 1 M-cell configuration.

1,000,000 cells of the clustered spheroid (seed 2, radius calibrated to a mean
of 40 neighbours within h = 2.5), neighbour lists on, the CIC deposit onto the
257^3 FP64 grid of GFH 8 and x += dt F (dt = 0.01) every step: three steps on
the GPU against the CPU oracle on all host cores (the oracle is pinned to the
reference's own functions by the golden vectors).  Checked after the last
step (potential.c:39-138, 209-259; patches.c:156-234):

* density, mindist, v and positions within 1e-12 relative; forces within
  1e-12 of max |F|; the grid within 1e-12 of its largest value; removal marks
  exact;
* the neighbour sets of the last step, on the same positions: count and
  fingerprint of every cell, v's candidate, and the sorted lists of a
  12,000-cell sample, all equal to the oracle's octree walk over those
  positions.  The lists were built two steps before and are evaluated with
  the exact cutoff of the step, so this also checks the list-rebuild rule.
"""
import numpy as np
import pytest

from timothy_gb300 import colonies as C

pytestmark = pytest.mark.gpu

N, SEED, STEPS, DT, GFH = 1_000_000, 2, 3, 0.01, 8.0
FIELDS = ["x", "y", "z", "density", "v", "mindist", "fx", "fy", "fz", "removecell", "nbcount", "nbhash", "vcand",
          "grid"]


def _rel(a, b, floor=1e-300):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor))) if len(a) else 0.0


@pytest.fixture(scope="module")
def scale_run():
    from timothy_gb300 import session

    session.load_library()
    col = C.make_colony("clustered", N, SEED, C.configured_radius("clustered", N, SEED))
    rng = np.random.Generator(np.random.PCG64(77))
    sample = np.sort(rng.choice(N, 12_000, replace=False))
    with session.Session(col.types, dim=3, max_slots=N + 64, diagnostics=True, list_capacity=384) as s:
        cid = s.add_colony(col, precision="fp64", update="dt", dt=DT, cic=True, gfh=GFH, verlet=True)
        s.step(STEPS - 1)
        s.sync()
        before = s.download(cid, ["x", "y", "z"])
        s.sample_neighbours(cid, sample, lcap=512)
        s.step(1)
        s.sync()
        out = s.download(cid, FIELDS)
        lists = s.read_neighbours(cid)
        st = s.stats(cid)
    return col, sample, before, out, lists, st


def test_fp64_1m_with_lists_and_cic_matches_oracle(scale_run, oracle_lib):
    col, _, _, out, _, st = scale_run
    ref = oracle_lib.run(col, STEPS, which="oracle", update_mode=1, dt=DT, cic=True, gfh=GFH)
    for k in ("x", "y", "z"):
        assert _rel(out[k], getattr(ref, k), 1.0) <= 1e-12, k
    assert _rel(out["density"], ref.density) <= 1e-12
    fin = ref.mindist < 1e300
    assert np.array_equal(out["mindist"] < 1e300, fin)
    assert _rel(out["mindist"][fin], ref.mindist[fin]) <= 1e-12
    vscale = max(np.max(np.abs(ref.v)), 1e-300)
    assert np.max(np.abs(out["v"] - ref.v)) <= 1e-12 * vscale
    fscale = np.max(np.abs(np.stack([ref.fx, ref.fy, ref.fz])))
    for k in ("fx", "fy", "fz"):
        assert np.max(np.abs(out[k] - getattr(ref, k))) <= 1e-12 * fscale, k
    assert np.array_equal(out["removecell"], ref.removecell)
    assert st["octsize"] == ref.octsize
    gscale = np.max(np.abs(ref.grid))
    assert out["grid"].shape == ref.grid.shape
    assert np.max(np.abs(out["grid"] - ref.grid)) <= 1e-12 * gscale


def test_fp64_1m_neighbour_sets_exact(scale_run, oracle_lib):
    col, sample, before, out, lists, _ = scale_run
    at = col.copy()
    at.x, at.y, at.z = before["x"], before["y"], before["z"]
    nb = oracle_lib.neighbours(at, lists=True)
    assert np.array_equal(out["nbcount"], nb.count)
    assert np.array_equal(out["nbhash"], nb.hash)
    assert np.array_equal(out["vcand"], nb.vcand)
    assert int(np.sum(nb.count)) > 30 * N    # the sets are not trivially empty
    for k, c in enumerate(sample):
        want = np.sort(nb.lists[nb.offsets[c]:nb.offsets[c + 1]])
        assert np.array_equal(lists[k], want), (int(c), len(lists[k]), len(want))
