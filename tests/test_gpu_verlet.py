"""Neighbour lists (Verlet mode): steps between rebuilds reuse lists of
neighbours within h + skin but decide the cutoff every step, so every step's
results must equal the search-every-step path and the oracle."""
import numpy as np
import pytest

from timothy_gb300 import colonies as C

pytestmark = pytest.mark.gpu


def rel(a, b, floor=1e-300):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor), initial=0.0))


def check64(out, ref, tag):
    for k in ("x", "y", "z"):
        assert rel(out[k], getattr(ref, k), 1.0) <= 1e-12, (tag, k)
    assert rel(out["density"], ref.density) <= 1e-12, tag
    fin = ref.mindist < 1e300
    assert rel(out["mindist"][fin], ref.mindist[fin]) <= 1e-12, tag
    vs = max(np.max(np.abs(ref.v)), 1e-300)
    assert np.max(np.abs(out["v"] - ref.v)) <= 1e-12 * vs, tag
    fs = np.max(np.abs(np.stack([ref.fx, ref.fy, ref.fz])))
    for k in ("fx", "fy", "fz"):
        assert np.max(np.abs(out[k] - getattr(ref, k))) <= 1e-12 * fs, (tag, k)


@pytest.mark.parametrize("dt,steps", [(0.01, 30), (0.5, 12)])
def test_verlet_fp64_multistep_matches_oracle(oracle_lib, dt, steps):
    from timothy_gb300 import session as S

    col = C.make_colony("clustered", 30000, 31, C.initial_radius("clustered", 30000))
    out, st = S.run_colony(col, steps, precision="fp64", update="dt", dt=dt, verlet=True, rmax=16)
    ref = oracle_lib.run(col, steps, which="oracle", update_mode=1, dt=dt)
    check64(out, ref, f"dt={dt}")
    assert st["octsize"] == ref.octsize
    assert st["list_rebuilds"] >= 2          # first step + age or displacement
    assert st["list_rebuilds"] < steps or dt > 0.1


def test_verlet_neighbour_sets_exact_between_rebuilds(oracle_lib):
    from timothy_gb300 import session as S

    col = C.make_colony("uniform", 20000, 32, C.initial_radius("uniform", 20000))
    with S.Session(col.types, max_slots=col.n + 64, diagnostics=True, list_capacity=256) as s:
        cid = s.add_colony(col, precision="fp64", update="dt", dt=0.01, verlet=True, rmax=16)
        s.step(5)
        s.sync()
        pos = s.download(cid, ["x", "y", "z"])
        s.set_active(cid, True)
        # one more step without moving, then compare on the same positions
        s.step(1)
        s.sync()
        st = s.stats(cid)
    assert st["list_rebuilds"] == 1
    moved = C.Colony(pos["x"], pos["y"], pos["z"], col.size, col.young, col.ctype, col.phase, col.types)
    out, _ = S.run_colony(moved, 1, precision="fp64", update="none", diagnostics=True)
    nb = oracle_lib.neighbours(moved)
    assert np.array_equal(out["nbcount"], nb.count)
    assert np.array_equal(out["nbhash"], nb.hash)
    assert np.array_equal(out["vcand"], nb.vcand)


def test_verlet_step_outputs_equal_search_every_step():
    from timothy_gb300 import session as S

    col = C.make_colony("clustered", 25000, 33, C.initial_radius("clustered", 25000))
    a, sa = S.run_colony(col, 10, precision="fp64", update="dt", dt=0.02, verlet=True, diagnostics=True)
    b, sb = S.run_colony(col, 10, precision="fp64", update="dt", dt=0.02, verlet=False, diagnostics=True)
    assert sa["list_rebuilds"] < 10
    assert np.array_equal(a["nbcount"], b["nbcount"])
    assert np.array_equal(a["nbhash"], b["nbhash"])
    assert np.array_equal(a["vcand"], b["vcand"])
    assert rel(a["density"], b["density"]) <= 1e-13
    fs = np.max(np.abs(np.stack([b["fx"], b["fy"], b["fz"]])))
    for k in ("fx", "fy", "fz"):
        assert np.max(np.abs(a[k] - b[k])) <= 1e-13 * fs


def test_verlet_fp32_against_fp64():
    from timothy_gb300 import session as S

    col = C.make_colony("clustered", 40000, 34, C.initial_radius("clustered", 40000))
    o64, _ = S.run_colony(col, 8, precision="fp64", update="dt", dt=0.01, verlet=True, diagnostics=True)
    o32, s32 = S.run_colony(col, 8, precision="fp32c", update="dt", dt=0.01, verlet=True, diagnostics=True)
    assert s32["list_rebuilds"] < 8
    assert np.array_equal(o32["nbcount"], o64["nbcount"])
    pos = o64["density"] > 0
    assert rel(o32["density"][pos], o64["density"][pos]) <= 1e-6
    f64 = np.stack([o64["fx"], o64["fy"], o64["fz"]])
    f32 = np.stack([o32["fx"], o32["fy"], o32["fz"]])
    assert np.max(np.abs(f32 - f64)) <= 1e-6 * np.max(np.abs(f64))


def _upload_case(oracle_lib, change):
    from timothy_gb300 import session as S

    col = C.make_colony("clustered", 20000, 35, C.initial_radius("clustered", 20000))
    with S.Session(col.types, max_slots=col.n + 64, list_capacity=384) as s:
        cid = s.add_colony(col, precision="fp64", update="dt", dt=0.01, verlet=True)
        s.step(3)
        s.sync()
        pos = s.download(cid, ["x", "y", "z"])
        moved = C.Colony(pos["x"].copy(), pos["y"].copy(), pos["z"].copy(), col.size.copy(), col.young, col.ctype,
                         col.phase, col.types)
        change(moved)
        rb = s.stats(cid)["list_rebuilds"]
        s.upload(cid, moved)
        s.step(2)
        s.sync()
        out = s.download(cid, ["x", "y", "z", "density", "v", "mindist", "fx", "fy", "fz"])
        rebuilt = s.stats(cid)["list_rebuilds"] - rb
    ref = oracle_lib.run(moved, 2, which="oracle", update_mode=1, dt=0.01)
    check64(out, ref, "upload")
    return rebuilt


def test_upload_same_cells_keeps_lists(oracle_lib):
    assert _upload_case(oracle_lib, lambda c: None) == 0


def test_upload_far_move_rebuilds(oracle_lib):
    def move(c):
        c.x[123] += 0.3      # beyond half the skin (0.25)
    assert _upload_case(oracle_lib, move) == 1


def test_upload_size_change_rebuilds(oracle_lib):
    def grow(c):
        c.size[7] *= 1.05
    assert _upload_case(oracle_lib, grow) == 1


def test_upload_bad_cell_type_empties_colony():
    from timothy_gb300 import session as S

    col = C.make_colony("uniform", 2000, 36, C.initial_radius("uniform", 2000))
    with S.Session(col.types, max_slots=col.n + 64, list_capacity=384) as s:
        cid = s.add_colony(col, precision="fp64", update="dt", dt=0.01, verlet=True)
        s.step(1)
        bad = col.copy()
        bad.ctype[5] = 3
        with pytest.raises(S.TimothyError):
            s.upload(cid, bad)
        assert s.stats(cid)["n"] == 0
        s.step(1)
        s.sync()
        s.upload(cid, col)
        s.step(1)
        s.sync()
        assert s.stats(cid)["n"] == col.n


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_list_overflow_falls_back_to_search(oracle_lib, precision):
    """Lists too short for the densest cells: every step searches instead, with the same results."""
    from timothy_gb300 import session as S

    col = C.make_colony("clustered", 20000, 37, C.initial_radius("clustered", 20000))
    with S.Session(col.types, max_slots=col.n + 64, list_capacity=32) as s:
        cid = s.add_colony(col, precision=precision, update="dt", dt=0.01, verlet=True)
        s.step(4)
        s.sync()
        out = s.download(cid, ["x", "y", "z", "density", "v", "mindist", "fx", "fy", "fz"])
        st = s.stats(cid)
    assert st["list_rebuilds"] == 4
    ref = oracle_lib.run(col, 4, which="oracle", update_mode=1, dt=0.01)
    if precision == "fp64":
        check64(out, ref, "overflow")
    else:
        pos = ref.density > 0
        assert rel(out["density"][pos], ref.density[pos]) <= 1e-6
        f = np.stack([ref.fx, ref.fy, ref.fz])
        assert np.max(np.abs(np.stack([out["fx"], out["fy"], out["fz"]]) - f)) <= 1e-6 * np.max(np.abs(f))


@pytest.mark.parametrize("kind,n,seed,dim", [("clustered", 40000, 38, 3), ("uniform", 30000, 39, 3),
                                              ("uniform", 20000, 40, 2)])
def test_fp32_lists_walk_skip_keeps_v(kind, n, seed, dim):
    """The list pass settles v = 0 without the octree walk when a list entry
    inside the query box precedes the first within-h neighbour in Morton
    order, and a cell without neighbours within h takes its mindist from its
    list when the nearest entry is a candidate within the list's sure radius.
    Diagnostics walk every cell; v and mindist must not change bit for bit,
    over steps with and without list rebuilds."""
    from timothy_gb300 import session as S

    col = C.make_colony(kind, n, seed, C.initial_radius(kind, n, dim=dim), dim=dim)
    fields = ["x", "y", "z", "density", "v", "mindist", "fx", "fy", "fz"]
    a, sa = S.run_colony(col, 6, precision="fp32c", update="dt", dt=0.01, verlet=True, fields=fields)
    b, sb = S.run_colony(col, 6, precision="fp32c", update="dt", dt=0.01, verlet=True, diagnostics=True,
                         fields=fields)
    for k in fields:
        assert np.array_equal(a[k], b[k]), k
    assert sb["walked_cells"] == col.n
    assert sa["walked_cells"] < sb["walked_cells"]
    assert sa["walked_isolated_cells"] <= sb["walked_isolated_cells"]
    assert 1 <= sa["list_rebuilds"] < 6


def test_fp32_lists_v_against_fp64_search(oracle_lib):
    """One step without diagnostics: v of the FP32 list path is within 1e-5
    of max |v| of the FP64 oracle's, and zero where the oracle's is, but for
    cells whose first neighbour barely touches them (the FP32 overlap test
    may round the other way there)."""
    from timothy_gb300 import session as S

    col = C.make_colony("clustered", 40000, 41, C.initial_radius("clustered", 40000))
    out, st = S.run_colony(col, 1, precision="fp32c", update="none", verlet=True, fields=["v"])
    ref = oracle_lib.run(col, 1, which="oracle", update_mode=0)
    vs = np.max(np.abs(ref.v))
    assert vs > 0.0
    assert np.max(np.abs(out["v"] - ref.v)) <= 1e-5 * vs
    flip = (out["v"] == 0.0) != (ref.v == 0.0)
    assert np.all(np.abs(ref.v[flip]) <= 1e-5 * vs)
    assert np.count_nonzero(ref.v) > 0 and np.count_nonzero(out["v"]) > 0
    assert st["walked_cells"] < col.n


@pytest.mark.parametrize("precision", ["fp32c", "fp64"])
def test_isolated_cells_mindist_from_lists(precision):
    """A sparse colony (about two neighbours within h per cell): many cells
    have none, and their mindist comes from the list when the nearest entry is
    a sure candidate of the walk.  Diagnostics walk every cell; mindist and v
    must not change bit for bit, and fewer isolated cells must walk."""
    from timothy_gb300 import session as S

    col = C.make_colony("uniform", 30000, 42, C.initial_radius("uniform", 30000, mean=2.0))
    fields = ["x", "y", "z", "density", "v", "mindist", "fx", "fy", "fz"]
    a, sa = S.run_colony(col, 4, precision=precision, update="dt", dt=0.01, verlet=True, fields=fields + ["nbcount"])
    b, sb = S.run_colony(col, 4, precision=precision, update="dt", dt=0.01, verlet=True, diagnostics=True,
                         fields=fields)
    for k in fields:
        assert np.array_equal(a[k], b[k]), k
    isolated = int(np.sum(a["nbcount"] == 0))
    assert isolated > 1000
    assert sb["walked_isolated_cells"] == isolated
    assert sa["walked_isolated_cells"] < isolated
