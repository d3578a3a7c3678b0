"""Resident colonies that shrink and grow: death compaction (cellsdeath,
cells.c:290-336) and appends (mitosis daughters, cells.c:156-205), checked
against the oracle run on the same cells."""
import numpy as np
import pytest

from timothy_gb300 import colonies as C

pytestmark = pytest.mark.gpu

FIELDS = ["x", "y", "z", "density", "v", "mindist", "fx", "fy", "fz"]


def rel_ok(a, b, tol=1e-12):
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0)) <= tol


def check(out, ref, idx=None):
    for k in ("x", "y", "z", "density", "mindist"):
        r = getattr(ref, k) if idx is None else getattr(ref, k)[idx]
        fin = r < 1e300
        assert rel_ok(out[k][fin], r[fin]), k
    f = np.stack([getattr(ref, k) if idx is None else getattr(ref, k)[idx] for k in ("fx", "fy", "fz")])
    assert np.max(np.abs(np.stack([out[k] for k in ("fx", "fy", "fz")]) - f)) <= 1e-12 * max(np.max(np.abs(f)),
                                                                                               1e-300)


def edge_colony(n, seed, k):
    """A colony with k cells just inside the box edge: the first update marks them."""
    col = C.make_colony("uniform", n, seed, C.initial_radius("uniform", n))
    rng = np.random.default_rng(seed)
    pick = rng.choice(n, k, replace=False)
    col.x[pick] = 1023.5 - 3.0 * np.arange(k)[::-1] * 0    # all at x = 1023.5 (+ r reaches 1024)
    col.y[pick] = -900.0 + 5.0 * np.arange(k)              # far apart from each other
    return col, np.sort(pick)


def test_compaction_removes_marked_cells_in_order(oracle_lib):
    from timothy_gb300 import session as S

    col, pick = edge_colony(3000, 71, 12)
    ref1 = oracle_lib.run(col, 1, which="oracle", update_mode=1, dt=0.01)
    assert ref1.removecell.sum() == len(pick)
    with S.Session(col.types, max_slots=col.n + 64, list_capacity=384) as s:
        cid = s.add_colony(col, precision="fp64", update="dt", dt=0.01, verlet=True)
        s.step(1)
        s.sync()
        assert s.compact(cid) == len(pick)
        keep = oracle_lib.survivors(col.n, col.n, ref1.removecell)
        out = s.download(cid, FIELDS)
        assert len(out["x"]) == len(keep)
        check(out, ref1, keep)
        # the compacted colony keeps stepping like the reference on the surviving cells
        s.step(3)
        s.sync()
        out3 = s.download(cid, FIELDS)
        assert s.compact(cid) == 0
    moved = C.Colony(ref1.x[keep], ref1.y[keep], ref1.z[keep], col.size[keep], col.young[keep], col.ctype[keep],
                     col.phase[keep], col.types)
    check(out3, oracle_lib.run(moved, 3, which="oracle", update_mode=1, dt=0.01))


def test_append_grows_the_colony(oracle_lib):
    from timothy_gb300 import session as S

    col = C.make_colony("clustered", 2500, 72, C.initial_radius("clustered", 2500))
    extra = C.make_colony("clustered", 600, 73, C.initial_radius("clustered", 600))
    extra.x += 40.0                                        # a second lump beside the first
    with S.Session(col.types, max_slots=5000, list_capacity=384) as s:
        cid = s.add_colony(col, precision="fp32c", update="dt", dt=0.01, verlet=True, reserve=4000)
        s.step(2)
        s.sync()
        pos = s.download(cid, ["x", "y", "z"])
        s.append(cid, extra)
        s.step(2)
        s.sync()
        out = s.download(cid, FIELDS)
        with pytest.raises(S.TimothyError):
            s.append(cid, C.make_colony("uniform", 2000, 74, 20.0))    # beyond the reserve
    both = C.Colony(np.concatenate([pos["x"], extra.x]), np.concatenate([pos["y"], extra.y]),
                    np.concatenate([pos["z"], extra.z]), np.concatenate([col.size, extra.size]),
                    np.concatenate([col.young, extra.young]), np.concatenate([col.ctype, extra.ctype]),
                    np.concatenate([col.phase, extra.phase]), col.types)
    ref = oracle_lib.run(both, 2, which="oracle", update_mode=1, dt=0.01)
    pos_ok = ref.density > 0
    assert np.max(np.abs(out["density"][pos_ok] - ref.density[pos_ok]) / ref.density[pos_ok]) <= 1e-6
    f = np.stack([ref.fx, ref.fy, ref.fz])
    assert np.max(np.abs(np.stack([out["fx"], out["fy"], out["fz"]]) - f)) <= 1e-6 * np.max(np.abs(f))
    for k in ("x", "y", "z"):
        assert np.max(np.abs(out[k] - getattr(ref, k))) <= 1e-6


def test_single_cell_is_never_removed():
    from timothy_gb300 import session as S

    col = C.make_colony("uniform", 1, 75, 1.0)
    col.x[0] = 1023.5
    with S.Session(col.types, max_slots=64, list_capacity=384) as s:
        cid = s.add_colony(col, precision="fp64", update="dt", dt=0.01, verlet=True)
        s.step(1)
        s.sync()
        assert s.stats(cid)["removecount"] == 1
        assert s.compact(cid) == 0
        assert s.stats(cid)["n"] == 1
