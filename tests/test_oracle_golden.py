"""Pin the CPU oracle to the reference's own outputs (tests/golden/*.npz).

The fixtures hold outputs of the reference's unmodified functions; the oracle
restatement must reproduce the strict build bit for bit and stay within the
reference's own fast-math spread of the shipped build.
"""
import glob
import os

import numpy as np
import pytest

from timothy_gb300 import colonies as C

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
               if not os.path.basename(p).startswith(("field_", "chain_")))


def load_case(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    t = C.CellTypes(d["th"], d["th2"], d["th3"], d["th4"], d["tsize"], d["trandommove"])
    col = C.Colony(d["x"], d["y"], d["z"], d["size"], d["young"], d["ctype"], d["phase"], t, int(d["dim"]))
    return d, col


def golden_grid(d, tag):
    shape = tuple(int(s) for s in d[f"{tag}_grid_shape"])
    g = np.zeros(shape)
    idx = d[f"{tag}_grid_idx"]
    if len(idx):
        g[idx[:, 0], idx[:, 1], idx[:, 2]] = d[f"{tag}_grid_val"]
    return g


def test_cases_present():
    assert len(CASES) >= 10


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_strict_bitwise(oracle_lib, name):
    d, col = load_case(name)
    r = oracle_lib.run(col, int(d["steps"]), which="oracle", update_mode=int(d["update_mode"]),
                       dt=float(d["dt"]), cic=bool(d["cic"]), gfh=float(d["gfh"]))
    for k in ("x", "y", "z", "density", "v", "mindist", "fx", "fy", "fz", "removecell"):
        assert np.array_equal(getattr(r, k), d[f"strict_{k}"]), k
    if col.n > 0:
        assert r.octsize == int(d["strict_octsize"])
        assert np.array_equal(r.aff, d["strict_aff"])
    assert r.removecount == int(d["strict_removecount"])
    if int(d["cic"]):
        assert np.array_equal(r.grid, golden_grid(d, "strict"))


@pytest.mark.parametrize("name", CASES)
def test_oracle_within_fast_math_spread(oracle_lib, name):
    """The shipped build uses -ffast-math; its outputs differ only in rounding."""
    d, col = load_case(name)
    r = oracle_lib.run(col, int(d["steps"]), which="oracle", update_mode=int(d["update_mode"]),
                       dt=float(d["dt"]), cic=bool(d["cic"]), gfh=float(d["gfh"]))
    if col.n == 0:
        return
    fmax = max(np.max(np.abs(d["fast_fx"])), np.max(np.abs(d["fast_fy"])), np.max(np.abs(d["fast_fz"])), 1e-300)
    for k in ("fx", "fy", "fz"):
        assert np.max(np.abs(getattr(r, k) - d[f"fast_{k}"])) <= 1e-9 * fmax, k
    for k in ("density", "mindist", "x", "y", "z"):
        ref = d[f"fast_{k}"]
        rel = np.abs(getattr(r, k) - ref) / np.maximum(np.abs(ref), 1e-300)
        assert np.max(rel, initial=0.0) <= 1e-9, k


# -- grid -> cell gather and field gradient ----------------------------------

def _field_colony(rec):
    from timothy_gb300 import colonies as C

    n = len(rec["x"])
    return C.Colony(rec["x"], rec["y"], rec["z"], np.full(n, 0.9), np.full(n, 2100.0, np.float32),
                    np.zeros(n, np.int32), rec["phase"], C.CellTypes.consistent(), int(rec["dim"]))


@pytest.mark.parametrize("name", ["field_env_clustered4k", "field_env_uniform2d", "field_env_coarse"])
def test_oracle_env2cells_matches_reference(oracle_lib, name):
    import sys

    sys.path.insert(0, GOLDEN)
    from fields import field, gradient_field

    rec = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    col = _field_colony(rec)
    gfh, nf = float(rec["gfh"]), int(rec["nfields"])
    dims = oracle_lib.grid_dims(col.dim, gfh)
    out = oracle_lib.env2cells(col, field(nf, dims), gradient_field(nf, dims), gfh=gfh, which="oracle")
    assert np.array_equal(out, rec["strict_cellenv"])
    scale = np.max(np.abs(rec["fast_cellenv"]))
    assert np.max(np.abs(out - rec["fast_cellenv"])) <= 1e-13 * scale


@pytest.mark.parametrize("name", ["field_grad_gfh32", "field_grad_gfh8", "field_grad_2d_gfh8"])
def test_oracle_fieldgradient_matches_reference(oracle_lib, name):
    import sys

    sys.path.insert(0, GOLDEN)
    from fields import field

    rec = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    dim, gfh, nf = int(rec["dim"]), float(rec["gfh"]), int(rec["nfields"])
    g = oracle_lib.fieldgradient(field(nf, tuple(rec["dims"])), dim=dim, gfh=gfh, which="oracle")
    comps = 3 if dim == 3 else 2          # a 2-D grid's z gradient reads outside the array in the reference
    sample = g[:, rec["ix"], rec["iy"], rec["iz"], :comps]
    for tag in ("strict", "fast"):
        assert np.array_equal(sample, rec[f"{tag}_sample"][..., :comps]), tag
        assert np.array_equal(g.reshape(nf, -1, 3).sum(axis=1)[:, :comps], rec[f"{tag}_sums"][:, :comps]), tag
    if dim == 2:
        assert not np.any(g[..., 2])


def test_oracle_vtk_matches_reference(oracle_lib, tmp_path):
    import hashlib

    rec = np.load(os.path.join(GOLDEN, "field_vtk_clustered3k.npz"))
    img = oracle_lib.write_vtk(str(tmp_path / "o.vtk"), rec["x"], rec["y"], rec["z"], rec["ctype"], rec["fx"],
                               rec["fy"], rec["fz"], which="oracle")
    assert len(img) == int(rec["nbytes"])
    assert hashlib.sha256(img).digest() == rec["sha256"].tobytes()


def test_cellsdeath_rule_matches_reference(oracle_lib):
    """The survivor order the session's compaction implements is the reference's cellsdeath."""
    if not oracle_lib.available("ref_strict"):
        pytest.skip("reference not built here")
    rng = np.random.default_rng(7)
    for n, oldlnc in ((200, 200), (200, 150), (1, 1), (60, 5), (30, 30)):
        rem = (rng.random(oldlnc) < 0.25).astype(np.uint8)
        assert np.array_equal(oracle_lib.survivors(n, oldlnc, rem), oracle_lib.ref_survivors(n, oldlnc, rem))


@pytest.mark.parametrize("name", ["field_cycle_3d", "field_cycle_2d"])
def test_oracle_cellcycle_matches_reference(oracle_lib, name):
    """updatecellcycles with mitosis: the restatement, fed the C library's
    rand() stream after the same srand(), reproduces the reference's cells."""
    import sys

    sys.path.insert(0, GOLDEN)
    from make_golden_fields import CYCLE_CL1, CYCLE_CL2, CYCLE_TYPES

    rec = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    st = {k[3:]: rec[k] for k in rec.files if k.startswith("in_")}
    out = oracle_lib.cellcycle(st, CYCLE_TYPES, dim=int(rec["dim"]), nfields=2, envvalue=rec["env"], cl1=CYCLE_CL1,
                               cl2=CYCLE_CL2, sps=3600.0, seed=int(rec["seed"]), removecell=rec["rem"],
                               which="oracle")
    for k in rec.files:
        if k.startswith("out_"):
            assert np.array_equal(np.asarray(out[k[4:]]), rec[k]), k


DIFFUSION = ["field_diffuse_3d_two", "field_diffuse_3d_stiff", "field_diffuse_2d", "field_diffuse_3d_step0"]


@pytest.mark.parametrize("name", DIFFUSION)
def test_oracle_diffusion_matches_reference(oracle_lib, name):
    """The implicit diffusion step (environment.c:131-523): solve count, z and
    the assembled operator exactly as the reference's own environment.c builds
    them (compiled on the Hypre stand-in); the right-hand side bit for bit
    when the step makes one solve (later solves start from a CG result); the
    solution within 1e-13 of the largest value (both solve to 1e-15)."""
    rec = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    gfh, sps, gfdt, step = float(rec["gfh"]), float(rec["sps"]), float(rec["gfdt"]), int(rec["step"])
    assert oracle_lib.diffusion_iters(sps, gfdt) == int(rec["iters"])
    assert int(rec["nsolves"]) == 2 * int(rec["iters"])
    assert float(rec["tol"]) == 1e-12 and int(rec["maxiter"]) == 50
    for f, dc in enumerate(rec["dc"]):
        z = oracle_lib.diffusion_z(float(dc), gfdt, gfh)
        assert z == rec["z"][f]
        assert rec["diag"][f] == 1 + 6.0 * z + rec["lam"][f] * float(np.float32(gfdt))
        assert rec["off"][f] == -z
    out = oracle_lib.diffuse(tuple(rec["gsize"]), gfh, sps, gfdt, step, rec["dc"], rec["bc"], rec["mean"],
                             rec["lam"])
    assert out["iters"] == int(rec["iters"])
    if int(rec["iters"]) == 1:
        assert np.array_equal(out["b"], rec["b"])
    else:
        assert np.max(np.abs(out["b"] - rec["b"])) <= 1e-14 * np.max(np.abs(rec["b"]))
    assert np.max(np.abs(out["u"] - rec["x"])) <= 1e-13 * np.max(np.abs(rec["x"]))


def test_oracle_diffusion_matches_live_reference(oracle_lib):
    """The same comparison against the reference's environment.c run here, with
    other parameters (one solve per step, so the right-hand side is exact)."""
    if not oracle_lib.available("ref_env"):
        pytest.skip("reference not built here")
    args = (3, 128.0, 7200.0, 7200.0, 3, [0.7, 30.0], [2.0, 0.0], [1.5, 0.25], [0.002, 0.0])
    r = oracle_lib.ref_environment(*args, ncalls=1)
    out = oracle_lib.diffuse(r["gsize"], *args[1:])
    assert out["iters"] == r["iters"] == 1
    assert np.array_equal(out["b"], r["b"])
    assert np.max(np.abs(out["u"] - r["x"])) <= 1e-13 * np.max(np.abs(r["x"]))

