"""GPU parity of the plain FP64 path and the FP32-compensated path.

Checked against the reference's own outputs (tests/golden) and against the CPU
oracle run on the same inputs.  Tolerances follow the path's contract:
neighbour sets bit-exact; density, mindist, v, positions within 1e-12
relative; forces within 1e-12 of max |F| (per-element relative error is
ill-conditioned under the cancellation of the force sum); the FP32 path within
1e-6 on density and force.
"""
import glob
import os

import numpy as np
import pytest

from timothy_gb300 import colonies as C

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
               if not os.path.basename(p).startswith(("field_", "chain_")))
UPDATE = {0: "reference", 1: "dt", 2: "none"}

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from timothy_gb300 import session

    session.load_library()
    if session.device_count() < 1:
        pytest.fail("no CUDA device visible")
    return session


def load_case(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    t = C.CellTypes(d["th"], d["th2"], d["th3"], d["th4"], d["tsize"], d["trandommove"])
    col = C.Colony(d["x"], d["y"], d["z"], d["size"], d["young"], d["ctype"], d["phase"], t, int(d["dim"]))
    return d, col


def golden_grid(d, tag="strict"):
    shape = tuple(int(s) for s in d[f"{tag}_grid_shape"])
    g = np.zeros(shape)
    idx = d[f"{tag}_grid_idx"]
    if len(idx):
        g[idx[:, 0], idx[:, 1], idx[:, 2]] = d[f"{tag}_grid_val"]
    return g


def rel(a, b, floor=1e-300):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if a.size == 0:
        return 0.0
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor)))


def assert_fp64_close(out, ref, n, what=""):
    for k in ("x", "y", "z"):
        assert rel(out[k], ref[k], 1.0) <= 1e-12, (what, k, rel(out[k], ref[k], 1.0))
    assert rel(out["density"], ref["density"]) <= 1e-12, (what, "density")
    md_ref = ref["mindist"]
    assert np.array_equal(out["mindist"] > 1e300, md_ref > 1e300), (what, "mindist DBL_MAX pattern")
    fin = md_ref < 1e300
    assert rel(out["mindist"][fin], md_ref[fin]) <= 1e-12, (what, "mindist")
    vscale = max(np.max(np.abs(ref["v"]), initial=0.0), 1e-300)
    assert np.max(np.abs(out["v"] - ref["v"]), initial=0.0) <= 1e-12 * vscale, (what, "v")
    fscale = max(np.max(np.abs(np.concatenate([ref["fx"], ref["fy"], ref["fz"]])), initial=0.0), 1e-300)
    for k in ("fx", "fy", "fz"):
        assert np.max(np.abs(out[k] - ref[k]), initial=0.0) <= 1e-12 * fscale, (what, k)
    assert np.array_equal(out["removecell"], ref["removecell"]), (what, "removecell")


@pytest.mark.parametrize("name", CASES)
def test_fp64_matches_reference_golden(gpu, name):
    d, col = load_case(name)
    out, st = gpu.run_colony(col, int(d["steps"]), precision="fp64", update=UPDATE[int(d["update_mode"])],
                             dt=float(d["dt"]), cic=bool(d["cic"]), gfh=float(d["gfh"]))
    ref = {k: d[f"strict_{k}"] for k in ("x", "y", "z", "density", "v", "mindist", "fx", "fy", "fz", "removecell")}
    assert_fp64_close(out, ref, col.n, name)
    assert st["removecount"] == int(d["strict_removecount"])
    if col.n > 0:
        assert st["octsize"] == int(d["strict_octsize"]), (st["octsize"], int(d["strict_octsize"]))
        assert rel(st["aff"], d["strict_aff"], 1.0) <= 1e-13
    if int(d["cic"]):
        g = golden_grid(d)
        scale = max(np.max(np.abs(g)), 1e-300)
        assert out["grid"].shape == g.shape
        assert np.max(np.abs(out["grid"] - g)) <= 1e-12 * scale


@pytest.mark.parametrize("name", CASES)
def test_fp64_one_step_neighbour_sets_exact(gpu, oracle_lib, name):
    """Same inputs on both sides: neighbour sets, v's candidate and octree size are exact."""
    d, col = load_case(name)
    out, st = gpu.run_colony(col, 1, precision="fp64", update="none", diagnostics=True)
    nb = oracle_lib.neighbours(col)
    if col.n > 1:
        assert np.array_equal(out["nbcount"], nb.count)
        assert np.array_equal(out["nbhash"], nb.hash)
        assert np.array_equal(out["vcand"], nb.vcand)
    ref = oracle_lib.run(col, 1, which="oracle", update_mode=2)
    # identical inputs: the density differs from the oracle only by summation order
    assert rel(out["density"], ref.density) <= 1e-14
    assert np.array_equal(out["mindist"], ref.mindist)
    assert np.array_equal(out["v"], ref.v)
    if col.n > 0:
        assert st["octsize"] == ref.octsize
        assert np.array_equal(st["aff"], ref.aff)


@pytest.mark.parametrize("kind,n,seed", [("uniform", 20000, 11), ("clustered", 30000, 12)])
def test_fp32_path_against_fp64(gpu, kind, n, seed):
    col = C.make_colony(kind, n, seed, C.initial_radius(kind, n))
    o64, _ = gpu.run_colony(col, 1, precision="fp64", update="none", diagnostics=True)
    o32, _ = gpu.run_colony(col, 1, precision="fp32c", update="none", diagnostics=True)
    assert np.array_equal(o32["nbcount"], o64["nbcount"])
    assert np.array_equal(o32["nbhash"], o64["nbhash"])
    assert np.array_equal(o32["vcand"], o64["vcand"])
    pos = o64["density"] > 0
    assert rel(o32["density"][pos], o64["density"][pos]) <= 1e-6
    f64 = np.stack([o64["fx"], o64["fy"], o64["fz"]])
    f32 = np.stack([o32["fx"], o32["fy"], o32["fz"]])
    assert np.max(np.abs(f32 - f64)) <= 1e-6 * np.max(np.abs(f64))
    fin = o64["mindist"] < 1e300
    assert rel(o32["mindist"][fin], o64["mindist"][fin]) <= 1e-6


def test_fp64_multistep_against_oracle(gpu, oracle_lib):
    col = C.make_colony("clustered", 50000, 21, C.initial_radius("clustered", 50000))
    out, st = gpu.run_colony(col, 5, precision="fp64", update="dt", dt=0.01, cic=True)
    ref = oracle_lib.run(col, 5, which="oracle", update_mode=1, dt=0.01, cic=True)
    r = {k: getattr(ref, k) for k in ("x", "y", "z", "density", "v", "mindist", "fx", "fy", "fz", "removecell")}
    assert_fp64_close(out, r, col.n, "clustered50k")
    assert st["octsize"] == ref.octsize
    scale = np.max(np.abs(ref.grid))
    assert np.max(np.abs(out["grid"] - ref.grid)) <= 1e-12 * scale


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_dense_clump_big_bins_against_oracle(gpu, oracle_lib, precision):
    """A clump of 1500 cells inside a cube of side 0.3 h amid a uniform colony:
    its bins hold far more than 32 cells, so their Morton order comes from the
    per-block bitonic sort, which also places those cells.  Octree size and
    every output must match the oracle (the FP32 path's lists overflow there
    and the search pass serves the colony)."""
    base = C.make_colony("uniform", 6000, 51, C.initial_radius("uniform", 6000))
    rng = np.random.Generator(np.random.PCG64(52))
    k = 1500
    clump = rng.uniform(-0.15, 0.15, size=(k, 3)) * C.H_DEFAULT
    col = C.Colony(np.concatenate([base.x, clump[:, 0]]), np.concatenate([base.y, clump[:, 1]]),
                   np.concatenate([base.z, clump[:, 2]]), np.concatenate([base.size, base.size[:k]]),
                   np.concatenate([base.young, base.young[:k]]), np.concatenate([base.ctype, base.ctype[:k]]),
                   np.concatenate([base.phase, base.phase[:k]]), base.types)
    steps = 2 if precision == "fp64" else 1
    out, st = gpu.run_colony(col, steps, precision=precision, update="dt", dt=0.01, verlet=True, list_capacity=384)
    ref = oracle_lib.run(col, steps, which="oracle", update_mode=1, dt=0.01)
    assert st["device_errors"] == 0
    assert st["octsize"] == ref.octsize
    r = {k2: getattr(ref, k2) for k2 in ("x", "y", "z", "density", "v", "mindist", "fx", "fy", "fz", "removecell")}
    if precision == "fp64":
        assert_fp64_close(out, r, col.n, "clump")
    else:
        pos = ref.density > 0
        assert rel(out["density"][pos], ref.density[pos]) <= 1e-6
        f = np.stack([ref.fx, ref.fy, ref.fz])
        assert np.max(np.abs(np.stack([out["fx"], out["fy"], out["fz"]]) - f)) <= 1e-6 * np.max(np.abs(f))
