"""Batched and serving forms: many colonies in one session give, per colony,
exactly what the colony gives alone."""
import numpy as np
import pytest

from timothy_gb300 import colonies as C

pytestmark = pytest.mark.gpu

FIELDS = ["x", "y", "z", "density", "v", "mindist", "fx", "fy", "fz"]


def mixed_colonies(count, seed, lo=300, hi=8000):
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for i in range(count):
        n = int(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        kind = "clustered" if i % 2 else "uniform"
        out.append(C.make_colony(kind, n, seed * 100 + i, C.initial_radius(kind, n)))
    return out


def alone(col, steps, precision, list_capacity=384, tuning=None):
    from timothy_gb300 import session as S

    with S.Session(col.types, max_slots=col.n + 64, list_capacity=list_capacity) as s:
        if tuning:
            s.set_tuning(**tuning)
        cid = s.add_colony(col, precision=precision, update="dt", dt=0.01, verlet=True)
        s.step(steps)
        s.sync()
        return s.download(cid, FIELDS)


def assert_same(a, b, tag):
    for k in FIELDS:
        assert np.array_equal(a[k], b[k]), (tag, k, float(np.max(np.abs(a[k] - b[k]))))


def test_batch_alone_vs_mixed_bitwise():
    from timothy_gb300 import batch as B

    cols = mixed_colonies(10, 41)
    precs = ["fp32c" if i % 3 else "fp64" for i in range(len(cols))]
    with B.open_session(cols) as s:
        ids = [s.add_colony(c, precision=p, update="dt", dt=0.01, verlet=True) for c, p in zip(cols, precs)]
        s.use_graph(True)
        s.step(8)
        s.sync()
        mixed = [s.download(cid, FIELDS) for cid in ids]
    for i, (c, p) in enumerate(zip(cols, precs)):
        assert_same(mixed[i], alone(c, 8, p), f"colony {i} ({p}, n={c.n})")


def test_batch_tuned_fp64_matches_oracle(oracle_lib):
    from timothy_gb300 import batch as B

    cols = mixed_colonies(6, 42, 500, 4000)
    info = B.run_batch(cols, 5, precision="fp64", warmup=0, tune=True, fields=["x", "y", "z", "density", "fx",
                                                                                "fy", "fz"])
    assert info["tuning"]["list_variant"] in (1, 2, 3, 4)
    assert info["gpu_launches"] > 0
    for c, out in zip(cols, info["results"]):
        ref = oracle_lib.run(c, 5, which="oracle", update_mode=1, dt=0.01)
        assert np.max(np.abs(out["density"] - ref.density) / ref.density) <= 1e-12
        fs = np.max(np.abs(np.stack([ref.fx, ref.fy, ref.fz])))
        for k in ("fx", "fy", "fz"):
            assert np.max(np.abs(out[k] - getattr(ref, k))) <= 1e-12 * fs
        for k in ("x", "y", "z"):
            assert np.max(np.abs(out[k] - getattr(ref, k)) / np.maximum(np.abs(getattr(ref, k)), 1.0)) <= 1e-12


def test_tuning_changes_shapes_not_results():
    """Block shapes leave every bit unchanged; the search level reorders the
    lists, so FP32 sums round differently (within the FP32 path's 1e-6)."""
    from timothy_gb300 import session as S

    col = C.make_colony("clustered", 6000, 43, C.initial_radius("clustered", 6000))
    base = alone(col, 6, "fp32c")
    for tuning in ({"list_variant": 2, "walk_block": 64}, {"list_variant": 4, "walk_block": 256},
                   {"list_variant": 3}):
        assert_same(alone(col, 6, "fp32c", tuning=tuning), base, str(tuning))
    other = alone(col, 6, "fp32c", tuning={"pair_lshift": 0})
    pos = base["density"] > 0
    assert np.max(np.abs(other["density"][pos] - base["density"][pos]) / base["density"][pos]) <= 1e-6
    f = np.stack([base["fx"], base["fy"], base["fz"]])
    g = np.stack([other["fx"], other["fy"], other["fz"]])
    assert np.max(np.abs(f - g)) <= 1e-6 * np.max(np.abs(f))
    with S.Session(col.types, max_slots=col.n + 64, list_capacity=384) as s:
        with pytest.raises(S.TimothyError):
            s.set_tuning(list_variant=7)
        assert s.tuning["list_variant"] == 1


def test_serving_alone_vs_mixed_bitwise():
    from timothy_gb300 import serving as SV

    cols = mixed_colonies(8, 44, 400, 6000)
    steps = [3, 7, 5, 2, 9, 4, 6, 3]
    reqs = [SV.Request(i, c.kind, c.n, k, arrival=float(i // 3), colony=c) for i, (c, k) in enumerate(zip(cols,
                                                                                                           steps))]
    # a pool with room for the two largest colonies: bursts must wait for room
    room = sorted(((c.n + 31) // 32) * 32 for c in cols)[-2:]
    with SV.Server(max_slots=sum(room) + 64, max_colonies=8, keep_results=True, fields=FIELDS) as srv:
        stats = srv.run(reqs, virtual=True)
    assert stats["finished"] == len(reqs)
    assert any(r.admitted > r.arrival for r in reqs)          # some waited for room
    for r, c, k in zip(reqs, cols, steps):
        assert_same(r.result, alone(c, k, "fp32c"), f"request {r.rid}")


def test_serving_realtime_reports_latency():
    from timothy_gb300 import serving as SV

    src = SV.RequestSource(n_template=50_000, seed=7)
    reqs = SV.poisson_requests(50.0, 1.0, seed=7, lo=1000, hi=50_000, steps=(5, 10))
    with SV.Server(max_slots=400_000, max_colonies=256) as srv:
        stats = srv.run(reqs, source=src)
    assert stats["finished"] == len(reqs) > 10
    assert 0 < stats["p50"] <= stats["p99"]
    assert stats["throughput"] > 0


def test_serving_from_source_matches_alone():
    """Requests cut from a source into page-locked staging (reused once their
    upload is done): every request's result equals the same colony alone."""
    import numpy as np

    from timothy_gb300 import serving as SV

    src = SV.RequestSource(n_template=60_000, seed=9)
    reqs = SV.poisson_requests(400.0, 0.05, seed=9, lo=2000, hi=40_000, steps=(3, 6))
    assert len(reqs) >= 8
    with SV.Server(max_slots=150_000, max_colonies=64, fields=("x", "y", "z", "density", "fx", "fy", "fz")) as srv:
        stats = srv.run(reqs, source=src, virtual=True)
    assert stats["finished"] == len(reqs)
    for r in reqs:
        want = SV.run_alone(src.colony(r.kind, r.n, r.seed), r.steps)
        assert r.result["density_sum"] == float(np.sum(want["density"])), r.rid
