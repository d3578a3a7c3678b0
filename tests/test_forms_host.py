"""Host logic of the batched and serving forms (no GPU)."""
import math

import numpy as np

from timothy_gb300 import autotune as AT
from timothy_gb300 import batch as B
from timothy_gb300 import colonies as C
from timothy_gb300 import serving as SV


def test_poisson_requests_follow_the_spec():
    reqs = SV.poisson_requests(200.0, 20.0, seed=7)
    assert abs(len(reqs) / 20.0 - 200.0) < 200.0 * 0.1
    n = np.array([r.n for r in reqs])
    assert n.min() >= 1000 and n.max() <= 1_000_000
    # log-uniform: the median is near sqrt(1e3 * 1e6)
    assert abs(math.log(np.median(n)) - 0.5 * math.log(1e9)) < 0.3
    assert set(r.steps for r in reqs) == {10, 50, 200}
    assert all(a.arrival < b.arrival for a, b in zip(reqs, reqs[1:]))
    kinds = [r.kind for r in reqs]
    assert 0.4 < kinds.count("clustered") / len(kinds) < 0.6


def test_request_source_keeps_density():
    src = SV.RequestSource(n_template=40_000, seed=3)
    for kind in ("uniform", "clustered"):
        col = src.colony(kind, 5000, 11)
        ref = C.make_colony(kind, 5000, 11, C.initial_radius(kind, 5000))
        got = C.count_neighbours_cpu(col).mean()
        want = C.count_neighbours_cpu(ref).mean()
        assert abs(got - want) < 0.08 * want, (kind, got, want)
        assert col.n == 5000
    a = src.colony("uniform", 1000, 1)
    b = src.colony("uniform", 1000, 2)
    assert not np.array_equal(a.x, b.x)


def test_request_source_into_staging_matches_allocation():
    """Cells cut into caller-provided (page-locked) position arrays are the
    same values as the allocating path; the other fields are template views."""
    src = SV.RequestSource(n_template=40_000, seed=3)
    stage = [np.full(9000, np.nan) for _ in range(3)]
    for kind, n, seed in (("uniform", 5000, 11), ("clustered", 8000, 12)):
        a = src.colony(kind, n, seed)
        b = src.colony(kind, n, seed, stage)
        for k in ("x", "y", "z", "size", "young", "ctype", "phase"):
            assert np.array_equal(getattr(a, k), getattr(b, k)), (kind, k)
        assert np.shares_memory(b.x, stage[0]) and np.shares_memory(b.z, stage[2])
        assert any(np.shares_memory(b.size, t) for t in src.template_arrays())
        assert b.n == n and a.radius == b.radius


def test_make_batch_sizes_kinds_seeds():
    cols = B.make_batch(40, seed=4, lo=1000, hi=20_000)
    n = np.array([c.n for c in cols])
    assert n.min() >= 1000 and n.max() <= 20_000
    assert [c.seed for c in cols] == list(range(1000, 1040))
    assert {c.kind for c in cols} == {"uniform", "clustered"}
    again = B.make_batch(40, seed=4, lo=1000, hi=20_000)
    assert all(np.array_equal(a.x, b.x) for a, b in zip(cols, again))


def test_bins_needed_follows_bin_level_rule():
    col = C.make_colony("uniform", 2000, 1, C.initial_radius("uniform", 2000))
    ext = max(np.ptp(col.x), np.ptp(col.y), np.ptp(col.z)) + 2 * (2.5 + 0.01)
    L = int(math.floor(math.log2(2 * ext / 2.5)))
    assert B.bins_needed(col) == 8 ** L + 2
    # bins of at least h/2 at this extent
    assert ext / 2 ** L >= 1.25


def test_session_bytes_scale_with_slots():
    from timothy_gb300 import session as S

    a = S.session_bytes(max_slots=1 << 20, list_capacity=384, max_bin_entries=1 << 20)
    b = S.session_bytes(max_slots=1 << 21, list_capacity=384, max_bin_entries=1 << 20)
    per_slot = (b - a) / (1 << 20)
    # state, scratch, outputs and 384 list entries of 4 bytes
    assert 384 * 4 < per_slot < 384 * 4 + 600


def test_tuning_cache_roundtrip(tmp_path):
    p = str(tmp_path / "tune.json")
    cols = B.make_batch(4, seed=1, lo=1000, hi=2000)
    key = AT.signature("GB300", cols)
    assert AT.load_cached(p, key) is None
    AT.store_cached(p, key, {"list_variant": 3})
    assert AT.load_cached(p, key) == {"list_variant": 3}
    assert "colonies~2^2" in key
