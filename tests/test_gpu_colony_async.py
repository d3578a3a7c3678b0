"""Colonies added and removed without waiting, and fences.

tm_colony_add_async queues a colony behind the step in flight, and
tm_colony_remove no longer waits; a colony placed in the ranges a removed
colony freed, while that colony's last step may still run, must give the
same bits as the same colony alone.  tm_session_fence / tm_session_wait
bound how far the host runs ahead."""
import numpy as np
import pytest

from timothy_gb300 import colonies as C

pytestmark = pytest.mark.gpu
FIELDS = ["x", "y", "z", "density", "v", "mindist", "fx", "fy", "fz"]


def _alone(col, steps):
    from timothy_gb300.session import Session

    with Session(col.types, dim=3, max_slots=col.n + 64, list_capacity=384) as s:
        cid = s.add_colony(col, precision="fp32c", update="dt", dt=0.01, verlet=True)
        s.step(steps)
        s.sync()
        return s.download(cid, FIELDS)


def test_async_add_into_freed_ranges_matches_alone():
    from timothy_gb300.session import Session, host_register, host_unregister

    a = C.make_colony("clustered", 12_000, 71, C.initial_radius("clustered", 12_000))
    b = C.make_colony("uniform", 11_000, 72, C.initial_radius("uniform", 11_000))
    # room for one of them at a time: b must reuse a's slots
    with Session(a.types, dim=3, max_slots=12_000 + 64, max_colonies=2, list_capacity=384) as s:
        ca = s.add_colony(a, precision="fp32c", update="dt", dt=0.01, verlet=True, wait=False)
        s.step(3)
        out_a = {k: np.zeros(a.n) for k in FIELDS}
        for v in out_a.values():
            host_register(v)
        s.download_async(ca, FIELDS, out_a)
        s.remove_colony(ca)                        # queued behind the gathers
        f0 = s.fence()
        cb = s.add_colony(b, precision="fp32c", update="dt", dt=0.01, verlet=True, wait=False)
        s.step(4)
        f1 = s.fence()
        s.wait(f0)
        s.wait(f1)
        out_b = s.download(cb, FIELDS)
        s.sync()
        got_a = {k: v.copy() for k, v in out_a.items()}
        for v in out_a.values():
            host_unregister(v)
    want_a = _alone(a, 3)
    want_b = _alone(b, 4)
    for k in FIELDS:
        assert np.array_equal(got_a[k], want_a[k]), ("a", k)
        assert np.array_equal(out_b[k], want_b[k]), ("b", k)


def test_fence_ids_increase_and_wait_rejects_unknown():
    from timothy_gb300.session import Session, TimothyError

    col = C.make_colony("uniform", 2000, 73, C.initial_radius("uniform", 2000))
    with Session(col.types, dim=3, max_slots=col.n + 64) as s:
        s.add_colony(col, precision="fp64", update="dt", dt=0.01)
        fs = []
        for _ in range(70):                        # more fences than the ring holds
            s.step(1)
            fs.append(s.fence())
        assert fs == list(range(fs[0], fs[0] + 70))
        s.wait(fs[0])                              # older than the ring: covered by a newer record
        s.wait(fs[-1])
        with pytest.raises(TimothyError):
            s.wait(fs[-1] + 5)
