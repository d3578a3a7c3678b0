"""Cell cycle of a resident colony (updatecellcycles with mitosis) against the
oracle restatement, which is pinned to the reference's own function: with
the C library's rand() stream after the same srand(), every cell, daughter
and removal mark matches bit for bit."""
import ctypes
import os
import sys

import numpy as np
import pytest

from timothy_gb300 import colonies as C

pytestmark = pytest.mark.gpu
sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))

TYPES = dict(g1=np.array([11.0, 9.0], np.float32), s=np.array([8.0, 7.0], np.float32),
             g2=np.array([4.0, 3.0], np.float32), m=np.array([1.0, 1.5], np.float32),
             v=np.array([0.2, 0.1], np.float32), rd=np.array([0.1, 0.3], np.float32),
             cd=np.array([6.0, 7.0], np.float32))
CL1 = np.array([0.3, 0.2, 0.25, 0.1], np.float32)
CL2 = np.array([0.1, 0.05, 0.1, 0.02], np.float32)


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def srand(seed):
    libc = ctypes.CDLL(None)
    libc.srand.argtypes = [ctypes.c_uint]
    libc.srand(seed)


@pytest.mark.parametrize("dim,seed", [(3, 31), (2, 32)])
def test_cellcycle_matches_oracle(oracle_lib, dim, seed):
    torch = _torch()
    from timothy_gb300 import session as S

    types = C.CellTypes.consistent(h=(2.5, 2.5), size=(1.0, 0.9))
    n = 4000
    col = C.make_colony("uniform", n, seed, C.initial_radius("uniform", n, dim=dim), dim=dim, types=types)
    rng = np.random.default_rng(seed)
    cyc = dict(phasetime=rng.uniform(0, 12, n).astype(np.float32), g1=rng.uniform(8, 12, n).astype(np.float32),
               s=rng.uniform(6, 9, n).astype(np.float32), g2=rng.uniform(2, 5, n).astype(np.float32),
               m=rng.uniform(0.5, 2, n).astype(np.float32), age=rng.integers(0, 5, n).astype(np.int32))
    col.phase[:] = rng.integers(0, 6, n)
    env = rng.uniform(0, 1, (2, n))
    cellenv = np.zeros((2, n, 4))
    cellenv[:, :, 0] = env
    tsize = np.array([1.0, 0.9])
    with S.Session(types, dim=dim, max_slots=2 * n + 64, list_capacity=384) as s:
        cid = s.add_colony(col, precision="fp64", update="none", verlet=True, reserve=2 * n)
        s.step(1)                                   # densities of this configuration
        s.sync()
        s.set_cycle(cid, cyc["phasetime"], cyc["g1"], cyc["s"], cyc["g2"], cyc["m"], cyc["age"])
        pos = s.download(cid, ["x", "y", "z", "density", "removecell"])
        before = s.get_cycle(cid)
        srand(seed)
        divided, marked = s.cellcycle(cid, TYPES, nfields=2, cl1=CL1, cl2=CL2,
                                      cellenv=torch.from_numpy(cellenv).cuda())
        after = s.get_cycle(cid)
        out = s.download(cid, ["x", "y", "z", "density", "removecell"])
        removed = s.compact(cid)
        kept = s.get_cycle(cid)
    state = dict(phase=before["phase"], phasetime=cyc["phasetime"], g1=cyc["g1"], s=cyc["s"], g2=cyc["g2"],
                 m=cyc["m"], age=cyc["age"], size=before["size"], young=before["young"], x=pos["x"], y=pos["y"],
                 z=pos["z"], density=pos["density"], ctype=col.ctype)
    ref = oracle_lib.cellcycle(state, dict(TYPES, size=tsize), dim=dim, nfields=2, envvalue=env.ravel(), cl1=CL1,
                               cl2=CL2, sps=3600.0, seed=seed, removecell=pos["removecell"], which="oracle")
    m = len(ref["phase"])
    assert divided == m - n > 0 and marked == ref["removecount"] > 0
    for k in ("phasetime", "g1", "s", "g2", "m", "age", "phase", "size", "young"):
        assert np.array_equal(after[k], ref[k]), k
    for k in ("x", "y", "z", "density"):
        assert np.array_equal(out[k], ref[k]), k
    assert np.array_equal(out["removecell"], ref["removecell"])
    # the marked cells leave in the reference's survivor order
    keep = oracle_lib.survivors(m, m, ref["removecell"])
    assert removed == marked
    for k in ("phase", "g1", "age", "size"):
        assert np.array_equal(kept[k], ref[k][keep]), k


def _cycle_run(types, col, cyc, env, stream_seed=None, libc_seed=None, calls=2):
    """Cell-cycle steps of one colony; the draws from the C library after
    srand(libc_seed), or from the device stream of stream_seed."""
    torch = _torch()
    from timothy_gb300 import session as S

    n = col.n
    cellenv = np.zeros((2, n, 4))
    cellenv[:, :, 0] = env
    outs = []
    stream = S.RandStream(stream_seed) if stream_seed is not None else None
    with S.Session(types, dim=col.dim, max_slots=4 * n + 64, list_capacity=384) as s:
        cid = s.add_colony(col, precision="fp64", update="none", verlet=True, reserve=4 * n)
        s.step(1)
        s.sync()
        s.set_cycle(cid, cyc["phasetime"], cyc["g1"], cyc["s"], cyc["g2"], cyc["m"], cyc["age"])
        if libc_seed is not None:
            srand(libc_seed)
        for _ in range(calls):
            m = s._n[cid]
            env_m = torch.from_numpy(np.ascontiguousarray(np.resize(cellenv, (2, m, 4)))).cuda()
            res = s.cellcycle(cid, TYPES, nfields=2, cl1=CL1, cl2=CL2, cellenv=env_m, stream=stream)
            outs.append((res, s.get_cycle(cid), s.download(cid, ["x", "y", "z", "removecell"])))
    return outs, stream


def test_device_rand_stream_matches_libc():
    """tm_cycle_params.rand_seeded: the values of the C library's stream after
    srand(seed), generated on the device, give the same cells bit for bit as
    the library's own rand() calls, over consecutive steps; the stream's
    offset then points where the library's next rand() would be."""
    types = C.CellTypes.consistent(h=(2.5, 2.5), size=(1.0, 0.9))
    n, seed = 6000, 77
    col = C.make_colony("uniform", n, seed, C.initial_radius("uniform", n), types=types)
    rng = np.random.default_rng(seed)
    cyc = dict(phasetime=rng.uniform(0, 12, n).astype(np.float32), g1=rng.uniform(8, 12, n).astype(np.float32),
               s=rng.uniform(6, 9, n).astype(np.float32), g2=rng.uniform(2, 5, n).astype(np.float32),
               m=rng.uniform(0.5, 2, n).astype(np.float32), age=rng.integers(0, 5, n).astype(np.int32))
    col.phase[:] = rng.integers(0, 6, n)
    env = rng.uniform(0, 1, (2, n))
    a, _ = _cycle_run(types, col, cyc, env, libc_seed=seed, calls=3)
    libc = ctypes.CDLL(None)
    libc.rand.restype = ctypes.c_int
    next_libc = libc.rand()
    b, stream = _cycle_run(types, col, cyc, env, stream_seed=seed, calls=3)
    for (ra, ca, oa), (rb, cb, ob) in zip(a, b):
        assert ra == rb
        for k in ca:
            assert np.array_equal(ca[k], cb[k]), k
        for k in oa:
            assert np.array_equal(oa[k], ob[k]), k
    lib = ctypes.CDLL(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "timothy_gb300",
                                   "libtimothy_gb300.so"))
    lib.tmi_libc_rand_host.argtypes = [ctypes.c_uint32, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p]
    nxt = np.zeros(1, np.int32)
    lib.tmi_libc_rand_host(seed, stream.offset, 1, nxt.ctypes.data)
    assert int(nxt[0]) == next_libc
    assert sum(r[0][0] for r in b) > 0                     # divisions happened
