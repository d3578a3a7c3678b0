"""The whole cell update of the reference (cellsupdate, cells.c:525-543)
through the drop-ins, against the reference's own step loop.

Each fixture (tests/golden/chain_*.npz, made by make_golden_fields.py --chain
from the reference compiled unmodified) holds a colony's celldata_t records,
the cell types' cycle parameters and a seed; the reference ran octbuild,
computepotential, computegradient and cellsupdate (random move with
randommove != 0, cell cycle with mitosis and death, removal) for a few steps
after srand(seed).  Here the same loop runs over the drop-ins with the C
library's generator seeded the same way: the rand() stream, the records (in
order, daughters and removals included) and the counters must come out as
the reference's.
"""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import bindings as B
from timothy_gb300 import colonies as CO

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CHAINS = ["chain_clustered3d", "chain_uniform2d"]
EXACT = ("lifetime", "phase", "age", "death", "phasetime", "g1", "s", "g2", "m", "young", "gid", "ctype", "size")


def load_chain(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    types = CO.CellTypes.consistent(h=d["h"], size=d["tsize"], randommove=d["randommove"])
    n = int(d["n"])
    col = CO.Colony(d["in_x"], d["in_y"], d["in_z"], d["in_size"], d["in_young"], d["in_ctype"], d["in_phase"],
                    types, int(d["dim"]))
    cyc = {k: d["cy_" + k] for k in ("g1", "s", "g2", "m", "v", "rd", "cd")}
    return d, n, col, cyc


def test_chain_fixture_counters():
    """The reference's localcount follows the records' phases; its per-type
    phase counters move only at mitosis and removal (cells.c:198-202, 306-334)."""
    for name in CHAINS:
        d, n, _, _ = load_chain(name)
        out_n = len(d["out_phase"])
        pc = B.phase_counts(d["out_phase"], d["out_ctype"], 1)
        assert np.array_equal(pc[:7], d["counts_out"][:7])
        assert int(d["counts_out"][7]) == out_n
        # a daughter's gid is its index at birth (cells.c:178-180): after a
        # removal the index comes round again, so gids need not be unique
        assert np.max(d["out_gid"]) < int(d["cap"])
        assert out_n != n


@pytest.mark.gpu
@pytest.mark.parametrize("name", CHAINS)
def test_cellsupdate_chain_matches_reference(name):
    from timothy_gb300.refabi import DropinRun

    d, n, col, cyc = load_chain(name)
    libc = C.CDLL(None)
    libc.srand.argtypes = [C.c_uint]
    with DropinRun(col, cap=int(d["cap"]), cycle=cyc, sps=float(d["sps"])) as run:
        for k in B.REF_CELL_DTYPE.names:
            run.cells[k][:n] = d["in_" + k]
        run.set_counts(d["counts_in"])
        libc.srand(int(d["seed"]))
        for _ in range(int(d["steps"])):
            run.cycle_step()
        out = run.cells[:run.n].copy()
        counts = run.counts()
    assert run.n == len(d["out_phase"])
    assert np.array_equal(counts, d["counts_out"])
    for k in EXACT:
        assert np.array_equal(out[k], d["out_" + k]), k
    for k in ("x", "y", "z"):
        assert np.max(np.abs(out[k] - d["out_" + k]) / np.maximum(np.abs(d["out_" + k]), 1.0)) <= 1e-12, k
    for k in ("density", "v"):
        ref = d["out_" + k]
        assert np.max(np.abs(out[k] - ref)) <= 1e-12 * max(np.max(np.abs(ref)), 1e-300), k
