"""ctypes bindings for the CPU oracle -- TEST INFRASTRUCTURE.

Loads either the plain-C restatement (oracle/liboracle.so, built from
tm_oracle.c) or the reference's own functions compiled from its sources
(oracle/_ref/libtimothy_ref.so, reference flags, or libtimothy_ref_strict.so).
Both export the same run signature (tm_oracle.h, ref_driver.c), so a caller
picks one by name.  Only tests, __graft_entry__.smoke() and bench.py's CPU legs
use this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBS = {
    "oracle": os.path.join(HERE, "liboracle.so"),
    "ref": os.path.join(HERE, "_ref", "libtimothy_ref.so"),
    "ref_strict": os.path.join(HERE, "_ref", "libtimothy_ref_strict.so"),
    "ref_env": os.path.join(HERE, "_ref", "libtimothy_ref_env.so"),
}

_P = C.c_void_p
_cache: dict[str, C.CDLL] = {}


def build(ref: bool | None = None, refsrc: str | None = None) -> None:
    """Compile the restatement; also the reference library when its sources
    are given (``refsrc`` or the TM_REFSRC environment variable: the
    reference's src/ directory).  ref=None builds it when they exist."""
    subprocess.run(["make", "-s", "-B", "-C", HERE, "liboracle.so"], check=True)
    refsrc = refsrc or os.environ.get("TM_REFSRC", "")
    have = bool(refsrc) and os.path.isfile(os.path.join(refsrc, "octree.c"))
    if ref is None:
        ref = have
    if ref:
        if not have:
            raise RuntimeError("building the reference needs its src/ directory: pass refsrc= or set TM_REFSRC")
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REFSRC={refsrc}"], check=True)


def available(which: str) -> bool:
    return os.path.exists(LIBS[which])


def load(which: str = "oracle") -> C.CDLL:
    if which in _cache:
        return _cache[which]
    path = LIBS[which]
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} is not built (oracle.bindings.build())")
    lib = C.CDLL(path)
    if which == "ref_env":
        lib.ref_environment.restype = C.c_int64
        lib.ref_environment.argtypes = [C.c_int, C.c_float, C.c_float, C.c_float, C.c_int, C.c_int] + [_P] * 4 + \
            [C.c_int, C.c_int64] + [_P] * 7
        _cache[which] = lib
        return lib
    fn = lib.tmo_run if which == "oracle" else lib.ref_run
    argt = [C.c_int64, C.c_int, C.c_int] + [_P] * 6 + [_P] * 7 + [C.c_int, C.c_int, C.c_double] + [_P] * 6 + \
        [_P, _P, _P, _P] + [C.c_int, C.c_float, _P, C.c_int64, _P, _P]
    if which == "oracle":
        argt = argt + [C.c_int]
        lib.tmo_env2cells.restype = C.c_int
        lib.tmo_env2cells.argtypes = [C.c_int64, C.c_int, _P, _P, _P, C.c_float, C.c_int, _P, _P, _P]
        lib.tmo_fieldgradient.restype = C.c_int
        lib.tmo_fieldgradient.argtypes = [C.c_int, C.c_float, C.c_int, _P, _P, _P]
        lib.tmo_write_vtk.restype = C.c_int
        lib.tmo_write_vtk.argtypes = [C.c_char_p, C.c_int64, _P, _P, _P, _P, _P, _P, _P, C.c_int]
        lib.tmo_cellcycle.restype = C.c_int
        lib.tmo_cellcycle.argtypes = [C.c_int64, C.c_int] + [_P] * 8 + [C.c_int, _P, _P, C.c_int, C.c_float, _P, _P,
                                                                         C.c_int64] + [_P] * 16 + [C.c_int64, _P, _P]
        lib.tmo_neighbours.restype = C.c_int
        lib.tmo_neighbours.argtypes = [C.c_int64, C.c_int, C.c_int, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P,
                                       C.c_int]
        lib.tmo_diffusion_iters.restype = C.c_int
        lib.tmo_diffusion_iters.argtypes = [C.c_float, C.c_float]
        lib.tmo_diffusion_z.restype = C.c_double
        lib.tmo_diffusion_z.argtypes = [C.c_double, C.c_float, C.c_float]
        lib.tmo_diffuse.restype = C.c_int
        lib.tmo_diffuse.argtypes = [C.c_int64, C.c_int64, C.c_int64, C.c_float, C.c_float, C.c_float, C.c_int,
                                    C.c_int] + [_P] * 6 + [C.c_double, _P, _P, _P, _P]
        lib.tm_mix64.restype = C.c_uint64
        lib.tm_mix64.argtypes = [C.c_uint64]
    else:
        lib.ref_sizeof.restype = C.c_int64
        lib.ref_sizeof.argtypes = [C.c_int]
        lib.ref_env2cells.restype = C.c_int64
        lib.ref_env2cells.argtypes = [C.c_int64, C.c_int, _P, _P, _P, _P, C.c_float, C.c_int, _P, _P, C.c_int64, _P]
        lib.ref_cellcycle.restype = C.c_int
        lib.ref_cellcycle.argtypes = [C.c_int64, C.c_int, C.c_int] + [_P] * 8 + [C.c_int, _P, _P, C.c_int, C.c_float,
                                                                                 C.c_uint, _P] + [_P] * 16 + \
            [C.c_int64, _P]
        lib.ref_cellsupdate_run.restype = C.c_int
        lib.ref_cellsupdate_run.argtypes = [_P, _P, C.c_int64, C.c_int, C.c_int] + [_P] * 13 + \
            [C.c_int, C.c_float, C.c_uint, C.c_int, _P]
        lib.ref_cellsdeath.restype = C.c_int64
        lib.ref_cellsdeath.argtypes = [C.c_int64, C.c_int64, _P, C.c_int64, C.c_int64, _P]
        lib.ref_write_vtk.restype = C.c_int
        lib.ref_write_vtk.argtypes = [C.c_char_p, C.c_int, C.c_int64, _P, _P, _P, _P, _P, _P, _P]
        lib.ref_fieldgradient.restype = C.c_int64
        lib.ref_fieldgradient.argtypes = [C.c_int, C.c_float, C.c_int, _P, C.c_int64, _P, _P]
    fn.restype = C.c_int
    fn.argtypes = argt
    _cache[which] = lib
    return lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


@dataclass
class RunResult:
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    density: np.ndarray
    v: np.ndarray
    mindist: np.ndarray
    fx: np.ndarray
    fy: np.ndarray
    fz: np.ndarray
    removecell: np.ndarray
    removecount: int
    octsize: int
    aff: np.ndarray
    grid: np.ndarray | None
    timing: np.ndarray


def run(col, nsteps: int = 1, *, which: str = "oracle", update_mode: int = 0, dt: float = 1.0,
        cic: bool = False, gfh: float = 8.0, nthreads: int = 0) -> RunResult:
    """Run the oracle (or the reference) on a copy of ``col``'s cells."""
    lib = load(which)
    n = col.n
    t = col.types
    x, y, z = col.x.copy(), col.y.copy(), col.z.copy()
    size = np.ascontiguousarray(col.size, np.float64)
    young = np.ascontiguousarray(col.young, np.float32)
    ctype = np.ascontiguousarray(col.ctype, np.int32)
    phase = np.ascontiguousarray(col.phase, np.int32)
    outs = {k: np.zeros(max(n, 1)) for k in ("density", "v", "mindist", "fx", "fy", "fz")}
    rem = np.zeros(max(n, 1), np.uint8)
    remc = np.zeros(1, np.int64)
    octsize = np.zeros(1, np.int64)
    aff = np.zeros(4)
    timing = np.zeros(5)
    gdims = np.zeros(3, np.int64)
    grid = None
    gcap = 0
    if cic:
        g = int((2049.0 + 1) / gfh) + 1
        gcap = g * g * (g if col.dim == 3 else 1)
        grid = np.zeros(gcap)
    th, th2, th3, th4 = (np.ascontiguousarray(a, np.float64) for a in (t.h, t.h2, t.h3, t.h4))
    tsize = np.ascontiguousarray(t.size, np.float64)
    trm = np.ascontiguousarray(t.randommove, np.float32)
    args = [n, col.dim, t.ntypes, _ptr(th), _ptr(th2), _ptr(th3), _ptr(th4), _ptr(tsize), _ptr(trm),
            _ptr(x), _ptr(y), _ptr(z), _ptr(size), _ptr(young), _ptr(ctype), _ptr(phase),
            nsteps, update_mode, dt,
            _ptr(outs["density"]), _ptr(outs["v"]), _ptr(outs["mindist"]),
            _ptr(outs["fx"]), _ptr(outs["fy"]), _ptr(outs["fz"]),
            _ptr(rem), _ptr(remc), _ptr(octsize), _ptr(aff),
            1 if cic else 0, gfh, _ptr(grid), gcap, _ptr(gdims), _ptr(timing)]
    if which == "oracle":
        rc = lib.tmo_run(*args, nthreads)
    else:
        rc = lib.ref_run(*args)
    if rc != 0:
        raise RuntimeError(f"{which} run failed with code {rc}")
    if cic:
        gx, gy, gz = (int(v) for v in gdims)
        grid = grid[:gx * gy * gz].reshape(gx, gy, gz)
    return RunResult(x, y, z, outs["density"][:n], outs["v"][:n], outs["mindist"][:n], outs["fx"][:n],
                     outs["fy"][:n], outs["fz"][:n], rem[:n], int(remc[0]), int(octsize[0]), aff, grid, timing)


@dataclass
class Neighbours:
    count: np.ndarray
    hash: np.ndarray
    vcand: np.ndarray
    ncand: np.ndarray
    offsets: np.ndarray | None
    lists: np.ndarray | None


def neighbours(col, *, lists: bool = False, nthreads: int = 0) -> Neighbours:
    """Per-cell neighbour-set diagnostics of one octree walk (tm_oracle.h)."""
    lib = load("oracle")
    n = col.n
    t = col.types
    th = np.ascontiguousarray(t.h, np.float64)
    cnt = np.zeros(max(n, 1), np.int32)
    hsh = np.zeros(max(n, 1), np.uint64)
    vc = np.zeros(max(n, 1), np.int64)
    nc = np.zeros(max(n, 1), np.int32)
    offs = np.zeros(n + 1, np.int64) if lists else None
    ctype = np.ascontiguousarray(col.ctype, np.int32)
    rc = lib.tmo_neighbours(n, col.dim, t.ntypes, _ptr(th), _ptr(col.x), _ptr(col.y), _ptr(col.z), _ptr(ctype),
                            _ptr(cnt), _ptr(hsh), _ptr(vc), _ptr(nc), _ptr(offs), None, nthreads)
    if rc != 0:
        raise RuntimeError(f"tmo_neighbours failed with code {rc}")
    lst = None
    if lists:
        lst = np.zeros(max(int(offs[n]), 1), np.int64)
        rc = lib.tmo_neighbours(n, col.dim, t.ntypes, _ptr(th), _ptr(col.x), _ptr(col.y), _ptr(col.z),
                                _ptr(ctype), None, None, None, None, _ptr(offs), _ptr(lst), nthreads)
        if rc != 0:
            raise RuntimeError(f"tmo_neighbours failed with code {rc}")
    return Neighbours(cnt[:n], hsh[:n], vc[:n], nc[:n], offs, lst)


def mix64(z: int) -> int:
    return int(load("oracle").tm_mix64(z))


def grid_dims(dim: int, gfh: float) -> tuple[int, int, int]:
    """Size of the one-rank grid (grid.c:37-77) for the given resolution."""
    g = int((np.float32(2049.0) + np.float32(1.0)) / np.float32(gfh)) + 1
    return (g, g, g if dim == 3 else 1)


def env2cells(col, data: np.ndarray, gradient: np.ndarray, *, gfh: float = 8.0, which: str = "oracle") -> np.ndarray:
    """Grid -> cell gather (patches_applyenv2cells at one rank).

    data: (nfields, gx, gy, gz) float64; gradient: (nfields, gx, gy, gz, 3).
    Returns cellenv (nfields, n, 4) = value, gx, gy, gz per field and cell."""
    lib = load(which)
    nf = int(data.shape[0])
    data = np.ascontiguousarray(data, np.float64)
    gradient = np.ascontiguousarray(gradient, np.float64)
    out = np.zeros((nf, col.n, 4))
    x, y, z = (np.ascontiguousarray(a, np.float64) for a in (col.x, col.y, col.z))
    if which == "oracle":
        rc = lib.tmo_env2cells(col.n, col.dim, _ptr(x), _ptr(y), _ptr(z), float(gfh), nf, _ptr(data),
                               _ptr(gradient), _ptr(out))
    else:
        ph = np.ascontiguousarray(col.phase, np.int32)
        rc = lib.ref_env2cells(col.n, col.dim, _ptr(x), _ptr(y), _ptr(z), _ptr(ph), float(gfh), nf, _ptr(data),
                               _ptr(gradient), int(np.prod(data.shape[1:])), _ptr(out))
        rc = 0 if rc > 0 else -1
    if rc:
        raise RuntimeError(f"env2cells ({which}) failed: {rc}")
    return out


def fieldgradient(data: np.ndarray, *, dim: int = 3, gfh: float = 8.0, which: str = "oracle") -> np.ndarray:
    """Field gradient (fieldgradient_compute at one rank) of data (nfields, gx, gy, gz);
    returns (nfields, gx, gy, gz, 3)."""
    lib = load(which)
    nf = int(data.shape[0])
    data = np.ascontiguousarray(data, np.float64)
    out = np.zeros(data.shape + (3,))
    dims = np.zeros(3, np.int64)
    if which == "oracle":
        rc = lib.tmo_fieldgradient(dim, float(gfh), nf, _ptr(data), _ptr(out), _ptr(dims))
    else:
        rc = lib.ref_fieldgradient(dim, float(gfh), nf, _ptr(data), int(np.prod(data.shape[1:])), _ptr(out),
                                   _ptr(dims))
        rc = 0 if rc > 0 else -1
    if rc or tuple(dims) != tuple(data.shape[1:]):
        raise RuntimeError(f"fieldgradient ({which}) failed: {rc}, grid {tuple(dims)} vs {data.shape[1:]}")
    return out


def write_vtk(path: str, x, y, z, ctype, fx, fy, fz, *, which: str = "oracle") -> bytes:
    """writevtk at one rank for cells in caller order; returns the file's bytes.
    The reference writes vtk/step00000000.vtk under the directory of path."""
    lib = load(which)
    arr = [np.ascontiguousarray(a, np.float64) for a in (x, y, z)]
    ct = np.ascontiguousarray(ctype, np.int32)
    fs = [np.ascontiguousarray(a, np.float64) for a in (fx, fy, fz)]
    n = len(arr[0])
    if which == "oracle":
        rc = lib.tmo_write_vtk(path.encode(), n, *[_ptr(a) for a in arr], _ptr(ct), *[_ptr(a) for a in fs], 0)
        out = path
    else:
        d = os.path.dirname(os.path.abspath(path))
        os.makedirs(os.path.join(d, "vtk"), exist_ok=True)
        rc = lib.ref_write_vtk(d.encode(), 0, n, *[_ptr(a) for a in arr], _ptr(ct), *[_ptr(a) for a in fs])
        out = os.path.join(d, "vtk", "step00000000.vtk")
    if rc:
        raise RuntimeError(f"write_vtk ({which}) failed: {rc}")
    with open(out, "rb") as f:
        return f.read()


def survivors(n: int, oldlnc: int, removecell, globalcount: int | None = None) -> np.ndarray:
    """Order of the cells after cellsdeath (cells.c:290-336): the unmarked
    cells before oldlnc, then every cell appended after it; nothing is
    removed when the simulation holds one cell."""
    removecell = np.asarray(removecell, np.uint8)
    if (globalcount if globalcount is not None else n) == 1:
        return np.arange(n)
    head = np.nonzero(removecell[:oldlnc] == 0)[0]
    return np.concatenate([head, np.arange(oldlnc, n)])


def ref_survivors(n: int, oldlnc: int, removecell, globalcount: int | None = None) -> np.ndarray:
    """The same through the reference's own cellsdeath."""
    lib = load("ref_strict")
    rc = np.ascontiguousarray(np.pad(np.asarray(removecell, np.uint8), (0, max(0, n - len(removecell)))))
    order = np.zeros(max(n, 1), np.int64)
    m = lib.ref_cellsdeath(n, oldlnc, _ptr(rc), int(rc[:oldlnc].sum()), globalcount if globalcount else n,
                           _ptr(order))
    return order[:m]


CYCLE_STATE = (("phase", np.int32), ("phasetime", np.float32), ("g1", np.float32), ("s", np.float32),
               ("g2", np.float32), ("m", np.float32), ("age", np.int32), ("size", np.float64),
               ("young", np.float32), ("x", np.float64), ("y", np.float64), ("z", np.float64),
               ("density", np.float64), ("ctype", np.int32))


def libc_draws(seed: int, count: int) -> np.ndarray:
    """The first count values of the C library's rand() after srand(seed)."""
    libc = C.CDLL(None)
    libc.rand.restype = C.c_int
    libc.srand.argtypes = [C.c_uint]
    libc.srand(seed)
    return np.array([libc.rand() for _ in range(count)], np.int32)


def cellcycle(state: dict, types: dict, *, dim: int = 3, nfields: int = 0, envvalue=None, cl1=None, cl2=None,
              simulationstart: int = 1, sps: float = 3600.0, seed: int = 1, cap: int | None = None,
              removecell=None, which: str = "oracle", draws=None) -> dict:
    """updatecellcycles with mitosis on caller-ordered cells.

    state: arrays named as in CYCLE_STATE; types: per-type g1, s, g2, m, v, rd,
    cd (criticaldensity) float arrays and size (float64).  The oracle takes its
    draws from the C library's rand() after srand(seed) (or from draws); the
    reference calls rand() itself.  Returns the new state (daughters appended),
    removecell, removecount, and, for the oracle, the draws used."""
    lib = load(which)
    n = len(state["phase"])
    cap = cap or 2 * n + 1
    st = {k: np.zeros(cap, dt) for k, dt in CYCLE_STATE}
    for k, dt in CYCLE_STATE:
        st[k][:n] = np.asarray(state[k], dt)
    rem = np.zeros(cap, np.uint8)
    if removecell is not None:
        rem[:n] = removecell
    ntypes = len(types["g1"])
    ty = [np.ascontiguousarray(types[k], np.float32) for k in ("g1", "s", "g2", "m", "v", "rd", "cd")]
    tsize = np.ascontiguousarray(types["size"], np.float64)
    nf = int(nfields)
    env = np.ascontiguousarray(envvalue if envvalue is not None else np.zeros(max(nf, 1) * max(n, 1)), np.float64)
    c1 = np.ascontiguousarray(cl1 if cl1 is not None else np.zeros(max(ntypes * nf, 1)), np.float32)
    c2 = np.ascontiguousarray(cl2 if cl2 is not None else np.zeros(max(ntypes * nf, 1)), np.float32)
    rc_count = C.c_int64(0)
    nout = C.c_int64(0)
    arrays = [_ptr(st[k]) for k, _ in CYCLE_STATE]
    out = {}
    if which == "oracle":
        dr = np.ascontiguousarray(draws if draws is not None else libc_draws(seed, 13 * n + 16), np.int32)
        used = C.c_int64(0)
        rc = lib.tmo_cellcycle(n, dim, *[_ptr(a) for a in ty], _ptr(tsize), nf, _ptr(c1), _ptr(c2),
                               simulationstart, sps, _ptr(env), _ptr(dr), len(dr), *arrays, _ptr(rem),
                               C.byref(rc_count), cap, C.byref(nout), C.byref(used))
        out["draws_used"] = int(used.value)
    else:
        rc = lib.ref_cellcycle(n, dim, ntypes, *[_ptr(a) for a in ty], _ptr(tsize), nf, _ptr(c1), _ptr(c2),
                               simulationstart, sps, seed, _ptr(env), *arrays, _ptr(rem), C.byref(rc_count), cap,
                               C.byref(nout))
    if rc:
        raise RuntimeError(f"cellcycle ({which}) failed: {rc}")
    m = int(nout.value)
    out.update({k: st[k][:m].copy() for k, _ in CYCLE_STATE})
    out["removecell"] = rem[:m].copy()
    out["removecount"] = int(rc_count.value)
    return out


# celldata_t (global.h:100-120) as the reference lays it out: 112-byte records
REF_CELL_DTYPE = np.dtype({
    "names": ["lifetime", "phase", "age", "death", "phasetime", "g1", "s", "g2", "m", "young", "gid", "x", "y", "z",
              "size", "v", "density", "mindist", "ctype"],
    "formats": ["<i4", "<i4", "<i4", "<i4", "<f4", "<f4", "<f4", "<f4", "<f4", "<f4", "<i4", "<f8", "<f8", "<f8",
                "<f8", "<f8", "<f8", "<f8", "<i4"],
    "offsets": [0, 4, 8, 12, 16, 20, 24, 28, 32, 36, 40, 48, 56, 64, 72, 80, 88, 96, 104],
    "itemsize": 112})


def phase_counts(phase, ctype, ntypes: int) -> np.ndarray:
    """localcount's 7 values then localtypecount's 7 per type (cellcount_t,
    global.h:90-98) for cells with the given phases and types."""
    out = np.zeros(7 + 7 * ntypes, np.uint64)
    phase = np.asarray(phase)
    ctype = np.asarray(ctype)
    out[0] = len(phase)
    for p in range(6):
        out[1 + p] = np.count_nonzero(phase == p)
    for t in range(ntypes):
        sel = ctype == t
        out[7 + 7 * t] = np.count_nonzero(sel)
        for p in range(6):
            out[7 + 7 * t + 1 + p] = np.count_nonzero(sel & (phase == p))
    return out


def ref_cellsupdate(records: np.ndarray, n: int, types, cycle: dict, *, dim: int = 3, simulationstart: int = 1,
                    sps: float = 3600.0, seed: int = 1, steps: int = 1, counts=None,
                    which: str = "ref_strict") -> tuple[np.ndarray, np.ndarray]:
    """The reference's step loop with its whole cell update (octbuild,
    computepotential, computegradient, cellsupdate) for ``steps`` steps after
    srand(seed) on REF_CELL_DTYPE records (len(records) = room for cells).
    types: a CellTypes; cycle: per-type g1, s, g2, m, v, rd, cd.  Returns the
    records in use and the counters after the run."""
    lib = load(which)
    rec = np.ascontiguousarray(records.copy())
    cap = len(rec)
    nt = types.ntypes
    cnt = np.ascontiguousarray(counts if counts is not None else
                               phase_counts(rec["phase"][:n], rec["ctype"][:n], nt), np.uint64).copy()
    tp = [np.ascontiguousarray(a, np.float64) for a in (types.h, types.h2, types.h3, types.h4, types.size)]
    rm = np.ascontiguousarray(types.randommove, np.float32)
    cy = [np.ascontiguousarray(cycle[k], np.float32) for k in ("g1", "s", "g2", "m", "v", "rd", "cd")]
    nn = C.c_int64(n)
    rc = lib.ref_cellsupdate_run(_ptr(rec), C.byref(nn), cap, dim, nt, *[_ptr(a) for a in tp], _ptr(rm),
                                 *[_ptr(a) for a in cy], simulationstart, sps, seed, steps, _ptr(cnt))
    if rc:
        raise RuntimeError(f"ref_cellsupdate_run failed: {rc}")
    return rec[:int(nn.value)].copy(), cnt


def diffuse(gsize, resolution: float, sps: float, gfdt: float, step: int, dc, bc, mean, lam, *, u0=None,
            source=None, tol: float = 1e-15) -> dict:
    """environment_compute's diffusion step at one rank (tmo_diffuse): fields
    of shape (nfields, nx, ny, nz), z fastest.  u0 replaces the mean as the
    start, source the point source."""
    lib = load("oracle")
    nx, ny, nz = (int(v) for v in gsize)
    nf = len(dc)
    arr = [np.ascontiguousarray(v, np.float64) for v in (dc, bc, mean, lam)]
    u = np.zeros((nf, nx, ny, nz))
    b = np.zeros((nf, nx, ny, nz))
    it = C.c_int(0)
    cg = C.c_int(0)
    u0c = None if u0 is None else np.ascontiguousarray(u0, np.float64)
    src = None if source is None else np.ascontiguousarray(source, np.float64)
    rc = lib.tmo_diffuse(nx, ny, nz, resolution, sps, gfdt, step, nf, *[_ptr(a) for a in arr], _ptr(u0c), _ptr(src),
                         tol, _ptr(u), _ptr(b), C.byref(it), C.byref(cg))
    if rc:
        raise RuntimeError(f"tmo_diffuse failed: {rc}")
    return {"u": u, "b": b, "iters": int(it.value), "cg_iters": int(cg.value)}


def diffusion_iters(sps: float, gfdt: float) -> int:
    return int(load("oracle").tmo_diffusion_iters(sps, gfdt))


def diffusion_z(dc: float, gfdt: float, resolution: float) -> float:
    return float(load("oracle").tmo_diffusion_z(dc, gfdt, resolution))


def ref_environment(dim: int, gfh: float, sps: float, gfdt: float, step: int, dc, bc, mean, lam,
                    ncalls: int = 1) -> dict:
    """The reference's environment_initsystem + ncalls x environment_compute
    on the Hypre stand-in (oracle/_ref/libtimothy_ref_env.so).  Returns the
    grid size, numberofiters, z, the requested tolerance and iteration cap,
    the solves made, the stencil coefficients (nfields, nx, ny, nz, 7), and
    the last right-hand side and solution (nfields, nx, ny, nz)."""
    lib = load("ref_env")
    nf = len(dc)
    gx, gy, gz = grid_dims(dim, gfh)
    cap = gx * gy * gz
    arr = [np.ascontiguousarray(v, np.float64) for v in (dc, bc, mean, lam)]
    gs = np.zeros(3, np.int64)
    info = np.zeros(4, np.int32)
    z = np.zeros(nf)
    tol = np.zeros(1)
    coef = np.zeros(nf * cap * 7)
    b = np.zeros(nf * cap)
    x = np.zeros(nf * cap)
    G = lib.ref_environment(dim, gfh, sps, gfdt, step, nf, *[_ptr(a) for a in arr], ncalls, cap, _ptr(gs),
                            _ptr(info), _ptr(z), _ptr(tol), _ptr(coef), _ptr(b), _ptr(x))
    if G < 0:
        raise RuntimeError("ref_environment: grid larger than expected")
    nx, ny, nz = (int(v) for v in gs)

    def xmajor(a, extra=()):
        # box order (x fastest) -> (nx, ny, nz), z fastest
        a = a.reshape((nf, nz, ny, nx) + extra)
        return np.ascontiguousarray(np.moveaxis(a, (1, 2, 3), (3, 2, 1)))

    return {"gsize": (nx, ny, nz), "iters": int(info[0]), "maxiter": int(info[1]), "nsolves": int(info[2]),
            "z": z, "tol": float(tol[0]), "coef": xmajor(coef[:nf * G * 7], (7,)), "b": xmajor(b[:nf * G]),
            "x": xmajor(x[:nf * G])}
