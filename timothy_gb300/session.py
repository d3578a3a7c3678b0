"""Python binding of the device-resident session API (include/timothy_gb300.h).

A thin ctypes layer over libtimothy_gb300.so: every call goes to the CUDA
library; there is no Python or CPU implementation behind it.  If the library
is missing, loading raises instead of falling back.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .colonies import CellTypes, Colony

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libtimothy_gb300.so")

PREC = {"fp64": 0, "fp32c": 1}
UPDATE = {"reference": 0, "dt": 1, "none": 2}


class TimothyError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"timothy_gb300 error {code}: {msg}")
        self.code = code


class _CellTypes(C.Structure):
    _fields_ = [("ntypes", C.c_int), ("h", C.c_void_p), ("h2", C.c_void_p), ("h3", C.c_void_p),
                ("h4", C.c_void_p), ("size", C.c_void_p), ("randommove", C.c_void_p)]


class _Config(C.Structure):
    _fields_ = [("dimension", C.c_int), ("device", C.c_int), ("max_slots", C.c_int64), ("max_colonies", C.c_int),
                ("max_bin_entries", C.c_int64), ("max_grid_entries", C.c_int64), ("diagnostics", C.c_int),
                ("list_capacity", C.c_int)]


class _Input(C.Structure):
    _fields_ = [("n", C.c_int64), ("x", C.c_void_p), ("y", C.c_void_p), ("z", C.c_void_p), ("size", C.c_void_p),
                ("young", C.c_void_p), ("ctype", C.c_void_p), ("phase", C.c_void_p)]


class _Options(C.Structure):
    _fields_ = [("precision", C.c_int), ("update_mode", C.c_int), ("dt", C.c_double), ("cic", C.c_int),
                ("gfh", C.c_float), ("lcap", C.c_int), ("reserve", C.c_int64), ("verlet", C.c_int),
                ("skin", C.c_float), ("rmax", C.c_int)]


class _Output(C.Structure):
    _fields_ = [(k, C.c_void_p) for k in ("x", "y", "z", "density", "v", "mindist", "fx", "fy", "fz", "removecell",
                                           "nbcount", "nbhash", "vcand", "grid")]


class _Info(C.Structure):
    _fields_ = [("aff_shift", C.c_double * 3), ("aff_scale", C.c_double), ("octsize", C.c_int64),
                ("removecount", C.c_int64), ("patch_lower", C.c_int64 * 3), ("patch_upper", C.c_int64 * 3),
                ("grid_size", C.c_int64 * 3), ("device_errors", C.c_uint32), ("bin_level", C.c_int),
                ("n", C.c_int64), ("list_rebuilds", C.c_int64), ("codes_slow", C.c_int64),
                ("list_maxdisp", C.c_float), ("list_skin", C.c_float), ("list_age", C.c_int32),
                ("density_fp64_cells", C.c_int64), ("walked_cells", C.c_int64),
                ("walked_isolated_cells", C.c_int64)]


class _CycleType(C.Structure):
    _fields_ = [("g1", C.c_float), ("s", C.c_float), ("g2", C.c_float), ("m", C.c_float), ("v", C.c_float),
                ("rd", C.c_float), ("criticaldensity", C.c_float)]


_DRAW = C.CFUNCTYPE(C.c_int, C.c_void_p)


class _CycleParams(C.Structure):
    _fields_ = [("types", C.POINTER(_CycleType)), ("nfields", C.c_int), ("criticallevel1", C.c_void_p),
                ("criticallevel2", C.c_void_p), ("cellenv", C.c_void_p), ("simulationstart", C.c_int),
                ("secondsperstep", C.c_float), ("draw", _DRAW), ("draw_ctx", C.c_void_p),
                ("rand_seeded", C.c_int), ("rand_seed", C.c_uint32), ("rand_offset", C.POINTER(C.c_int64))]


class RandStream:
    """The C library's rand() stream after srand(seed), for cellcycle(): the
    values are generated on the device (tm_cycle_params.rand_seeded);
    ``offset`` counts the values taken so far."""

    def __init__(self, seed: int, offset: int = 0):
        self.seed = int(seed) & 0xffffffff
        self.offset = int(offset)


class _Tuning(C.Structure):
    _fields_ = [("pair_lshift", C.c_int), ("list_variant", C.c_int), ("walk_block", C.c_int),
                ("skin_over_h", C.c_float), ("rmax", C.c_int)]


_lib = None


def load_library(path: str = LIB_PATH) -> C.CDLL:
    """Load the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} missing: build it with `python -m timothy_gb300.build`")
    lib = C.CDLL(path)
    P = C.c_void_p
    sigs = {
        "tm_last_error": (C.c_char_p, []),
        "tm_version": (C.c_char_p, []),
        "tm_device_count": (C.c_int, []),
        "tm_measure_fp32_peak": (C.c_int, [C.c_int, C.POINTER(C.c_double)]),
        "tm_check_numerics": (C.c_int, [C.c_int, C.c_int64, C.c_uint64, P]),
        "tm_session_create": (C.c_int, [C.POINTER(P), C.POINTER(_Config), C.POINTER(_CellTypes)]),
        "tm_session_destroy": (C.c_int, [P]),
        "tm_session_stream": (P, [P]),
        "tm_colony_add": (C.c_int, [P, C.POINTER(_Input), C.POINTER(_Options), C.POINTER(C.c_int)]),
        "tm_colony_remove": (C.c_int, [P, C.c_int]),
        "tm_colony_upload": (C.c_int, [P, C.c_int, C.POINTER(_Input)]),
        "tm_colony_set_active": (C.c_int, [P, C.c_int, C.c_int]),
        "tm_colony_download": (C.c_int, [P, C.c_int, C.POINTER(_Output)]),
        "tm_colony_upload_async": (C.c_int, [P, C.c_int, C.POINTER(_Input)]),
        "tm_colony_download_async": (C.c_int, [P, C.c_int, C.POINTER(_Output)]),
        "tm_colony_stats": (C.c_int, [P, C.c_int, C.POINTER(_Info)]),
        "tm_session_step": (C.c_int, [P, C.c_int]),
        "tm_session_sync": (C.c_int, [P]),
        "tm_session_use_graph": (C.c_int, [P, C.c_int]),
        "tm_session_profile": (C.c_int, [P, C.c_int]),
        "tm_session_profile_read": (C.c_int, [P, P, C.c_int, P]),
        "tm_session_capacity": (C.c_int, [P, P, P, P]),
        "tm_session_timer": (C.c_int, [P, C.c_int, P]),
        "tm_session_launches": (C.c_int64, [P]),
        "tm_session_list_rate": (C.c_int, [P, P, P]),
        "tm_env2cells": (C.c_int, [P, P, P, C.c_int64, C.c_int, P, C.c_float, P, C.c_int, P, P, P, P]),
        "tm_field_gradient": (C.c_int, [P, P, C.c_float, C.c_int, P, P]),
        "tm_diffusion_create": (C.c_int, [C.POINTER(P), P, C.c_int]),
        "tm_diffusion_destroy": (C.c_int, [P]),
        "tm_diffusion_levels": (C.c_int, [P]),
        "tm_diffusion_step": (C.c_int, [P, P, C.c_float, C.c_int, P, P, P, C.c_float, C.c_float, P, C.c_double, P,
                                        P]),
        "tm_field_diffuse": (C.c_int, [P, P, C.c_float, C.c_int, P, P, P, C.c_float, C.c_float, P, C.c_double, P,
                                       P]),
        "tm_colony_env2cells": (C.c_int, [P, C.c_int, P, C.c_float, P, C.c_int, P, P, P]),
        "tm_colony_write_vtk": (C.c_int, [P, C.c_int, C.c_char_p, C.c_int]),
        "tm_colony_compact": (C.c_int, [P, C.c_int, P]),
        "tm_colony_set_cycle": (C.c_int, [P, C.c_int, P, P, P, P, P, P]),
        "tm_colony_get_cycle": (C.c_int, [P, C.c_int, P, P, P, P, P, P, P, P, P]),
        "tm_colony_cellcycle": (C.c_int, [P, C.c_int, C.POINTER(_CycleParams), P, P]),
        "tm_colony_append": (C.c_int, [P, C.c_int, C.POINTER(_Input)]),
        "tm_session_bytes": (C.c_int64, [C.POINTER(_Config), C.c_int]),
        "tm_device_memory": (C.c_int, [C.c_int, P, P]),
        "tm_session_get_tuning": (C.c_int, [P, C.POINTER(_Tuning)]),
        "tm_session_set_tuning": (C.c_int, [P, C.POINTER(_Tuning)]),
        "tm_host_register": (C.c_int, [P, C.c_int64]),
        "tm_host_unregister": (C.c_int, [P]),
        "tm_session_set_diagnostics": (C.c_int, [P, C.c_int]),
        "tm_colony_add_async": (C.c_int, [P, C.POINTER(_Input), C.POINTER(_Options), C.POINTER(C.c_int)]),
        "tm_session_fence": (C.c_int, [P, C.POINTER(C.c_int64)]),
        "tm_session_wait": (C.c_int, [P, C.c_int64]),
        "tm_colony_sample_neighbours": (C.c_int, [P, C.c_int, P, C.c_int64, C.c_int]),
        "tm_colony_read_neighbours": (C.c_int, [P, C.c_int, P, P]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _check(rc: int):
    if rc != 0:
        raise TimothyError(rc, load_library().tm_last_error().decode())


def _p(a):
    return None if a is None else a.ctypes.data


def session_bytes(*, max_slots: int, max_colonies: int = 1, dim: int = 3, ntypes: int = 1, max_bin_entries: int = 0,
                  max_grid_entries: int = 0, diagnostics: bool = False, list_capacity: int = 0) -> int:
    """Device bytes a Session with these arguments allocates."""
    cfg = _Config(dim, 0, int(max_slots), int(max_colonies), int(max_bin_entries), int(max_grid_entries),
                  1 if diagnostics else 0, int(list_capacity))
    b = int(load_library().tm_session_bytes(C.byref(cfg), int(ntypes)))
    if b < 0:
        raise ValueError("bad session configuration")
    return b


def device_memory(device: int = 0) -> tuple[int, int]:
    """(free, total) bytes of a device."""
    f = np.zeros(1, np.int64)
    t = np.zeros(1, np.int64)
    _check(load_library().tm_device_memory(int(device), _p(f), _p(t)))
    return int(f[0]), int(t[0])


def _dptr(a) -> int:
    """Device address of a CUDA array (anything with data_ptr(), or an int)."""
    return int(a.data_ptr()) if hasattr(a, "data_ptr") else int(a)


def env2cells_device(x, y, z, n: int, dim: int, lower, resolution: float, gsize, nfields: int, data, gradient,
                     cellenv, stream=None):
    """tm_env2cells on device arrays (x, y, z, data, gradient, cellenv: CUDA arrays)."""
    lo = np.ascontiguousarray(lower, np.float64)
    gs = np.ascontiguousarray(gsize, np.int64)
    _check(load_library().tm_env2cells(_dptr(x), _dptr(y), _dptr(z), int(n), int(dim), _p(lo), float(resolution),
                                       _p(gs), int(nfields), _dptr(data), _dptr(gradient), _dptr(cellenv),
                                       None if stream is None else _dptr(stream)))


def field_gradient_device(data, gsize, resolution: float, nfields: int, gradient, stream=None):
    """tm_field_gradient on device arrays."""
    gs = np.ascontiguousarray(gsize, np.int64)
    _check(load_library().tm_field_gradient(_dptr(data), _p(gs), float(resolution), int(nfields), _dptr(gradient),
                                            None if stream is None else _dptr(stream)))


class DiffusionStats(C.Structure):
    _fields_ = [("solves_per_field", C.c_int), ("iterations", C.c_int), ("max_iterations", C.c_int),
                ("refinements", C.c_int), ("multigrid_fields", C.c_int), ("levels", C.c_int),
                ("max_relative_residual", C.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class Diffusion:
    """tm_diffusion: the implicit diffusion step of environment_compute on
    device fields of one grid size (work vectors allocated once)."""

    def __init__(self, gsize, device: int = 0):
        self.lib = load_library()
        self.gsize = tuple(int(v) for v in gsize)
        gs = np.ascontiguousarray(self.gsize, np.int64)
        h = C.c_void_p()
        _check(self.lib.tm_diffusion_create(C.byref(h), _p(gs), int(device)))
        self.h = h

    @property
    def levels(self) -> int:
        return int(self.lib.tm_diffusion_levels(self.h))

    def step(self, data, resolution: float, dc, bc, lam, secondsperstep: float, gfdt: float, source=None,
             tol: float = 1e-12, stream=None) -> dict:
        """One step on data (CUDA array, nfields x gsize, z fastest), in place."""
        dcs, bcs, lams = (np.ascontiguousarray(np.atleast_1d(v), np.float64) for v in (dc, bc, lam))
        st = DiffusionStats()
        _check(self.lib.tm_diffusion_step(self.h, _dptr(data), float(resolution), len(dcs), _p(dcs), _p(bcs),
                                          _p(lams), float(secondsperstep), float(gfdt),
                                          None if source is None else _dptr(source), float(tol), C.byref(st),
                                          None if stream is None else _dptr(stream)))
        return st.as_dict()

    def close(self):
        if self.h:
            self.lib.tm_diffusion_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def host_register(a: np.ndarray):
    """Page-lock a numpy array for full-speed copies."""
    _check(load_library().tm_host_register(a.ctypes.data, a.nbytes))


def host_unregister(a: np.ndarray):
    _check(load_library().tm_host_unregister(a.ctypes.data))


def device_count() -> int:
    return int(load_library().tm_device_count())


def check_numerics(n: int = 1 << 24, seed: int = 1, device: int = 0) -> dict:
    """Mismatch counts of the kernels' own arithmetic against the hardware
    and library operations (tm_check_numerics); every count must be 0."""
    m = np.zeros(3, np.int64)
    _check(load_library().tm_check_numerics(int(device), int(n), int(seed), _p(m)))
    return {"quotient": int(m[0]), "round_to_float": int(m[1]), "float_to_double": int(m[2])}


def measure_fp32_peak(device: int = 0) -> float:
    """Measured FP32 FMA rate of the device in TFLOP/s."""
    r = C.c_double(0.0)
    _check(load_library().tm_measure_fp32_peak(int(device), C.byref(r)))
    return float(r.value)


class Session:
    """A set of colonies resident on one GPU."""

    def __init__(self, types: CellTypes | None = None, *, dim: int = 3, max_slots: int = 1 << 16,
                 max_colonies: int = 1, diagnostics: bool = False, device: int = 0, max_bin_entries: int = 0,
                 max_grid_entries: int = 0, list_capacity: int = 0):
        lib = load_library()
        self.types = types or CellTypes.consistent()
        self._keep = [np.ascontiguousarray(a, dt) for a, dt in
                      ((self.types.h, np.float64), (self.types.h2, np.float64), (self.types.h3, np.float64),
                       (self.types.h4, np.float64), (self.types.size, np.float64),
                       (self.types.randommove, np.float32))]
        ct = _CellTypes(self.types.ntypes, *[_p(a) for a in self._keep])
        cfg = _Config(dim, device, int(max_slots), int(max_colonies), int(max_bin_entries), int(max_grid_entries),
                      1 if diagnostics else 0, int(list_capacity))
        h = C.c_void_p()
        _check(lib.tm_session_create(C.byref(h), C.byref(cfg), C.byref(ct)))
        self._h = h
        self.dim = dim
        self.diagnostics = diagnostics
        self._n = {}
        self._keep_async = []          # (fence id after them, arrays) of queued asynchronous uploads
        self._fences = 0               # id of the next fence
        self._grid = {}

    # -- lifetime ---------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            load_library().tm_session_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return int(load_library().tm_session_stream(self._h) or 0)

    # -- colonies -----------------------------------------------------------
    @staticmethod
    def _input(col: Colony):
        arrs = [np.ascontiguousarray(col.x, np.float64), np.ascontiguousarray(col.y, np.float64),
                np.ascontiguousarray(col.z, np.float64), np.ascontiguousarray(col.size, np.float64),
                np.ascontiguousarray(col.young, np.float32), np.ascontiguousarray(col.ctype, np.int32),
                np.ascontiguousarray(col.phase, np.int32)]
        return _Input(col.n, *[_p(a) for a in arrs]), arrs

    def add_colony(self, col: Colony, *, precision: str = "fp64", update: str = "reference", dt: float = 1.0,
                   cic: bool = False, gfh: float = 8.0, lcap: int = 0, reserve: int = 0, verlet: bool = False,
                   skin: float = 0.0, rmax: int = 0, wait: bool = True) -> int:
        """Add a colony; wait=False queues it behind the work in flight
        (tm_colony_add_async) instead of waiting for the copies."""
        inp, keep = self._input(col)
        opt = _Options(PREC[precision], UPDATE[update], float(dt), 1 if cic else 0, float(gfh), int(lcap),
                       int(reserve), 1 if verlet else 0, float(skin), int(rmax))
        cid = C.c_int(-1)
        fn = load_library().tm_colony_add if wait else load_library().tm_colony_add_async
        _check(fn(self._h, C.byref(inp), C.byref(opt), C.byref(cid)))
        if not wait:
            self._keep_async.append((self._fences, keep))
        self._n[cid.value] = col.n
        if cic:
            g = int((2049.0 + 1) / gfh) + 1
            self._grid[cid.value] = (g, g, g if self.dim == 3 else 1)
        return cid.value

    def remove_colony(self, cid: int):
        _check(load_library().tm_colony_remove(self._h, cid))
        self._n.pop(cid, None)
        self._grid.pop(cid, None)

    def upload(self, cid: int, col: Colony):
        inp, keep = self._input(col)
        rc = load_library().tm_colony_upload(self._h, cid, C.byref(inp))
        if rc == 0:
            self._n[cid] = col.n
        elif rc == -4:      # a cell type outside the table: the colony was left empty
            self._n[cid] = 0
        _check(rc)

    def upload_async(self, cid: int, col: Colony):
        """Queue the re-upload of the colony's cells (same n, same order); the
        arrays must stay unchanged until sync()."""
        inp, keep = self._input(col)
        self._keep_async.append((self._fences, keep))
        _check(load_library().tm_colony_upload_async(self._h, cid, C.byref(inp)))

    def upload_positions_async(self, cid: int, x, y, z):
        """Queue an upload of new positions only (same cells, same order; the
        other attributes keep their values); the arrays must stay unchanged
        until sync()."""
        arrs = [np.ascontiguousarray(a, np.float64) for a in (x, y, z)]
        inp = _Input(len(arrs[0]), *[_p(a) for a in arrs], None, None, None, None)
        self._keep_async.append((self._fences, arrs))
        _check(load_library().tm_colony_upload_async(self._h, cid, C.byref(inp)))

    def download_async(self, cid: int, fields, out: dict):
        """Queue the copy of results into out's arrays (caller order); they are
        valid after sync()."""
        n = self._n[cid]
        for k in fields:
            need = int(np.prod(self._grid[cid])) if k == "grid" else n
            if k not in out or out[k].size < need or not out[k].flags.c_contiguous:
                raise ValueError(f"download_async needs a contiguous output array for {k} with {need} entries")
        o = _Output(*[_p(out.get(k)) if k in fields else None for k, _ in _Output._fields_])
        _check(load_library().tm_colony_download_async(self._h, cid, C.byref(o)))

    def compact(self, cid: int) -> int:
        """Remove the cells marked for removal (cellsdeath); returns how many."""
        r = np.zeros(1, np.int64)
        _check(load_library().tm_colony_compact(self._h, cid, _p(r)))
        self._n[cid] -= int(r[0])
        return int(r[0])

    def append(self, cid: int, col: Colony):
        """Append cells after the colony's current ones (needs reserved slots)."""
        inp, keep = self._input(col)
        rc = load_library().tm_colony_append(self._h, cid, C.byref(inp))
        if rc in (0, -4):
            self._n[cid] += col.n
        _check(rc)

    # -- cell cycle -----------------------------------------------------------
    def set_cycle(self, cid: int, phasetime, g1, sphase, g2, m, age):
        """Cell-cycle state of the colony's cells (caller order)."""
        arrs = [np.ascontiguousarray(a, np.float32) for a in (phasetime, g1, sphase, g2, m)]
        ag = np.ascontiguousarray(age, np.int32)
        _check(load_library().tm_colony_set_cycle(self._h, cid, *[_p(a) for a in arrs], _p(ag)))

    def get_cycle(self, cid: int) -> dict:
        n = self._n[cid]
        out = {k: np.zeros(n, np.float32) for k in ("phasetime", "g1", "s", "g2", "m")}
        out["age"] = np.zeros(n, np.int32)
        out["phase"] = np.zeros(n, np.int32)
        out["size"] = np.zeros(n)
        out["young"] = np.zeros(n, np.float32)
        _check(load_library().tm_colony_get_cycle(self._h, cid, *[_p(out[k]) for k in
                                                                  ("phasetime", "g1", "s", "g2", "m", "age",
                                                                   "phase", "size", "young")]))
        return out

    def cellcycle(self, cid: int, types: dict, *, nfields: int = 0, cl1=None, cl2=None, cellenv=None,
                  simulationstart: int = 1, secondsperstep: float = 3600.0, draw=None,
                  stream: RandStream | None = None) -> tuple[int, int]:
        """One cell-cycle step; types holds per-type g1, s, g2, m, v, rd, cd arrays.
        cellenv: device array (nfields, n, 4).  draw: None (the C library's
        rand()) or a callable returning the next value.  Returns (divided, marked)."""
        nt = len(types["g1"])
        tarr = (_CycleType * nt)(*[_CycleType(*(float(types[k][t]) for k in ("g1", "s", "g2", "m", "v", "rd",
                                                                               "cd"))) for t in range(nt)])
        c1 = np.ascontiguousarray(cl1 if cl1 is not None else np.zeros(1), np.float32)
        c2 = np.ascontiguousarray(cl2 if cl2 is not None else np.zeros(1), np.float32)
        fn = _DRAW(lambda ctx: int(draw())) if draw is not None else _DRAW()
        off = C.c_int64(stream.offset if stream is not None else 0)
        prm = _CycleParams(C.cast(tarr, C.POINTER(_CycleType)), int(nfields), _p(c1), _p(c2),
                           _dptr(cellenv) if cellenv is not None else None, int(simulationstart),
                           float(secondsperstep), fn, None, 1 if stream is not None else 0,
                           stream.seed if stream is not None else 0, C.pointer(off))
        d = np.zeros(1, np.int64)
        mk = np.zeros(1, np.int64)
        rc = load_library().tm_colony_cellcycle(self._h, cid, C.byref(prm), _p(d), _p(mk))
        _check(rc)
        if stream is not None:
            stream.offset = int(off.value)
        self._n[cid] += int(d[0])
        return int(d[0]), int(mk[0])

    def set_active(self, cid: int, active: bool):
        _check(load_library().tm_colony_set_active(self._h, cid, 1 if active else 0))

    # -- stepping -----------------------------------------------------------
    def step(self, nsteps: int = 1):
        _check(load_library().tm_session_step(self._h, int(nsteps)))

    def sync(self):
        _check(load_library().tm_session_sync(self._h))
        self._keep_async.clear()

    def fence(self) -> int:
        """A fence after the work queued so far (see tm_session_fence)."""
        f = C.c_int64(-1)
        _check(load_library().tm_session_fence(self._h, C.byref(f)))
        self._fences = int(f.value) + 1
        return int(f.value)

    def wait(self, fence: int):
        """Wait for a fence; the arrays of asynchronous uploads queued before it are released."""
        _check(load_library().tm_session_wait(self._h, int(fence)))
        self._keep_async = [(t, k) for t, k in self._keep_async if t > fence]

    def use_graph(self, on: bool = True):
        _check(load_library().tm_session_use_graph(self._h, 1 if on else 0))

    def profile(self, on: bool = True):
        _check(load_library().tm_session_profile(self._h, 1 if on else 0))

    def set_diagnostics(self, on: bool = True):
        """Neighbour-set fingerprints, v candidates and every cell's octree walk
        for the following steps."""
        _check(load_library().tm_session_set_diagnostics(self._h, 1 if on else 0))
        self.diagnostics = bool(on)

    def sample_neighbours(self, cid: int, cells, lcap: int = 512):
        """Record, in each following step, the neighbours within h of the given
        cells (caller indices) as the pair kernels decide them."""
        c = np.ascontiguousarray(cells, np.int64)
        self._sample = (cid, len(c), int(lcap))
        _check(load_library().tm_colony_sample_neighbours(self._h, cid, _p(c) if len(c) else None, len(c),
                                                          int(lcap)))

    def read_neighbours(self, cid: int) -> list:
        """The sampled cells' neighbour lists of the last step, each sorted
        (caller indices)."""
        scid, m, lcap = self._sample
        if scid != cid:
            raise ValueError("no neighbour sample on this colony")
        cnt = np.zeros(max(m, 1), np.int32)
        lst = np.zeros(max(m * lcap, 1), np.int32)
        _check(load_library().tm_colony_read_neighbours(self._h, cid, _p(cnt), _p(lst)))
        if np.any(cnt[:m] > lcap):
            raise RuntimeError(f"a sampled cell has more than {lcap} neighbours")
        return [np.sort(lst[k * lcap:k * lcap + cnt[k]]) for k in range(m)]

    def profile_read(self) -> dict:
        ms = np.zeros(7)
        steps = np.zeros(1, np.int64)
        _check(load_library().tm_session_profile_read(self._h, _p(ms), 7, _p(steps)))
        out = {"build_ms": ms[0], "search_ms": ms[1], "list_ms": ms[2], "fix_ms": ms[3], "octree_ms": ms[4],
               "update_ms": ms[5], "cic_ms": ms[6], "steps": int(steps[0])}
        out["pair_ms"] = ms[1] + ms[2] + ms[3]
        return {k: (float(v) if k != "steps" else v) for k, v in out.items()}

    def timer_start(self):
        _check(load_library().tm_session_timer(self._h, 0, None))

    def timer_stop(self) -> float:
        ms = np.zeros(1)
        _check(load_library().tm_session_timer(self._h, 1, _p(ms)))
        return float(ms[0])

    @property
    def launches(self) -> int:
        return int(load_library().tm_session_launches(self._h))

    def capacity(self) -> dict:
        fs = np.zeros(1, np.int64)
        fb = np.zeros(1, np.int64)
        fc = np.zeros(1, np.int32)
        _check(load_library().tm_session_capacity(self._h, _p(fs), _p(fb), _p(fc)))
        return {"free_slots": int(fs[0]), "free_bins": int(fb[0]), "free_colonies": int(fc[0])}

    # -- results ------------------------------------------------------------
    def download(self, cid: int, fields=None, out: dict | None = None) -> dict:
        """Copy results to host arrays (caller order); ``out`` may supply them."""
        n = self._n[cid]
        want = fields or ("x", "y", "z", "density", "v", "mindist", "fx", "fy", "fz", "removecell", "nbcount")
        out = dict(out or {})
        dtypes = {"removecell": np.uint8, "nbcount": np.int32, "nbhash": np.uint64, "vcand": np.int32}
        for k in want:
            if k == "grid" or k in out:
                continue
            out[k] = np.zeros(n, dtypes.get(k, np.float64))
        if "grid" in want and cid in self._grid:
            out["grid"] = np.zeros(self._grid[cid])
        o = _Output(*[_p(out.get(k)) for k, _ in _Output._fields_])
        _check(load_library().tm_colony_download(self._h, cid, C.byref(o)))
        return out

    def stats(self, cid: int) -> dict:
        info = _Info()
        _check(load_library().tm_colony_stats(self._h, cid, C.byref(info)))
        return {"aff": np.array(list(info.aff_shift) + [info.aff_scale]), "octsize": int(info.octsize),
                "removecount": int(info.removecount), "patch_lower": list(info.patch_lower),
                "patch_upper": list(info.patch_upper), "device_errors": int(info.device_errors),
                "bin_level": int(info.bin_level), "n": int(info.n), "list_rebuilds": int(info.list_rebuilds),
                "codes_slow": int(info.codes_slow), "list_maxdisp": float(info.list_maxdisp),
                "list_skin": float(info.list_skin), "list_age": int(info.list_age),
                "density_fp64_cells": int(info.density_fp64_cells), "walked_cells": int(info.walked_cells),
                "walked_isolated_cells": int(info.walked_isolated_cells)}

    def list_rate(self) -> tuple[float, int]:
        """(expected fraction of cells rebuilding their lists per step, rebuilds so far)."""
        r = np.zeros(1, np.float64)
        n = np.zeros(1, np.int64)
        _check(load_library().tm_session_list_rate(self._h, _p(r), _p(n)))
        return float(r[0]), int(n[0])

    def env2cells(self, cid: int, lower, resolution: float, gsize, nfields: int, data, gradient) -> np.ndarray:
        """Grid -> cell gather for a colony (device field arrays); (nfields, n, 4) in caller order."""
        n = self._n[cid]
        out = np.zeros((nfields, n, 4))
        lo = np.ascontiguousarray(lower, np.float64)
        gs = np.ascontiguousarray(gsize, np.int64)
        _check(load_library().tm_colony_env2cells(self._h, cid, _p(lo), float(resolution), _p(gs), int(nfields),
                                                  _dptr(data), _dptr(gradient), _p(out)))
        return out

    def write_vtk(self, cid: int, path: str, rank: int = 0):
        """The reference's VTK file of the colony (positions, types, forces of the last step)."""
        _check(load_library().tm_colony_write_vtk(self._h, cid, str(path).encode(), int(rank)))

    # -- tuning -------------------------------------------------------------
    @property
    def tuning(self) -> dict:
        t = _Tuning()
        _check(load_library().tm_session_get_tuning(self._h, C.byref(t)))
        return {k: getattr(t, k) for k, _ in _Tuning._fields_}

    def set_tuning(self, **kw):
        """Change launch shapes / list parameters (see tm_tuning); others keep their values."""
        cur = self.tuning
        unknown = set(kw) - set(cur)
        if unknown:
            raise ValueError(f"unknown tuning keys {sorted(unknown)}")
        cur.update(kw)
        t = _Tuning(**cur)
        _check(load_library().tm_session_set_tuning(self._h, C.byref(t)))


def run_colony(col: Colony, nsteps: int, *, precision: str = "fp64", update: str = "reference", dt: float = 1.0,
               cic: bool = False, gfh: float = 8.0, diagnostics: bool = False, fields=None, verlet: bool = False,
               skin: float = 0.0, rmax: int = 0, list_capacity: int = 256):
    """Upload one colony, advance it nsteps, return (outputs, stats)."""
    with Session(col.types, dim=col.dim, max_slots=max(col.n, 1) + 64, diagnostics=diagnostics,
                 list_capacity=list_capacity if verlet else 0) as s:
        cid = s.add_colony(col, precision=precision, update=update, dt=dt, cic=cic, gfh=gfh, verlet=verlet,
                           skin=skin, rmax=rmax)
        s.step(nsteps)
        s.sync()
        f = fields
        if f is None:
            f = ["x", "y", "z", "density", "v", "mindist", "fx", "fy", "fz", "removecell", "nbcount"]
            if diagnostics:
                f += ["nbhash", "vcand"]
            if cic:
                f += ["grid"]
        return s.download(cid, f), s.stats(cid)
