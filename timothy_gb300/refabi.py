"""ctypes mirror of include/timothy_refabi.h and a driver for the drop-ins.

``DropinRun`` calls the reference-signature entry points of
libtimothy_gb300.so in the order of the reference step loop (main.c:67-79,
step.c:41-100): octbuild, patches_alloc + patches_cells2envinfo,
computepotential, computegradient, updatepositions, octfree.  Cells live in a
host array of celldata_t exactly as in the reference program.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .session import load_library


class cellcount_t(C.Structure):
    _fields_ = [(k, C.c_uint64) for k in ("n", "g0phase", "g1phase", "sphase", "g2phase", "mphase",
                                          "necroticphase")]


class celldata_t(C.Structure):
    _fields_ = [("lifetime", C.c_int), ("phase", C.c_int), ("age", C.c_int), ("death", C.c_int),
                ("phasetime", C.c_float), ("g1", C.c_float), ("s", C.c_float), ("g2", C.c_float),
                ("m", C.c_float), ("young", C.c_float), ("gid", C.c_int), ("x", C.c_double), ("y", C.c_double),
                ("z", C.c_double), ("size", C.c_double), ("v", C.c_double), ("density", C.c_double),
                ("mindist", C.c_double), ("ctype", C.c_int)]


class double3dv_t(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double)]


class int643dv_t(C.Structure):
    _fields_ = [("x", C.c_int64), ("y", C.c_int64), ("z", C.c_int64)]


class octnode_t(C.Structure):
    _fields_ = [("xcode", C.c_uint), ("ycode", C.c_uint), ("zcode", C.c_uint), ("xlimit", C.c_uint),
                ("ylimit", C.c_uint), ("zlimit", C.c_uint), ("level", C.c_uint), ("father", C.c_int64),
                ("child", C.c_int64 * 8), ("data", C.c_int)]


class cellsinfo_t(C.Structure):
    _fields_ = [("localcount", cellcount_t), ("globalcount", cellcount_t), ("localtypecount", C.c_void_p),
                ("globaltypecount", C.c_void_p), ("cellsperproc", C.c_void_p), ("cells", C.c_void_p),
                ("forces", C.c_void_p), ("octree", C.c_void_p), ("octsize", C.c_int64), ("octmaxsize", C.c_int64),
                ("dimension", C.c_int), ("velocity", C.c_void_p)]


class grid_t(C.Structure):
    _fields_ = [("globalsize", int643dv_t), ("lowercorner", double3dv_t), ("uppercorner", double3dv_t),
                ("localsize", int643dv_t), ("resolution", C.c_float), ("loweridx", C.POINTER(int643dv_t)),
                ("upperidx", C.POINTER(int643dv_t)), ("lowleftnear", C.c_void_p), ("uprightfar", C.c_void_p)]


class cellcommdata_t(C.Structure):
    _fields_ = [("explist", C.c_void_p), ("explistmaxsize", C.c_int), ("reqsend", C.c_void_p),
                ("reqrecv", C.c_void_p), ("sendoffset", C.c_void_p), ("recvoffset", C.c_void_p),
                ("recvcount", C.c_void_p), ("sendcount", C.c_void_p), ("sendcellindata", C.c_void_p),
                ("recvcellindata", C.c_void_p), ("sendcelloutdata", C.c_void_p), ("recvcelloutdata", C.c_void_p),
                ("numexp", C.c_int), ("numimp", C.c_int)]


class settings_t(C.Structure):
    _fields_ = [("maxcells", C.c_int64), ("maxlocalcells", C.c_int64), ("numberofsteps", C.c_int),
                ("secondsperstep", C.c_float), ("numberofcelltypes", C.c_int), ("numberoffields", C.c_int),
                ("dimension", C.c_int), ("restart", C.c_int), ("rstfilename", C.c_char * 128),
                ("outdir", C.c_char * 128), ("visoutstep", C.c_int), ("statoutstep", C.c_int),
                ("rstoutstep", C.c_int), ("maxspeed", C.c_float), ("gfdt", C.c_float), ("gfh", C.c_float),
                ("simulationstart", C.c_int), ("rseed", C.c_uint), ("step", C.c_int)]


class systeminfo_t(C.Structure):
    _fields_ = [("rank", C.c_int), ("size", C.c_int), ("nthreads", C.c_int), ("dim", C.c_int * 3),
                ("noderank", C.c_int), ("nodesize", C.c_int), ("memperproc", C.c_int), ("MPI_CART_COMM", C.c_int),
                ("coords", C.c_void_p), ("endian", C.c_int)]


class celltype_t(C.Structure):
    _fields_ = [("name", C.c_char * 128), ("g1", C.c_float), ("s", C.c_float), ("g2", C.c_float),
                ("m", C.c_float), ("v", C.c_float), ("rd", C.c_float), ("size", C.c_double), ("h", C.c_double),
                ("h2", C.c_double), ("h3", C.c_double), ("h4", C.c_double), ("inputfile", C.c_char * 128),
                ("criticaldensity", C.c_float), ("production", C.c_void_p), ("consumption", C.c_void_p),
                ("criticallevel1", C.c_void_p), ("criticallevel2", C.c_void_p), ("randommove", C.c_float)]


class patches_t(C.Structure):
    _fields_ = [("data", C.POINTER(C.POINTER(C.c_double))), ("intersect", C.POINTER(C.c_int)),
                ("receiver", C.c_void_p), ("sender", C.c_void_p), ("recvdata", C.c_void_p),
                ("reqsend", C.c_void_p), ("reqrecv", C.c_void_p), ("lowercorner", C.POINTER(int643dv_t)),
                ("uppercorner", C.POINTER(int643dv_t)), ("lowercornerR", C.c_void_p),
                ("uppercornerR", C.c_void_p), ("size", C.POINTER(int643dv_t)), ("commbuff", C.c_void_p),
                ("buff", C.POINTER(C.c_void_p))]


class cellenvdata_t(C.Structure):
    _fields_ = [("value", C.c_double), ("gx", C.c_double), ("gy", C.c_double), ("gz", C.c_double)]


class environment_t(C.Structure):
    _fields_ = [("name", C.c_char * 128), ("diffusioncoefficient", C.c_double), ("boundarycondition", C.c_double),
                ("initialconditionmean", C.c_double), ("initialconditionvariance", C.c_double),
                ("lambdadelay", C.c_double), ("data", C.c_void_p), ("gradient", C.c_void_p),
                ("production", C.c_void_p)]


SIZES = {"celldata_t": 112, "cellsinfo_t": 192, "celltype_t": 368, "systeminfo_t": 56, "settings_t": 336,
         "cellcommdata_t": 104, "environment_t": 192, "cellenvdata_t": 32}

CELL_DTYPE = np.dtype({"names": [f for f, _ in celldata_t._fields_],
                       "formats": ["<i4", "<i4", "<i4", "<i4", "<f4", "<f4", "<f4", "<f4", "<f4", "<f4", "<i4",
                                   "<f8", "<f8", "<f8", "<f8", "<f8", "<f8", "<f8", "<i4"],
                       "offsets": [getattr(celldata_t, f).offset for f, _ in celldata_t._fields_],
                       "itemsize": C.sizeof(celldata_t)})


def _bind(lib):
    if getattr(lib, "_refabi_bound", False):
        return lib
    lib.octbuild.argtypes = [systeminfo_t, C.POINTER(cellsinfo_t), C.POINTER(celltype_t)]
    lib.octfree.argtypes = [C.POINTER(cellsinfo_t)]
    for f in ("computepotential", "computeremotepotential", "computegradient", "computeremotegradient"):
        getattr(lib, f).argtypes = [systeminfo_t, C.POINTER(cellsinfo_t), C.POINTER(celltype_t), cellcommdata_t]
    lib.updatepositions.argtypes = [settings_t, C.POINTER(celltype_t), C.POINTER(cellsinfo_t), C.c_void_p,
                                    C.POINTER(C.c_int64)]
    lib.patches_alloc.argtypes = [systeminfo_t, settings_t, C.POINTER(patches_t), C.POINTER(cellsinfo_t),
                                  C.POINTER(grid_t)]
    lib.patches_cells2envinfo.argtypes = lib.patches_alloc.argtypes
    lib.patches_applyenv2cells.argtypes = [systeminfo_t, settings_t, C.POINTER(patches_t), C.POINTER(cellsinfo_t),
                                           C.POINTER(grid_t), C.POINTER(C.POINTER(C.POINTER(cellenvdata_t)))]
    lib.fieldgradient.argtypes = [systeminfo_t, settings_t, C.POINTER(C.POINTER(environment_t)), C.POINTER(grid_t)]
    lib.updatecellcycles.argtypes = [systeminfo_t, settings_t, C.POINTER(celltype_t), C.POINTER(cellsinfo_t),
                                     C.c_void_p, C.c_void_p, C.POINTER(C.c_int64)]
    lib.updatecellcycles.restype = C.c_int
    lib.cellsdeath.argtypes = [C.c_int, C.POINTER(cellsinfo_t), C.c_void_p, C.c_int64]
    PENV = C.POINTER(C.POINTER(environment_t))
    lib.environment_allocate.argtypes = [systeminfo_t, settings_t, grid_t, PENV, C.c_void_p, C.c_void_p]
    lib.environment_init.argtypes = [systeminfo_t, settings_t, grid_t, PENV]
    lib.environment_initsystem.argtypes = [systeminfo_t, settings_t, C.POINTER(grid_t), PENV, C.c_void_p,
                                           C.c_void_p]
    lib.environment_compute.argtypes = lib.environment_initsystem.argtypes
    lib.tm_dropin_env_solution.argtypes = [C.c_int, C.c_void_p]
    lib.tm_dropin_env_solution.restype = C.c_int
    lib.tm_dropin_set_env_writeback.argtypes = [C.c_int]
    for f in ("octbuild", "octfree", "computepotential", "computeremotepotential", "computegradient",
              "computeremotegradient", "updatepositions", "patches_alloc", "patches_cells2envinfo",
              "patches_applyenv2cells", "fieldgradient", "cellsdeath", "environment_allocate", "environment_init",
              "environment_initsystem", "environment_compute", "tm_dropin_set_env_writeback",
              "tm_dropin_shutdown"):
        getattr(lib, f).restype = None
    lib._refabi_bound = True
    return lib


def grid_geometry(dim: int, gfh: float):
    """computegridsize at one rank (grid.c:37-77), float arithmetic as there."""
    f = np.float32
    gx = f(f(1024.0 - (-1024.0)) + f(1))
    sx = int(np.float32((gx + f(1)) / f(gfh)))
    sx += 1 - sx % 1
    if dim == 3:
        sz = sx
        lower = (-1024.0, -1024.0, -1024.0)
    else:
        sz = 1
        lower = (-1024.0, -1024.0, 0.0)
    return (sx, sx, sz), lower


def free_patches(p):
    """Free what patches_alloc allocated for one rank (the C library's free)."""
    libc = C.CDLL(None)
    libc.free.argtypes = [C.c_void_p]
    libc.free.restype = None
    if p.data:
        libc.free(C.cast(p.data[0], C.c_void_p))
    for k in ("data", "intersect", "lowercorner", "uppercorner", "lowercornerR", "uppercornerR", "size"):
        ptr = getattr(p, k)
        if ptr:
            libc.free(C.cast(ptr, C.c_void_p))
        setattr(p, k, None)


class DropinRun:
    """The reference step loop on host celldata_t cells, through the drop-ins."""

    def __init__(self, col, *, cic: bool = False, gfh: float = 8.0, nfields: int = 1, cap: int | None = None,
                 cycle: dict | None = None, sps: float = 3600.0, simulationstart: int = 1):
        """cap: records the cells array holds (settings.maxlocalcells); cycle:
        the cell types' g1, s, g2, m, v, rd and cd (criticaldensity), for
        cellsupdate."""
        self.lib = _bind(load_library())
        n = col.n
        self.n = n
        self.dim = col.dim
        cells = np.zeros(max(n, 1, cap or 0), CELL_DTYPE)
        for k in ("x", "y", "z", "size", "young", "ctype", "phase"):
            cells[k][:n] = getattr(col, k)
        cells["gid"][:n] = np.arange(n)
        self.cells = cells
        self.forces = np.zeros((len(cells), 3))           # settings.maxlocalcells entries, as main.c allocates
        t = col.types
        self.celltype = (celltype_t * t.ntypes)()
        for k in range(t.ntypes):
            ct = self.celltype[k]
            ct.h, ct.h2, ct.h3, ct.h4 = float(t.h[k]), float(t.h2[k]), float(t.h3[k]), float(t.h4[k])
            ct.size = float(t.size[k])
            ct.randommove = float(t.randommove[k])
            if cycle is not None:
                ct.g1, ct.s, ct.g2, ct.m = (float(cycle[q][k]) for q in ("g1", "s", "g2", "m"))
                ct.v, ct.rd, ct.criticaldensity = float(cycle["v"][k]), float(cycle["rd"][k]), float(cycle["cd"][k])
        self.si = systeminfo_t()
        self.si.rank, self.si.size = 0, 1
        self.si.dim[0] = self.si.dim[1] = self.si.dim[2] = 1
        self.st = settings_t()
        self.st.dimension = col.dim
        self.st.numberofcelltypes = t.ntypes
        self.st.numberoffields = nfields if cic else 0
        self.st.gfh = gfh
        self.st.maxlocalcells = len(cells)
        self.st.maxcells = len(cells)
        self.st.secondsperstep = sps
        self.st.simulationstart = simulationstart
        self.ci = cellsinfo_t()
        self.ci.localcount.n = n
        self.typecount = (cellcount_t * t.ntypes)()
        self.ci.localtypecount = C.addressof(self.typecount)
        self.ci.cells = cells.ctypes.data
        self.ci.forces = self.forces.ctypes.data
        self.ci.dimension = col.dim
        self.cc = cellcommdata_t()
        self.cic = cic
        if cic:
            (gx, gy, gz), lower = grid_geometry(col.dim, gfh)
            self.gsize = (gx, gy, gz)
            g = grid_t()
            g.resolution = gfh
            g.lowercorner.x, g.lowercorner.y, g.lowercorner.z = lower
            g.localsize.x, g.localsize.y, g.localsize.z = gx, gy, gz
            g.globalsize.x, g.globalsize.y, g.globalsize.z = gx, gy, (gz if col.dim == 3 else 0)
            self._lo = (int643dv_t * 1)()
            self._hi = (int643dv_t * 1)()
            self._hi[0].x, self._hi[0].y, self._hi[0].z = gx - 1, gy - 1, gz - 1
            g.loweridx = self._lo
            g.upperidx = self._hi
            self.grid = g
        self.removecount = C.c_int64(0)
        self.removecell = np.zeros(max(n, 1), np.uint8)
        self.octsize = 0
        self.aff = None
        self.deposit = None

    def step(self, update: bool = True, env=None):
        """One reference step; with env = (data, gradient) (grid arrays of
        shape (nfields, gx, gy, gz) and (nfields, gx, gy, gz, 3)) the fields are
        gathered to the cells before the position update, as step.c:84-86 does
        (self.cellenv, shape (nfields, n, 4))."""
        lib = self.lib
        ct = self.celltype
        lib.octbuild(self.si, C.byref(self.ci), ct)
        self.octsize = int(self.ci.octsize)
        if self.cic:
            p = patches_t()
            lib.patches_alloc(self.si, self.st, C.byref(p), C.byref(self.ci), C.byref(self.grid))
            lib.patches_cells2envinfo(self.si, self.st, C.byref(p), C.byref(self.ci), C.byref(self.grid))
            # at one rank the patch is added into the zeroed grid (patches.c:321-367)
            dep = np.zeros(self.gsize)
            self.patch_corners = None
            if p.intersect and p.intersect[0]:
                lo = p.lowercorner[0]
                up = p.uppercorner[0]
                self.patch_corners = (lo.x, lo.y, lo.z, up.x, up.y, up.z)
                sz = p.size[0]
                vol = sz.x * sz.y * sz.z
                patch = np.ctypeslib.as_array(p.data[0], shape=(vol,)).reshape(sz.x, sz.y, sz.z).copy()
                dep[lo.x:lo.x + sz.x, lo.y:lo.y + sz.y, lo.z:lo.z + sz.z] += patch
            self.deposit = dep
        lib.computepotential(self.si, C.byref(self.ci), ct, self.cc)
        lib.computeremotepotential(self.si, C.byref(self.ci), ct, self.cc)
        lib.computegradient(self.si, C.byref(self.ci), ct, self.cc)
        lib.computeremotegradient(self.si, C.byref(self.ci), ct, self.cc)
        if env is not None and self.cic:
            self._env2cells(p, *env)
        if update:
            lib.updatepositions(self.st, ct, C.byref(self.ci), self.removecell.ctypes.data,
                                C.byref(self.removecount))
        lib.octfree(C.byref(self.ci))
        aff = double3dv_t.in_dll(lib, "affShift")
        self.aff = np.array([aff.x, aff.y, aff.z, C.c_double.in_dll(lib, "affScale").value])

    def step_loop(self, update: bool = True):
        """One step of the reference loop as a host program makes it, and
        nothing else: octbuild, patches_alloc + patches_cells2envinfo (with a
        grid), computepotential, computeremotepotential, computegradient,
        computeremotegradient, updatepositions, octfree (main.c:67-79,
        step.c:41-100).  At one rank the host's own patches_applycells2env
        then adds the patch into its grid and frees the patch buffers
        (patches.c:321-367); here the buffers are only freed."""
        lib = self.lib
        ct = self.celltype
        lib.octbuild(self.si, C.byref(self.ci), ct)
        p = None
        if self.cic:
            p = patches_t()
            lib.patches_alloc(self.si, self.st, C.byref(p), C.byref(self.ci), C.byref(self.grid))
            lib.patches_cells2envinfo(self.si, self.st, C.byref(p), C.byref(self.ci), C.byref(self.grid))
        lib.computepotential(self.si, C.byref(self.ci), ct, self.cc)
        lib.computeremotepotential(self.si, C.byref(self.ci), ct, self.cc)
        lib.computegradient(self.si, C.byref(self.ci), ct, self.cc)
        lib.computeremotegradient(self.si, C.byref(self.ci), ct, self.cc)
        if update:
            lib.updatepositions(self.st, ct, C.byref(self.ci), self.removecell.ctypes.data,
                                C.byref(self.removecount))
        lib.octfree(C.byref(self.ci))
        if p is not None:
            free_patches(p)

    def step_loop_timed(self) -> dict:
        """step_loop with the wall time of each call (seconds)."""
        import time

        lib = self.lib
        ct = self.celltype
        out = {}
        t = time.perf_counter()
        lib.octbuild(self.si, C.byref(self.ci), ct)
        out["octbuild"] = time.perf_counter() - t
        t = time.perf_counter()
        p = None
        if self.cic:
            p = patches_t()
            lib.patches_alloc(self.si, self.st, C.byref(p), C.byref(self.ci), C.byref(self.grid))
            lib.patches_cells2envinfo(self.si, self.st, C.byref(p), C.byref(self.ci), C.byref(self.grid))
        out["patches"] = time.perf_counter() - t
        t = time.perf_counter()
        lib.computepotential(self.si, C.byref(self.ci), ct, self.cc)
        lib.computeremotepotential(self.si, C.byref(self.ci), ct, self.cc)
        out["computepotential"] = time.perf_counter() - t
        t = time.perf_counter()
        lib.computegradient(self.si, C.byref(self.ci), ct, self.cc)
        lib.computeremotegradient(self.si, C.byref(self.ci), ct, self.cc)
        out["computegradient"] = time.perf_counter() - t
        t = time.perf_counter()
        lib.updatepositions(self.st, ct, C.byref(self.ci), self.removecell.ctypes.data, C.byref(self.removecount))
        out["updatepositions"] = time.perf_counter() - t
        lib.octfree(C.byref(self.ci))
        if p is not None:
            free_patches(p)
        return out

    COUNT_FIELDS = ("n", "g0phase", "g1phase", "sphase", "g2phase", "mphase", "necroticphase")

    def set_counts(self, counts):
        """localcount's 7 values then localtypecount's 7 per type; globalcount
        follows localcount (one rank)."""
        for k, f in enumerate(self.COUNT_FIELDS):
            setattr(self.ci.localcount, f, int(counts[k]))
            for t in range(len(self.typecount)):
                setattr(self.typecount[t], f, int(counts[7 + 7 * t + k]))
        self._globalcounts()

    def counts(self) -> np.ndarray:
        out = [getattr(self.ci.localcount, f) for f in self.COUNT_FIELDS]
        for t in range(len(self.typecount)):
            out += [getattr(self.typecount[t], f) for f in self.COUNT_FIELDS]
        return np.array(out, np.uint64)

    def _globalcounts(self):
        # updateglobalcounts (utils.c:80-101) at one rank
        for f in self.COUNT_FIELDS:
            setattr(self.ci.globalcount, f, getattr(self.ci.localcount, f))

    def cellsupdate(self) -> int:
        """cellsupdate (cells.c:525-543) over the drop-ins: random move,
        cell cycle with mitosis, removal, global counts.  Returns the step's
        removecount."""
        lib = self.lib
        oldlnc = int(self.ci.localcount.n)
        rem = np.zeros(max(oldlnc, 1), np.uint8)
        rc = C.c_int64(0)
        lib.updatepositions(self.st, self.celltype, C.byref(self.ci), rem.ctypes.data, C.byref(rc))
        lib.updatecellcycles(self.si, self.st, self.celltype, C.byref(self.ci), None, rem.ctypes.data, C.byref(rc))
        lib.cellsdeath(oldlnc, C.byref(self.ci), rem.ctypes.data, rc.value)
        self._globalcounts()
        self.n = int(self.ci.localcount.n)
        return int(rc.value)

    def cycle_step(self) -> int:
        """One step of the reference loop without fields: octree, potential,
        gradient, then the whole cell update."""
        if self.ci.localcount.n == 0:
            return 0
        self.step(update=False)
        return self.cellsupdate()

    def _env2cells(self, p, data, gradient):
        # the received patch in the reference's layout (patches.c:380-416):
        # every field over the patch box, then 3 gradient values per node and field
        libc = C.CDLL(None)
        libc.malloc.restype = C.c_void_p
        libc.malloc.argtypes = [C.c_size_t]
        nf = int(data.shape[0])
        lo, sz = p.lowercorner[0], p.size[0]
        if not (p.intersect and p.intersect[0]):
            sz = int643dv_t(0, 0, 0)
        box = (slice(None), slice(lo.x, lo.x + sz.x), slice(lo.y, lo.y + sz.y), slice(lo.z, lo.z + sz.z))
        packed = np.concatenate([np.ascontiguousarray(data[box]).ravel(),
                                 np.ascontiguousarray(gradient[box]).ravel()]) if sz.x else np.zeros(1)
        p.buff = C.cast(libc.malloc(C.sizeof(C.c_void_p)), C.POINTER(C.c_void_p))
        p.buff[0] = libc.malloc(max(packed.nbytes, 8))
        C.memmove(p.buff[0], packed.ctypes.data, packed.nbytes)
        st = settings_t.from_buffer_copy(self.st)
        st.numberoffields = nf
        out = C.POINTER(C.POINTER(cellenvdata_t))()
        self.lib.patches_applyenv2cells(self.si, st, C.byref(p), C.byref(self.ci), C.byref(self.grid),
                                        C.byref(out))
        ce = np.zeros((nf, self.n, 4))
        for f in range(nf):
            ce[f] = np.ctypeslib.as_array(C.cast(out[f], C.POINTER(C.c_double)), shape=(self.n * 4,)).reshape(-1, 4)
            libc.free.argtypes = [C.c_void_p]
            libc.free(C.cast(out[f], C.c_void_p))
        libc.free(C.cast(out, C.c_void_p))
        self.cellenv = ce

    def fieldgradient(self, data: np.ndarray) -> np.ndarray:
        """fieldgradient() drop-in on (nfields, gx, gy, gz) host data."""
        nf = int(data.shape[0])
        data = np.ascontiguousarray(data, np.float64)
        grad = np.zeros(data.shape + (3,))
        envs = (environment_t * nf)()
        for f in range(nf):
            envs[f].data = data[f].ctypes.data
            envs[f].gradient = grad[f].ctypes.data
        st = settings_t.from_buffer_copy(self.st)
        st.numberoffields = nf
        penv = C.cast(envs, C.POINTER(environment_t))
        self.lib.fieldgradient(self.si, st, C.byref(penv), C.byref(self.grid))
        return grad

    def outputs(self) -> dict:
        n = self.n
        c = self.cells[:n]
        return {"x": c["x"].copy(), "y": c["y"].copy(), "z": c["z"].copy(), "density": c["density"].copy(),
                "v": c["v"].copy(), "mindist": c["mindist"].copy(), "fx": self.forces[:n, 0].copy(),
                "fy": self.forces[:n, 1].copy(), "fz": self.forces[:n, 2].copy(),
                "removecell": self.removecell[:n].copy()}

    def shutdown(self):
        """Release the drop-ins' device session and the page-locking of this run's cells."""
        self.lib.tm_dropin_shutdown()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.shutdown()


class EnvironmentRun:
    """The reference's field set-up and implicit diffusion step
    (environment.c:33-523: environment_allocate, environment_init,
    environment_initsystem, environment_compute) through the drop-ins, at one
    rank on the grid of the given resolution."""

    def __init__(self, dim: int, gfh: float, fields: list[dict], *, secondsperstep: float, gfdt: float,
                 step: int = 1):
        """fields: dicts with dc, bc, mean, variance, lam."""
        self.lib = _bind(load_library())
        self.si = systeminfo_t()
        self.si.rank, self.si.size = 0, 1
        self.si.dim[0] = self.si.dim[1] = self.si.dim[2] = 1
        self.st = settings_t()
        self.st.dimension = dim
        self.st.numberoffields = len(fields)
        self.st.gfh = gfh
        self.st.gfdt = gfdt
        self.st.secondsperstep = secondsperstep
        self.st.step = step
        (gx, gy, gz), lower = grid_geometry(dim, gfh)
        self.gsize = (gx, gy, gz)
        g = grid_t()
        g.resolution = gfh
        g.lowercorner.x, g.lowercorner.y, g.lowercorner.z = lower
        g.localsize.x, g.localsize.y, g.localsize.z = gx, gy, gz
        g.globalsize.x, g.globalsize.y, g.globalsize.z = gx, gy, (gz if dim == 3 else 0)
        self.grid = g
        self.envs = (environment_t * len(fields))()
        for e, f in zip(self.envs, fields):
            e.diffusioncoefficient = f["dc"]
            e.boundarycondition = f["bc"]
            e.initialconditionmean = f["mean"]
            e.initialconditionvariance = f.get("variance", 0.0)
            e.lambdadelay = f.get("lam", 0.0)
        self.penv = C.cast(self.envs, C.POINTER(environment_t))
        self.lib.environment_allocate(self.si, self.st, self.grid, C.byref(self.penv), None, None)
        self.lib.environment_init(self.si, self.st, self.grid, C.byref(self.penv))
        self.lib.environment_initsystem(self.si, self.st, C.byref(self.grid), C.byref(self.penv), None, None)

    def compute(self, writeback: bool = False):
        self.lib.tm_dropin_set_env_writeback(1 if writeback else 0)
        self.lib.environment_compute(self.si, self.st, C.byref(self.grid), C.byref(self.penv), None, None)

    def data(self, f: int) -> np.ndarray:
        n = int(np.prod(self.gsize))
        return np.ctypeslib.as_array(C.cast(self.envs[f].data, C.POINTER(C.c_double)), shape=(n,)).reshape(
            self.gsize).copy()

    def solution(self, f: int) -> np.ndarray:
        out = np.zeros(self.gsize)
        rc = self.lib.tm_dropin_env_solution(f, out.ctypes.data)
        if rc:
            raise RuntimeError(f"tm_dropin_env_solution: {rc}")
        return out

    def close(self):
        libc = C.CDLL(None)
        libc.free.argtypes = [C.c_void_p]
        for e in self.envs:
            for k in ("data", "production", "gradient"):
                if getattr(e, k):
                    libc.free(getattr(e, k))
                    setattr(e, k, None)
        self.lib.tm_dropin_set_env_writeback(0)
        self.lib.tm_dropin_shutdown()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
