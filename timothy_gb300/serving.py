"""Serving form: a request loop over one device-resident session.

A request is a colony simulation: cells plus a number of steps.  The server
holds one session whose slot pool is sized at start-up from the device's free
HBM (``tm_device_memory`` and ``tm_session_bytes``).  Requests queue in
arrival order and are admitted while the pool has room for their cells (slot
range, bin table, colony entry); an admitted colony stays resident until its
last step.  Every engine iteration advances all resident colonies one step in
the same launches, so a colony admitted now steps alongside colonies that are
part-way through theirs (continuous batching).  After its last step a colony's
results are queued for download into page-locked buffers and the colony is
removed, which frees room for the queue at once.

The host keeps one step ahead of the device: admissions
(``tm_colony_add_async``), retirements and the next step are queued behind
the step in flight, and the host then waits only for the fence of the step
before (``tm_session_fence``/``tm_session_wait``), when that step's retired
results have reached the host.  The device never waits for the host's
bookkeeping, and a request's latency ends when its results are on the host.

Because a colony's results do not depend on what else is resident (per-colony
frames, bins, lists; groups aligned to the colony's first slot), a request
gives the same result alone and in the mix.
"""
from __future__ import annotations

import math
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from . import colonies as C

ENOMEM = -2


@dataclass
class Request:
    rid: int
    kind: str
    n: int
    steps: int
    arrival: float                      # seconds after the start (or engine iteration, virtual clock)
    seed: int = 0
    colony: C.Colony | None = None      # cells; built on admission when None
    stage: dict | None = field(default=None, repr=False)   # page-locked positions the colony's cells use
    admitted: float = math.nan
    finished: float = math.nan
    result: dict | None = field(default=None, repr=False)

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


class RequestSource:
    """Colonies for requests, cut from two pre-generated template colonies.

    A request for n cells of a kind takes n consecutive cells of that kind's
    template (independent draws, so any n of them are a sample of the same
    shape) at a seed-chosen offset and shrinks their positions by
    (n / N_template)^(1/3), which keeps the cell density of a colony drawn
    directly with n cells.  This keeps the client's cost per request to a few
    array operations.
    """

    def __init__(self, n_template: int = 1_000_000, seed: int = 7, types: C.CellTypes | None = None):
        self.n_template = n_template
        self.types = types or C.CellTypes.consistent()
        self.templates = {k: C.make_colony(k, n_template, seed + i, C.initial_radius(k, n_template), types=self.types)
                          for i, k in enumerate(("uniform", "clustered"))}

    def colony(self, kind: str, n: int, seed: int, xyz=None) -> C.Colony:
        """The request's cells; with ``xyz`` (three float64 arrays of at least
        n entries) the positions are written into those arrays."""
        t = self.templates[kind]
        n = int(min(n, self.n_template))
        off = int(np.random.Generator(np.random.PCG64(seed)).integers(0, self.n_template - n + 1))
        f = (n / self.n_template) ** (1.0 / 3.0)
        sl = slice(off, off + n)
        if xyz is None:
            pos = [t.x[sl] * f, t.y[sl] * f, t.z[sl] * f]
        else:
            pos = [np.multiply(src[sl], f, out=dst[:n]) for src, dst in zip((t.x, t.y, t.z), xyz)]
        return C.Colony(pos[0], pos[1], pos[2], t.size[sl], t.young[sl], t.ctype[sl], t.phase[sl],
                        self.types, t.dim, kind, seed, t.radius * f)

    def template_arrays(self) -> list:
        """The templates' per-cell arrays that requests take slices of."""
        return [getattr(t, k) for t in self.templates.values() for k in ("size", "young", "ctype", "phase")]


def poisson_requests(rate: float, duration: float, *, seed: int = 7, lo: int = 1000, hi: int = 1_000_000,
                     steps=(10, 50, 200)) -> list[Request]:
    """Arrivals of a Poisson stream over [0, duration): cell counts log-uniform in
    [lo, hi], uniform or clustered with equal probability, steps uniform over ``steps``."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out, t, rid = [], 0.0, 0
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            break
        n = int(math.floor(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        kind = "clustered" if rng.integers(0, 2) else "uniform"
        k = int(steps[int(rng.integers(0, len(steps)))])
        out.append(Request(rid, kind, n, k, t, seed=10_000 + rid))
        rid += 1
    return out


class Server:
    """Continuous-batching server over one session (see the module docstring)."""

    def __init__(self, types: C.CellTypes | None = None, *, precision: str = "fp32c", dt: float = 0.01,
                 hbm_fraction: float = 0.6, max_slots: int | None = None, max_colonies: int = 2048,
                 list_capacity: int = 384, device: int = 0, graph: bool = True, tuning: dict | None = None,
                 fields=("x", "y", "z", "density", "fx", "fy", "fz"), keep_results: bool = False,
                 prepare_ahead: int = 16):
        from .session import Session, device_memory, session_bytes

        self.types = types or C.CellTypes.consistent()
        self.precision, self.dt, self.fields, self.keep = precision, dt, list(fields), keep_results
        self.prepare_ahead = prepare_ahead
        bins_per_slot = 8

        def nbytes(slots):
            return session_bytes(max_slots=slots, max_colonies=max_colonies, ntypes=self.types.ntypes,
                                 max_bin_entries=bins_per_slot * slots + (1 << 24), list_capacity=list_capacity)

        free, total = device_memory(device)
        if max_slots is None:
            budget = hbm_fraction * free
            lo, hi = 1 << 15, 1 << 31
            while hi - lo > 1 << 14:            # largest pool that fits the budget
                mid = (lo + hi) // 2
                lo, hi = (mid, hi) if nbytes(mid) <= budget else (lo, mid)
            max_slots = lo
        self.max_slots = int(max_slots)
        self.pool_bytes = nbytes(self.max_slots)
        self.hbm_free_at_start, self.hbm_total = free, total
        self.s = Session(self.types, max_slots=self.max_slots, max_colonies=max_colonies, device=device,
                         max_bin_entries=bins_per_slot * self.max_slots + (1 << 24), list_capacity=list_capacity)
        if tuning:
            self.s.set_tuning(**tuning)
        self.s.use_graph(graph)
        self._free_bufs: list[dict] = []
        self._all_bufs: list[dict] = []
        # page-locked positions for the cells of requests being admitted (an
        # upload from pageable memory stages through the driver and holds the
        # host for the copy: it was most of the host loop's time)
        self._free_stage: list[dict] = []
        self._all_stage: list[dict] = []
        self._pinned_sources: list = []

    def close(self):
        from .session import host_unregister

        self.s.close()
        for b in self._all_bufs + self._all_stage:
            for a in b.values():
                host_unregister(a)
        for a in self._pinned_sources:
            host_unregister(a)
        self._all_bufs, self._free_bufs, self._all_stage, self._free_stage = [], [], [], []
        self._pinned_sources = []

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _stage(self, n: int) -> dict:
        """Page-locked position arrays for one request's cells (reused)."""
        from .session import host_register

        for k, b in enumerate(self._free_stage):
            if len(b["x"]) >= n:
                return self._free_stage.pop(k)
        cap = max(n, 1 << 16)
        b = {k: np.zeros(cap) for k in ("x", "y", "z")}
        for a in b.values():
            host_register(a)
        self._all_stage.append(b)
        return b

    def _prepare(self, req: Request, source: RequestSource):
        """Build the request's cells (into page-locked staging unless results are kept)."""
        if self.keep:
            req.colony = source.colony(req.kind, req.n, req.seed)
            return
        if not self._pinned_sources:
            from .session import TimothyError, host_register

            # the templates' other fields are sliced, not copied: lock them once
            for a in source.template_arrays():
                if a.flags.c_contiguous and not any(a is b for b in self._pinned_sources):
                    try:
                        host_register(a)
                    except TimothyError:     # locked already (another server): the copies still work
                        continue
                    self._pinned_sources.append(a)
        req.stage = self._stage(req.n)
        req.colony = source.colony(req.kind, req.n, req.seed, (req.stage["x"], req.stage["y"], req.stage["z"]))

    def _admit(self, req: Request, source: RequestSource | None) -> int | None:
        from .session import TimothyError

        if req.colony is None:
            self._prepare(req, source)
        try:
            # queued behind the step in flight (tm_colony_add_async)
            return self.s.add_colony(req.colony, precision=self.precision, update="dt", dt=self.dt, verlet=True,
                                     wait=False)
        except TimothyError as e:
            if e.code == ENOMEM:
                return None
            raise

    def _buffers(self, n: int) -> dict:
        """Page-locked host arrays for one finished colony's results (reused)."""
        from .session import host_register

        for k, b in enumerate(self._free_bufs):
            if len(b[self.fields[0]]) >= n:
                return self._free_bufs.pop(k)
        cap = max(n, 1 << 16)
        b = {f: np.zeros(cap, np.uint8 if f == "removecell" else np.float64) for f in self.fields}
        for a in b.values():
            host_register(a)
        self._all_bufs.append(b)
        return b

    def run(self, requests: list[Request], *, source: RequestSource | None = None, virtual: bool = False,
            horizon: float | None = None, drain: bool = False, admit_window: int = 32, log=None) -> dict:
        """Serve ``requests`` (sorted by arrival).  With ``virtual`` the clock is
        the engine iteration (deterministic mixes for tests); otherwise wall time
        in seconds.  With ``horizon`` the run stops at that time, leaving later
        arrivals and unfinished colonies out; with ``drain`` as well, arrivals
        stop at the horizon and the run goes on until every request that
        arrived before it has finished, so the latencies cover all of them.
        Admission takes queued requests in arrival order, and looks past one
        that does not fit (too many cells for the free slots) at most
        ``admit_window`` places, so a large request waits for room while
        smaller ones behind it start."""
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        queue: deque[Request] = deque()
        active: dict[int, list] = {}
        # steps queued on the device whose fence the host has not waited for,
        # with the colonies each retired (their results travelling back) and
        # the staging of the colonies admitted before it (free once it is done)
        inflight: deque[tuple[int, list, list]] = deque()
        lag = 1
        s = self.s
        t0 = time.perf_counter()
        it = 0
        stepped_cells = 0
        resident_max = 0
        clock = (lambda: float(it)) if virtual else (lambda: time.perf_counter() - t0)
        if drain and horizon is not None:
            pending = deque(r for r in pending if r.arrival < horizon)
        stepped_at_horizon = None
        while pending or queue or active or inflight:
            now = clock()
            if horizon is not None and now >= horizon and stepped_at_horizon is None:
                stepped_at_horizon = stepped_cells
            if horizon is not None and now >= horizon and not drain:
                break
            while pending and pending[0].arrival <= now:
                queue.append(pending.popleft())
            # admission in arrival order, looking past requests that do not fit
            k = 0
            admitted = []
            while k < min(len(queue), admit_window):
                cid = self._admit(queue[k], source)
                if cid is None:
                    k += 1
                    continue
                req = queue[k]
                del queue[k]
                req.admitted = clock()
                active[cid] = [req, req.steps]
                admitted.append(req)
            if active:
                resident_max = max(resident_max, sum(r.n for r, _ in active.values()))
                s.step(1)
                it += 1
                stepped_cells += sum(r.n for r, _ in active.values())
                # the step runs on the device: meanwhile build the cells of the
                # requests that wait, so their admission costs only the upload
                if source is not None:
                    for req in list(queue)[:self.prepare_ahead]:
                        if req.colony is None:
                            self._prepare(req, source)
                retiring = []
                for cid in [c for c, e in active.items() if e[1] == 1]:
                    req = active.pop(cid)[0]
                    bufs = self._buffers(req.n)
                    s.download_async(cid, self.fields, bufs)
                    s.remove_colony(cid)            # queued behind the download's gathers
                    retiring.append((req, bufs))
                for e in active.values():
                    e[1] -= 1
                inflight.append((s.fence(), retiring, admitted))
            elif not inflight:
                if virtual:
                    it += 1
                elif pending:
                    time.sleep(max(0.0, min(pending[0].arrival - clock(), 0.005)))
                continue
            # stay at most `lag` steps ahead of the device; settle everything
            # when nothing more is queued
            while inflight and (len(inflight) > lag or not active):
                f, retiring, admitted_then = inflight.popleft()
                s.wait(f)
                t = clock()
                for req in admitted_then:           # their uploads are done
                    if req.stage is not None:
                        self._free_stage.append(req.stage)
                        req.stage = None
                for req, bufs in retiring:
                    req.finished = t
                    out = {k: bufs[k][:req.n].copy() for k in self.fields} if self.keep else None
                    req.result = out if self.keep else {"density_sum": float(np.sum(bufs["density"][:req.n]))
                                                        if "density" in bufs else None}
                    req.colony = None if not self.keep else req.colony
                    self._free_bufs.append(bufs)
                    if log:
                        log(f"t={req.finished:.3f} done rid={req.rid} n={req.n} K={req.steps} lat={req.latency:.3f}")
        s.sync()
        wall = clock() if not virtual else time.perf_counter() - t0
        if stepped_at_horizon is None and horizon:
            # every request finished before the horizon: the whole run was arrivals
            horizon_used = max(wall, 1e-9)
            stepped_at_horizon = stepped_cells
        else:
            horizon_used = horizon
        arrived = [r for r in requests if horizon is None or r.arrival < horizon]
        fin = [r for r in requests if not math.isnan(r.finished)]
        lat = np.array([r.latency for r in fin]) if fin else np.zeros(0)
        served = sum(r.n * r.steps for r in fin)
        return {"requests": len(requests), "arrived": len(arrived), "finished": len(fin), "wall_s": wall,
                "iterations": it,
                "throughput_during_arrivals": (stepped_at_horizon / horizon_used
                                               if stepped_at_horizon is not None and horizon else None),
                "cell_updates_finished": served, "cell_updates_stepped": stepped_cells,
                "throughput": stepped_cells / wall if wall > 0 else 0.0,
                "p50": float(np.percentile(lat, 50)) if len(lat) else None,
                "p99": float(np.percentile(lat, 99)) if len(lat) else None,
                "max_resident_cells": resident_max, "pool_slots": self.max_slots, "pool_bytes": self.pool_bytes}


def run_alone(colony: C.Colony, steps: int, *, precision: str = "fp32c", dt: float = 0.01, list_capacity: int = 384,
              tuning: dict | None = None, fields=("x", "y", "z", "density", "fx", "fy", "fz"), device: int = 0) -> dict:
    """The same simulation in a session of its own (the invariance reference)."""
    from .session import Session

    with Session(colony.types, dim=colony.dim, max_slots=colony.n + 64, device=device,
                 list_capacity=list_capacity) as s:
        if tuning:
            s.set_tuning(**tuning)
        cid = s.add_colony(colony, precision=precision, update="dt", dt=dt, verlet=True)
        s.step(steps)
        s.sync()
        return s.download(cid, list(fields))
