"""Batched form: hundreds of independent colonies of uneven size advanced together.

All colonies live in one session, each in its own 32-aligned slot range with
its own frame (affine map, bin level), bin table and neighbour lists.  Every
kernel of a step covers all colonies in one launch; the step's launches are
captured in one CUDA graph and replayed; the search kernel is persistent
(grid-stride over the 8-cell groups of all colonies, sized to the resident
blocks).  Launch shapes and the list skin come from the autotuner.

A colony's results do not depend on its neighbours in the batch: every
reduction, sort and list is per colony and the groups of the pair kernels are
aligned to the colony's first slot, so a colony gives the same bits alone and
in any mix (the CIC grid, accumulated with atomics, to rounding).
"""
from __future__ import annotations

import math
import time

import numpy as np

from . import colonies as C


def make_batch(count: int = 512, seed: int = 4, lo: int = 1000, hi: int = 200_000, first_seed: int = 1000,
               types: C.CellTypes | None = None) -> list[C.Colony]:
    """``count`` colonies, cell counts log-uniform in [lo, hi], uniform or clustered
    with equal probability; colony i uses seed first_seed + i and the radius that
    gives about 40 neighbours within h in the bulk."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sizes = np.floor(np.exp(rng.uniform(math.log(lo), math.log(hi), size=count))).astype(np.int64)
    kinds = rng.integers(0, 2, size=count)
    out = []
    for i in range(count):
        kind = "clustered" if kinds[i] else "uniform"
        n = int(sizes[i])
        out.append(C.make_colony(kind, n, first_seed + i, C.initial_radius(kind, n), types=types))
    return out


def bins_needed(col: C.Colony) -> int:
    """Bin-table entries a colony takes (the session's bin level rule, 8^L + 2)."""
    if col.n <= 1:
        return 8 + 2
    ext = max(float(np.ptp(col.x)), float(np.ptp(col.y)), float(np.ptp(col.z)))
    hmax = float(np.max(col.types.h))
    ext += 2.0 * (hmax + 0.01)
    L = max(1, min(8, int(math.floor(math.log2(2.0 * ext / hmax)))))
    return (1 << (3 * L)) + 2


def open_session(colonies, *, precision="fp32c", list_capacity: int = 384, device: int = 0, diagnostics=False,
                 extra_slots: int = 0, extra_colonies: int = 0, extra_bins: int = 0):
    """A session sized for ``colonies`` (plus optional room for more)."""
    from .session import Session

    types = colonies[0].types
    slots = sum(((c.n + 31) // 32) * 32 for c in colonies) + extra_slots
    bins = sum(bins_needed(c) for c in colonies) + extra_bins + 16
    return Session(types, dim=colonies[0].dim, max_slots=slots + 32, max_colonies=len(colonies) + extra_colonies,
                   device=device, diagnostics=diagnostics, max_bin_entries=bins, list_capacity=list_capacity)


def add_all(s, colonies, *, precision="fp32c", update="dt", dt=0.01, cic=False, verlet=True) -> list[int]:
    return [s.add_colony(c, precision=precision, update=update, dt=dt, cic=cic, verlet=verlet) for c in colonies]


def run_batch(colonies, steps: int, *, precision: str = "fp32c", dt: float = 0.01, warmup: int = 3,
              tune: bool = True, tuning: dict | None = None, graph: bool = True, list_capacity: int = 384,
              device: int = 0, fields=None, log=None) -> dict:
    """Advance every colony ``steps`` steps in one session; returns timings and,
    if ``fields`` is given, each colony's results (caller order)."""
    from . import autotune as AT

    total = sum(c.n for c in colonies)
    info = {"colonies": len(colonies), "cells": total, "precision": precision, "steps": steps, "warmup": warmup}
    with open_session(colonies, precision=precision, list_capacity=list_capacity, device=device) as s:
        t0 = time.time()
        ids = add_all(s, colonies, precision=precision, dt=dt)
        s.sync()
        info["upload_s"] = time.time() - t0
        if tuning:
            s.set_tuning(**tuning)
        elif tune:
            res = AT.autotune(s, log=log)
            info["tune_s"] = res["seconds"]
            info["tune_trials"] = res["trials"]
            # fresh state for the measured run
            for cid in ids:
                s.remove_colony(cid)
            ids = add_all(s, colonies, precision=precision, dt=dt)
        info["tuning"] = s.tuning
        s.use_graph(graph)
        s.step(warmup)
        s.sync()
        rate0, rb0 = s.list_rate()
        l0 = s.launches
        s.timer_start()
        s.step(steps)
        ms = s.timer_stop()
        info["gpu_launches"] = s.launches - l0
        _, rb1 = s.list_rate()
        info["rebuilds"] = rb1 - rb0
        info["ms"] = ms
        info["ms_per_step"] = ms / steps
        info["value"] = total * steps / (ms * 1e-3)
        if fields:
            info["results"] = [s.download(cid, fields) for cid in ids]
    return info
