#!/usr/bin/env python
"""Benchmark of the Timothy cell-mechanics hot path on GB300.

Prints ONE JSON line (rank 0).  Metric: cell-updates/s, where one cell-update
is one cell advanced by one full step of the path (neighbour search + SPH
density/potential + force + FP64 position update; plus the CIC deposit for the
workload that has it).

Workloads (seeded synthetic colonies; the reference ships no datasets):
  precision16m  16,000,000 cells, clustered spheroid (seed 3), FP32 +
                compensated path; the plain FP64 path runs on the same colony
                and GPU for the ratio and the error report.  Default.
  scale1m       1,000,000 cells, clustered spheroid (seed 2), plain FP64 path
                with a CIC deposit onto a 257^3 FP64 grid each step.
  uniform10k    10,000 cells uniform in a ball (seed 1), plain FP64 path.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload precision16m|scale1m|uniform10k] [--no-forms]

The line also carries the two other forms ("forms"): the batched form (512
colonies of 1e3..2e5 cells, autotuned, one step graph per step, FP32+comp and
FP64) and the serving form (Poisson request streams at the given rates for a
bounded time; offered and served cell-updates/s, p50/p99 latency).
Under torchrun each rank runs an independent replica (the path has no
cross-colony exchange), so scaling is weak and value is the total over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from timothy_gb300 import colonies as C  # noqa: E402

METRIC = "cell-updates/s at 16M cells (FP64 vs FP32+comp, same GPU); p50/p99 latency"
UNIT = "cell-updates/s"
# Algorithmic bytes per cell-update: reads x,y,z,size (4x8) + young (4) + ctype (4);
# writes density, v, mindist, Fx, Fy, Fz, x, y, z (9x8).  The CIC workload adds
# the phase (4) per cell and one write of the grid per step.
B_CELL = 112
# DRAM bytes per cell of one list-pass launch (dram__bytes_read.sum +
# dram__bytes_write.sum over the cells of the launch), from the ncu capture
# summarised in profiles/k_plist32_fp32_clustered2m.txt; traffic grows with the
# cell count, so a launch over n cells moves n times this.
TRAFFIC_PER_CELL = {"k_plist32": 370.3}
WORKLOADS = {
    "precision16m": dict(kind="clustered", n=16_000_000, seed=3, precision="fp32c", cic=False, dt=0.01),
    "scale1m": dict(kind="clustered", n=1_000_000, seed=2, precision="fp64", cic=True, dt=0.01),
    "uniform10k": dict(kind="uniform", n=10_000, seed=1, precision="fp64", cic=False, dt=0.01),
}


def radius_for(kind, n, seed):
    """Calibrated radius, or the calibrated one of the same generator scaled by n^(1/3)."""
    return C.configured_radius(kind, n, seed)


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=2)
        except Exception:
            self.proc.kill()
        rows = self.rows
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, nm in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(rows),
                "power_w_max": max(float(r[3]) for r in rows if r[3].replace(".", "").isdigit())
                if any(r[3].replace(".", "").isdigit() for r in rows) else None}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist

        backend = "nccl"
        try:
            import torch

            torch.cuda.set_device(local)
        except Exception:
            backend = "gloo"
        dist.init_process_group(backend=backend)
        pg = dist
    return world, rank, local, pg


def dist_max(pg, value: float) -> float:
    if pg is None:
        return value
    import torch

    dev = "cuda" if pg.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def aggregate_value(n, world, steps, ms_max):
    """Whole-job cell-updates/s: every replica's cells over the slowest rank's time."""
    return n * world * steps / (ms_max * 1e-3)


def dist_barrier(pg):
    if pg is not None:
        pg.barrier()


def cpu_colony(workload, n_cap=1_000_000):
    """A sample of the workload: n_cap cells of the same generator and seed,
    the radius scaled so that the mean neighbour count stays 40."""
    kind, seed = workload["kind"], workload["seed"]
    n = min(workload["n"], n_cap)
    return C.make_colony(kind, n, seed, radius_for(kind, n, seed))


def cpu_sample(workload, threads=0, col=None):
    """Time the CPU implementation of the path (the reference compiled here, or
    the oracle port) for one step on a bounded sample of the workload."""
    from oracle import bindings

    col = col if col is not None else cpu_colony(workload)
    which = "ref" if bindings.available("ref") else "oracle"
    try:
        bindings.load(which)
    except OSError:
        which = "oracle"
    if which == "oracle" and not bindings.available("oracle"):
        bindings.build(ref=False)
    threads = threads or os.cpu_count() or 1
    steps = 1
    kw = dict(which=which, update_mode=1, dt=workload["dt"], cic=workload["cic"])
    if which == "oracle":
        kw["nthreads"] = threads
    else:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    t0 = time.perf_counter()
    bindings.run(col, steps, **kw)
    dt = time.perf_counter() - t0
    return {"value": col.n * steps / dt, "unit": UNIT, "cores": threads,
            "kind": "reference" if which == "ref" else "port",
            "sample": f"{col.n} cells of the {col.kind} generator (seed {col.seed}), {steps} step, {dt:.2f} s"}


def run_reference_arm(args, workload, budget_s=200.0):
    """CPU path of the reference on the host cores, one bounded sample per step:
    the largest sample of the workload (cells of the same generator, up to
    the whole colony) that keeps the whole run near budget_s."""
    world, rank, local, pg = dist_setup()
    if rank != 0:
        return
    probe = cpu_sample(workload, col=cpu_colony(workload, 200_000))
    per_step = budget_s / max(1, args.steps + args.warmup)
    n = int(max(20_000, min(workload["n"], probe["value"] * per_step)))
    col = cpu_colony(workload, n)
    samples = []
    cb = None
    for _ in range(args.warmup):
        cpu_sample(workload, col=col)
    for _ in range(args.steps):
        cb = cpu_sample(workload, col=col)
        samples.append(cb["value"])
    value = float(np.mean(samples))
    cb["value"] = value
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": col.n / value * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": args.workload, **{k: workload[k] for k in ("kind", "n", "seed")},
                       "sample_cells": col.n,
                       "sample": f"{col.n} of the {workload['n']} cells per step (same generator and density)"},
            "cpu_baseline": cb, "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                                        "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def batched_form(args, device, log=None):
    """512 colonies (log-uniform 1e3..2e5 cells, uniform or clustered, seeds
    1000+i), autotuned, 50 steps per step-graph; FP32+comp, then FP64."""
    from timothy_gb300 import batch as B

    t0 = time.time()
    cols = B.make_batch(args.batch_colonies, seed=4)
    gen_s = time.time() - t0
    out = {"colonies": len(cols), "cells": int(sum(c.n for c in cols)), "steps": args.batch_steps,
           "generate_s": gen_s}
    for prec in ("fp32c", "fp64"):
        info = B.run_batch(cols, args.batch_steps, precision=prec, warmup=3, tune=True, device=device, log=log)
        out[prec] = {"value": info["value"], "ms_per_step": info["ms_per_step"], "tuning": info["tuning"],
                     "tune_s": round(info.get("tune_s", 0.0), 2), "rebuilds": info["rebuilds"],
                     "gpu_launches_per_step": info["gpu_launches"] / args.batch_steps,
                     "graph": True}
    out["fp32c_over_fp64"] = out["fp32c"]["value"] / out["fp64"]["value"]
    return out


def serving_form(args, device, rate, seconds):
    """Poisson requests (log-uniform 1e3..1e6 cells, uniform or clustered, K in
    {10, 50, 200}, FP32+comp) for ``seconds``; stops at the horizon."""
    from timothy_gb300 import serving as SV

    src = SV.RequestSource(n_template=1_000_000, seed=7)
    reqs = SV.poisson_requests(rate, seconds, seed=7)
    offered = sum(r.n * r.steps for r in reqs) / seconds
    with SV.Server(device=device, hbm_fraction=0.5) as srv:
        # arrivals for `seconds`, then the queue drains: every request's
        # latency is counted, none is left out for being unfinished
        st = srv.run(reqs, source=src, horizon=seconds, drain=True)
    fin = [r for r in reqs if r.finished == r.finished]
    return {"rate_per_s": rate, "arrival_seconds": seconds, "wall_s": st["wall_s"], "requests": len(reqs),
            "finished": st["finished"], "offered_cell_updates_per_s": offered,
            "served_cell_updates_per_s": st["throughput"],
            "served_while_arriving_cell_updates_per_s": st["throughput_during_arrivals"],
            "p50_s": st["p50"], "p99_s": st["p99"],
            "latency_over": "every request (arrivals stop at arrival_seconds, then the queue drains)",
            "p50_by_size": _size_bins(fin), "max_resident_cells": st["max_resident_cells"],
            "pool_slots": st["pool_slots"], "pool_gb": st["pool_bytes"] / 1e9}


def field_rows(device, peak, steps=10):
    """The grid -> cell gather and the field gradient on the scale1m layout:
    1,000,000 clustered cells (seed 2) and one field on the 257^3 FP64 grid of
    GFH 8.  Each launch is timed alone with CUDA events after a write of 256 MB
    (flushes L2); achieved bandwidth counts the algorithmic bytes."""
    import torch

    from oracle import bindings as OB
    from timothy_gb300 import session as S

    torch.cuda.set_device(device)
    n, gfh, nf = 1_000_000, 8.0, 1
    col = C.make_colony("clustered", n, 2, radius_for("clustered", n, 2))
    dims = OB.grid_dims(3, gfh)
    G = int(np.prod(dims))
    rng = np.random.Generator(np.random.PCG64(5))
    data = torch.from_numpy(rng.random((nf,) + dims)).cuda()
    grad = torch.zeros((nf,) + dims + (3,), dtype=torch.float64, device="cuda")
    xs = [torch.from_numpy(np.ascontiguousarray(getattr(col, k))).cuda() for k in ("x", "y", "z")]
    out = torch.zeros((nf, n, 4), dtype=torch.float64, device="cuda")
    flush = torch.empty(32 * 1024 * 1024, dtype=torch.float64, device="cuda")
    lower = (-1024.0, -1024.0, -1024.0)

    def timed(fn):
        for _ in range(3):
            fn()
        ms = []
        for _ in range(steps):
            flush.fill_(1.0)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
        return float(np.mean(ms))

    ms_g = timed(lambda: S.field_gradient_device(data, dims, gfh, nf, grad))
    ms_e = timed(lambda: S.env2cells_device(*xs, n, 3, lower, gfh, dims, nf, data, grad, out))
    # grid nodes the cells touch (each read once: its value and 3 gradient components)
    ci = [np.floor((getattr(col, k) + 1024.0) / gfh).astype(np.int64) for k in ("x", "y", "z")]
    keys = []
    for ax in (0, 1):
        for ay in (0, 1):
            for az in (0, 1):
                keys.append(((ci[0] + ax) * dims[1] + ci[1] + ay) * dims[2] + ci[2] + az)
    touched = int(np.unique(np.concatenate(keys)).size)
    b_g = 32 * G * nf                              # read u, write 3 components
    b_e = n * (24 + 32 * nf) + touched * 32 * nf   # positions in, cellenvdata out, touched nodes in
    return {"config": "1,000,000 clustered cells (seed 2), 257^3 FP64 grid (GFH 8), 1 field; L2 flushed",
            "field_gradient": {"ms": ms_g, "bytes": b_g, "achieved_gbs": b_g / ms_g / 1e6,
                               "frac_of_measured_hbm": b_g / ms_g / 1e6 / peak},
            "env2cells": {"ms": ms_e, "bytes": b_e, "touched_nodes": touched, "achieved_gbs": b_e / ms_e / 1e6,
                          "frac_of_measured_hbm": b_e / ms_e / 1e6 / peak,
                          "cell_gathers_per_s": n / (ms_e * 1e-3)}}


def cic_rows(device, peak, steps=10):
    """The CIC deposit (patches_alloc + patches_cells2envinfo) on the 1,000,000
    clustered cells of the scale1m workload (seed 2) onto the 257^3 FP64 grid
    of GFH 8: inside a session step (the deposit phase of an FP32 + compensated
    step, CUDA events) and through the allocation-free entry point on device
    arrays (L2 flushed before each call).  Algorithmic bytes: the cells'
    positions and phases in (28 B/cell) and one write of the grid."""
    import ctypes

    import torch

    from oracle import bindings as OB
    from timothy_gb300 import session as S

    torch.cuda.set_device(device)
    n, gfh = 1_000_000, 8.0
    col = C.make_colony("clustered", n, 2, radius_for("clustered", n, 2))
    dims = OB.grid_dims(3, gfh)
    G = int(np.prod(dims))
    bytes_ = n * 28 + G * 8
    out = {"config": "1,000,000 clustered cells (seed 2), 257^3 FP64 grid (GFH 8)", "bytes": bytes_}
    with S.Session(col.types, dim=3, max_slots=n + 64, list_capacity=384, device=device) as s:
        s.add_colony(col, precision="fp32c", update="dt", dt=0.01, cic=True, gfh=gfh, verlet=True)
        s.step(3)
        s.sync()
        s.profile(True)
        s.step(steps)
        s.sync()
        prof = s.profile_read()
        s.profile(False)
    ms = prof["cic_ms"]
    out["in_step"] = {"ms": ms, "achieved_gbs": bytes_ / ms / 1e6, "frac_of_measured_hbm": bytes_ / ms / 1e6 / peak}
    lib = S.load_library()
    fn = lib.tm_cic_deposit_noalloc
    P = ctypes.c_void_p
    fn.restype = ctypes.c_int
    fn.argtypes = [P, P, P, P, ctypes.c_int64, ctypes.c_int, P, ctypes.c_float, P, P, P, P]
    xs = [torch.from_numpy(np.ascontiguousarray(getattr(col, k))).cuda() for k in ("x", "y", "z")]
    ph = torch.from_numpy(np.ascontiguousarray(col.phase, np.int32)).cuda()
    grid = torch.zeros(G, dtype=torch.float64, device="cuda")
    corners = torch.zeros(6, dtype=torch.int64, device="cuda")
    lower = np.array([-1024.0, -1024.0, -1024.0])
    gs = np.array(dims, np.int64)
    flush = torch.empty(32 * 1024 * 1024, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream

    def call():
        rc = fn(xs[0].data_ptr(), xs[1].data_ptr(), xs[2].data_ptr(), ph.data_ptr(), n, 3, lower.ctypes.data, gfh,
                gs.ctypes.data, grid.data_ptr(), corners.data_ptr(), stream)
        if rc:
            raise RuntimeError(f"tm_cic_deposit_noalloc: {rc}")

    for _ in range(3):
        call()
    ts = []
    for _ in range(steps):
        flush.fill_(1.0)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        call()
        b.record()
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b))
    ms2 = float(np.mean(ts))
    out["noalloc_call"] = {"ms": ms2, "achieved_gbs": bytes_ / ms2 / 1e6,
                           "frac_of_measured_hbm": bytes_ / ms2 / 1e6 / peak}
    return out


def diffusion_rows(device, steps=3):
    """The implicit diffusion step (environment_compute) on the 257^3 FP64 grid
    of GFH 8, one field, from the reference's start (the mean) with its point
    source: with the reference's sample parameters (DC 1.82e-5, SECPERSTEP =
    GFDT = 16000: z = 4.6e-3, one solve per step) and with DC 2.0 (z = 500, a
    stiff operator: the multigrid preconditioner).  Each step is timed with
    CUDA events on the default stream (it waits for each iteration's norm)."""
    import torch

    from timothy_gb300 import session as S

    torch.cuda.set_device(device)
    gs = (257, 257, 257)
    src = torch.zeros((1,) + gs, dtype=torch.float64, device="cuda")
    src[0, 5, 5, 5] = 100.0
    out = {"config": "257^3 FP64 grid (GFH 8), 1 field, mean 0.1575e-6, BC 0.1575e-6, point source 100 at "
                     "(5,5,5), SECPERSTEP = GFDT = 16000, tolerance 1e-12 (the reference's)"}
    with S.Diffusion(gs, device=device) as d:
        for name, dc in (("reference_parameters", 1.82e-5), ("stiff_dc2", 2.0)):
            ms, st = [], None
            for k in range(steps + 1):
                u = torch.full((1,) + gs, 0.1575e-6, dtype=torch.float64, device="cuda")
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record()
                st = d.step(u, 8.0, [dc], [0.1575e-6], [0.0], 16000.0, 16000.0, source=src, tol=1e-12)
                b.record()
                torch.cuda.synchronize()
                if k:
                    ms.append(a.elapsed_time(b))
            out[name] = {"ms_per_step": float(np.mean(ms)), "nodes_per_s": float(np.prod(gs)) / (np.mean(ms) * 1e-3),
                         "z": dc * 16000.0 / 64.0, **st}
    return out


def cycle_rows(device, reps=5):
    """The cell cycle with mitosis (tm_colony_cellcycle) and the removal that
    follows (tm_colony_compact) on a resident colony of 1,000,000 clustered
    cells (seed 2): phases G0/G1/S/G2/M with probabilities .1/.4/.25/.21/.04,
    phase times uniform in [0, 12) h, lengths 11/8/4/1 h, death probability
    0.1, one step of 3600 s, so that the M cells (4 %) divide and about 2 %
    die; wall time per call (each waits for its draw counts).  The draws come
    from the C library's stream, generated on the device or, for comparison,
    by calling rand() on the host."""
    import dataclasses
    import time

    from timothy_gb300 import session as S

    n = 1_000_000
    col = C.make_colony("clustered", n, 2, radius_for("clustered", n, 2))
    rng = np.random.Generator(np.random.PCG64(9))
    rng2 = np.random.Generator(np.random.PCG64(10))
    types = {"g1": [11.0], "s": [8.0], "g2": [4.0], "m": [1.0], "v": [0.2], "rd": [0.1], "cd": [1e9]}
    t_cyc, t_cmp, t_libc, divided, marked = [], [], [], [], []
    with S.Session(col.types, dim=3, max_slots=3 * n, device=device) as s:
        for k in range(reps + 1):
            phase = rng.choice(5, size=n, p=[0.1, 0.4, 0.25, 0.21, 0.04]).astype(np.int32)
            cid = s.add_colony(dataclasses.replace(col, phase=phase), precision="fp64", update="dt", dt=0.01,
                               reserve=2 * n)
            s.set_cycle(cid, rng.uniform(0.0, 12.0, n), np.full(n, 11.0), np.full(n, 8.0), np.full(n, 4.0),
                        np.full(n, 1.0), np.zeros(n, np.int32))
            s.sync()
            # the C library's stream after srand(k), generated on the device
            t0 = time.perf_counter()
            dv, mk = s.cellcycle(cid, types, secondsperstep=3600.0, stream=S.RandStream(k))
            s.sync()
            t1 = time.perf_counter()
            s.compact(cid)
            s.sync()
            t2 = time.perf_counter()
            s.remove_colony(cid)
            # the same step drawing through the C library's rand() on the host
            cid = s.add_colony(dataclasses.replace(col, phase=phase), precision="fp64", update="dt", dt=0.01,
                               reserve=2 * n)
            s.set_cycle(cid, rng2.uniform(0.0, 12.0, n), np.full(n, 11.0), np.full(n, 8.0), np.full(n, 4.0),
                        np.full(n, 1.0), np.zeros(n, np.int32))
            s.sync()
            t3 = time.perf_counter()
            s.cellcycle(cid, types, secondsperstep=3600.0)
            s.sync()
            t4 = time.perf_counter()
            s.remove_colony(cid)
            if k:
                t_cyc.append((t1 - t0) * 1e3)
                t_cmp.append((t2 - t1) * 1e3)
                t_libc.append((t4 - t3) * 1e3)
                divided.append(dv)
                marked.append(mk)
    return {"config": "1,000,000 clustered cells (seed 2), phases G0/G1/S/G2/M .1/.4/.25/.21/.04, phase times "
                      "uniform in [0, 12) h, lengths 11/8/4/1 h, rd 0.1, one step of 3600 s",
            "cellcycle_ms": float(np.mean(t_cyc)), "compact_ms": float(np.mean(t_cmp)),
            "cellcycle_host_rand_ms": float(np.mean(t_libc)),
            "draws": "cellcycle_ms: the C library's rand() stream after srand(step) generated on the device "
                     "(tm_cycle_params.rand_seeded); cellcycle_host_rand_ms: the same step calling rand() on the host",
            "cells_per_s": n / (np.mean(t_cyc) * 1e-3), "divided": int(np.mean(divided)),
            "marked": int(np.mean(marked))}


def _size_bins(reqs):
    out = {}
    for lo, hi in ((1e3, 1e4), (1e4, 1e5), (1e5, 1e6 + 1)):
        lat = [r.latency for r in reqs if lo <= r.n < hi]
        if lat:
            out[f"{int(lo)}-{int(min(hi, 1e6))}"] = float(np.median(lat))
    return out


def r4(v):
    """4 significant digits (the short line), None kept."""
    if v is None:
        return None
    if isinstance(v, (int, np.integer)):
        return int(v)
    v = float(v)
    return float(f"{v:.4g}") if np.isfinite(v) else None


def neighbour_check(s, cid, col, local):
    """Neighbour sets of the FP32 + compensated colony, evaluated from its
    Verlet lists (built steps before), against a plain FP64 pass that searches
    the bins on the same positions with no lists: per cell the count and the
    fingerprint of the set within h (potential.c:39-78, dist <= h).  The same
    positions' v from a step without diagnostics (the list pass settles most
    cells without the octree walk) against the FP64 pass's walk, which
    diagnostics run for every cell."""
    from timothy_gb300 import session as S

    pos = s.download(cid, ["x", "y", "z"])
    st = s.stats(cid)
    s.step(1)
    s.sync()
    fast_v = s.download(cid, ["v"])["v"]
    walked = s.stats(cid)["walked_cells"]
    s.upload_positions_async(cid, pos["x"], pos["y"], pos["z"])
    s.set_diagnostics(True)
    s.step(1)
    s.sync()
    fast = s.download(cid, ["nbcount", "nbhash"])
    s.set_diagnostics(False)
    at = col.copy()
    at.x, at.y, at.z = pos["x"], pos["y"], pos["z"]
    with S.Session(col.types, dim=3, max_slots=col.n + 64, device=local, diagnostics=True) as s64:
        c64 = s64.add_colony(at, precision="fp64", update="none")
        s64.step(1)
        s64.sync()
        ref = s64.download(c64, ["nbcount", "nbhash", "v"])
    bad = (fast["nbcount"] != ref["nbcount"]) | (fast["nbhash"] != ref["nbhash"])
    vs = float(np.max(np.abs(ref["v"])))
    dv = np.abs(fast_v - ref["v"])
    flips = (fast_v == 0.0) != (ref["v"] == 0.0)
    return {"cells": int(col.n), "pairs_within_h": int(np.sum(ref["nbcount"].astype(np.int64))),
            "mismatched_cells": int(np.sum(bad)), "list_age_steps": st["list_age"],
            "against": "plain FP64 bin search on the same positions, no lists",
            "v": {"nonzero_cells": int(np.count_nonzero(ref["v"])), "walked_cells": int(walked),
                  "max_abs_rel_to_max": float(np.max(dv) / vs) if vs > 0 else 0.0,
                  "zero_pattern_flips": int(np.sum(flips)),
                  "flips_above_1e-5_of_max": int(np.sum(flips & (np.abs(ref["v"]) > 1e-5 * vs)))}}


def e2e_loop(s, cid, col, steps, positions_only=True):
    """End to end through the public API with host buffers, as a host program
    that drives the colony step by step: every step uploads the cells from
    pinned host memory (the positions are the ones the previous step sent
    back; with positions_only the cells' other attributes stay resident and
    only x, y, z travel), runs one step and downloads all its results.  The
    upload of step k + 1 waits on the device for step k's positions to reach
    the host and overlaps the rest of step k's download."""
    from timothy_gb300 import session as S

    n = col.n
    fields = ["x", "y", "z", "density", "v", "mindist", "fx", "fy", "fz", "removecell"]
    res = {k: np.zeros(n, np.uint8 if k == "removecell" else np.float64) for k in fields}
    start = s.download(cid, ["x", "y", "z"])
    for k in ("x", "y", "z"):
        res[k][:] = start[k]
    fixed = [np.ascontiguousarray(a).copy() for a in (col.size, col.young, col.ctype, col.phase)]
    pinned = list(res.values()) + fixed
    for a in pinned:
        S.host_register(a)
    # the upload reads the arrays the previous download writes
    ecol = C.Colony(res["x"], res["y"], res["z"], *fixed, col.types, 3)
    rb0 = s.stats(cid)["list_rebuilds"]
    s.sync()
    t0 = time.perf_counter()
    for _ in range(steps):
        if positions_only:
            s.upload_positions_async(cid, res["x"], res["y"], res["z"])
        else:
            s.upload_async(cid, ecol)
        s.step(1)
        s.download_async(cid, fields, res)
    s.sync()
    ems = (time.perf_counter() - t0) * 1e3
    for a in pinned:
        S.host_unregister(a)
    rebuilds = s.stats(cid)["list_rebuilds"] - rb0
    return ems, rebuilds


def scale1m_record(local, steps, args):
    """The 1 M-cell configuration: 1,000,000 clustered cells (seed 2), plain
    FP64 path with neighbour lists and a CIC deposit onto the 257^3 FP64 grid
    every step: device time over `steps` steps, the CPU implementation on all
    host cores (one step of the whole colony), and parity after 3 steps
    against the oracle (the neighbour sets on the same positions)."""
    from oracle import bindings
    from timothy_gb300 import autotune as AT
    from timothy_gb300 import session as S

    n, seed = 1_000_000, 2
    col = C.make_colony("clustered", n, seed, C.configured_radius("clustered", n, seed))
    out = {"cells": n, "kind": "clustered", "seed": seed, "cic": "257^3 FP64 grid, GFH 8", "precision": "fp64"}
    with S.Session(col.types, dim=3, max_slots=n + 64, device=local, list_capacity=384) as s:
        s.set_tuning(skin_over_h=0.05)
        cid = s.add_colony(col, precision="fp64", update="dt", dt=0.01, cic=True, verlet=True)
        res = AT.autotune(s)
        s.remove_colony(cid)
        cid = s.add_colony(col, precision="fp64", update="dt", dt=0.01, cic=True, verlet=True)
        s.step(3)
        s.sync()
        rb0 = s.stats(cid)["list_rebuilds"]
        s.timer_start()
        s.step(steps)
        ms = s.timer_stop()
        out.update({"steps": steps, "ms_per_step": ms / steps, "value": n * steps / (ms * 1e-3),
                    "rebuilds": s.stats(cid)["list_rebuilds"] - rb0, "tuning": res["best"]})
    # parity: 3 steps, GPU against the oracle
    k = 3
    with S.Session(col.types, dim=3, max_slots=n + 64, device=local, list_capacity=384, diagnostics=True) as s:
        cid = s.add_colony(col, precision="fp64", update="dt", dt=0.01, cic=True, verlet=True)
        s.step(k - 1)
        s.sync()
        before = s.download(cid, ["x", "y", "z"])
        s.step(1)
        s.sync()
        g = s.download(cid, ["x", "y", "z", "density", "mindist", "v", "fx", "fy", "fz", "grid", "nbcount",
                             "nbhash"])
    if not bindings.available("oracle"):
        bindings.build(ref=False)
    t0 = time.perf_counter()
    ref = bindings.run(col, k, which="oracle", update_mode=1, dt=0.01, cic=True)
    cpu_s = time.perf_counter() - t0
    at = col.copy()
    at.x, at.y, at.z = before["x"], before["y"], before["z"]
    nb = bindings.neighbours(at)
    fscale = np.max(np.abs(np.stack([ref.fx, ref.fy, ref.fz])))
    fin = ref.mindist < 1e300
    out["parity_after_3_steps"] = {
        "density_max_rel": float(np.max(np.abs(g["density"] - ref.density) / np.maximum(np.abs(ref.density),
                                                                                       1e-300))),
        "mindist_max_rel": float(np.max(np.abs(g["mindist"][fin] - ref.mindist[fin]) / ref.mindist[fin])),
        "v_max_abs": float(np.max(np.abs(g["v"] - ref.v))),
        "force_max_rel_to_max": float(max(np.max(np.abs(g[q] - getattr(ref, q))) for q in ("fx", "fy", "fz"))
                                      / fscale),
        "position_max_rel": float(max(np.max(np.abs(g[q] - getattr(ref, q)) / np.maximum(np.abs(getattr(ref, q)),
                                                                                         1.0))
                                      for q in ("x", "y", "z"))),
        "grid_max_rel_to_max": float(np.max(np.abs(g["grid"] - ref.grid)) / np.max(np.abs(ref.grid))),
        "neighbour_sets_mismatched_cells": int(np.sum((g["nbcount"] != nb.count) | (g["nbhash"] != nb.hash))),
        "oracle": f"oracle restatement on {os.cpu_count()} host threads"}
    # the CPU implementation on all host cores, one step of the whole colony
    if not args.no_cpu:
        out["cpu_baseline"] = cpu_sample(WORKLOADS["scale1m"], col=col)
        out["cpu_baseline"]["oracle_3_steps_s"] = cpu_s
    return out


def dropin_record(n, kind, seed, cic, steps, warmup=1, precision="fp64"):
    """The reference's own API: the step loop of a host program over the
    drop-ins (octbuild, patches_alloc, patches_cells2envinfo,
    computepotential, computegradient, updatepositions, octfree) on host
    celldata_t records, wall clock per step.  updatepositions draws the
    caller's rand() for every cell as the reference does (cells.c:353-356).
    precision "fp32c": tm_dropin_set_precision(TM_PREC_FP32C, lists on)."""
    import ctypes

    from timothy_gb300 import session as S
    from timothy_gb300.refabi import CELL_DTYPE, DropinRun

    lib = S.load_library()
    lib.tm_dropin_set_precision.argtypes = [ctypes.c_int, ctypes.c_int]
    lib.tm_dropin_pinned_bytes.restype = ctypes.c_int64
    col = C.make_colony(kind, n, seed, C.configured_radius(kind, n, seed))
    if precision == "fp32c":
        lib.tm_dropin_set_precision(1, 1)
    try:
        run = DropinRun(col, cic=cic)
        for _ in range(warmup):
            run.step_loop()
        pinned = int(lib.tm_dropin_pinned_bytes())
        t0 = time.perf_counter()
        for _ in range(steps):
            run.step_loop()
        dt = time.perf_counter() - t0
        # the same loop call by call (each drop-in call returns with its results on the host)
        calls = {k: 0.0 for k in ("octbuild", "patches", "computepotential", "computegradient", "updatepositions")}
        for _ in range(steps):
            for k, v in run.step_loop_timed().items():
                calls[k] += v
        run.shutdown()
    finally:
        lib.tm_dropin_set_precision(0, 0)
    rec = CELL_DTYPE.itemsize
    return {"cells": n, "kind": kind, "cic": cic, "precision": precision, "steps": steps,
            "ms_per_step": dt / steps * 1e3,
            "value": n * steps / dt, "unit": UNIT,
            # per step: the records up (octbuild); density, v, mindist and the
            # forces, then positions and removal marks down; forces and marks up
            "h2d_bytes_per_step": n * (rec + 24 + 1), "d2h_bytes_per_step": n * (24 + 24 + 24 + 1),
            "records_page_locked": pinned >= n * rec,
            "calls_ms": {k: v / steps * 1e3 for k, v in calls.items()}}


def _record_in_process(call, limit_s=900):
    """Run `bench.<call>` in a process of its own and return its JSON record."""
    code = f"import json, bench; print('RECORD ' + json.dumps(bench.{call}))"
    try:
        r = subprocess.run([sys.executable, "-c", code], cwd=os.path.dirname(os.path.abspath(__file__)),
                           capture_output=True, text=True, timeout=limit_s)
    except subprocess.TimeoutExpired:
        return {"error": f"no record within {limit_s} s"}
    for ln in r.stdout.splitlines():
        if ln.startswith("RECORD "):
            return json.loads(ln[7:])
    return {"error": (r.stderr or r.stdout).strip().splitlines()[-1:] if (r.stderr or r.stdout) else "no output",
            "returncode": r.returncode}


def dropin_record_process(n, kind, seed, cic, steps, precision="fp64"):
    """dropin_record in a process of its own, as a host program that links
    the drop-ins would run: the records, their page-locking and the device
    session start from a clean process, not from this one's other sessions
    and registered buffers."""
    return _record_in_process(f"dropin_record({n}, {kind!r}, {seed}, {cic}, {steps}, precision={precision!r})")


def serving_form_process(device, rate, seconds):
    """serving_form in a process of its own, as a server would run: its host
    loop does not share the interpreter with this process's other records."""
    # arrivals for `seconds`, then the drain (at most about twice as long when
    # the offered load is below twice the served rate)
    return _record_in_process(f"serving_form(None, {device}, {rate}, {seconds})", limit_s=900 + 4 * int(seconds))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="precision16m", choices=sorted(WORKLOADS))
    ap.add_argument("--n", type=int, default=0, help="override the cell count")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-check", action="store_true", help="skip the neighbour-set check")
    ap.add_argument("--no-scale1m", action="store_true", help="skip the 1 M-cell FP64 + CIC record")
    ap.add_argument("--no-dropin", action="store_true", help="skip the drop-in (reference API) record")
    ap.add_argument("--e2e-steps", type=int, default=30)
    ap.add_argument("--list-capacity", type=int, default=384,
                    help="neighbour-list entries per cell (0: search the bins every step)")
    ap.add_argument("--rmax", type=int, default=64, help="rebuild the neighbour lists at least every rmax steps")
    ap.add_argument("--skin", type=float, default=0.1, help="neighbour-list skin as a fraction of h (before tuning)")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner (launch shapes, list skin)")
    ap.add_argument("--list-variant", type=int, default=0, help="list kernel variant (with --no-tune; 0: default)")
    ap.add_argument("--no-forms", action="store_true", help="skip the batched and serving forms")
    ap.add_argument("--batch-colonies", type=int, default=512)
    ap.add_argument("--batch-steps", type=int, default=50)
    ap.add_argument("--serve-rates", default="200,50", help="request rates (per s) of the serving runs")
    ap.add_argument("--serve-seconds", type=float, default=20.0)
    ap.add_argument("--detail", default="", help="also write the full record (rows, forms, ...) to this file")
    ap.add_argument("--row", choices=["grid_to_cell", "cic_deposit", "diffusion", "cell_cycle"],
                    help="measure one of the rows beside the path alone and print it (no bench line)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.row:
        peak = measured_peaks()[0]
        fn = {"grid_to_cell": lambda: field_rows(0, peak), "cic_deposit": lambda: cic_rows(0, peak),
              "diffusion": lambda: diffusion_rows(0),
              "cell_cycle": lambda: cycle_rows(0)}[args.row]
        print(json.dumps({args.row: fn()}))
        return 0
    wl = dict(WORKLOADS[args.workload])
    if args.n:
        wl["n"] = args.n
    if args.impl == "reference":
        return run_reference_arm(args, wl)

    world, rank, local, pg = dist_setup()
    from timothy_gb300 import session as S

    # the drop-in records first, each in a process of its own, before this
    # process holds sessions and page-locked buffers of its own
    dropin = None
    if world == 1 and not args.no_dropin:
        dropin = {"1m_cic": dropin_record_process(1_000_000, "clustered", 2, True, 5)}
        if wl["n"] >= 16_000_000:
            dropin["16m"] = dropin_record_process(wl["n"], wl["kind"], wl["seed"], False, 3,
                                                  precision=wl["precision"])

    kind, n, seed = wl["kind"], wl["n"], wl["seed"]
    radius = radius_for(kind, n, seed)
    col = C.make_colony(kind, n, seed, radius)
    prec = wl["precision"]

    tuned = {}

    def new_session(p):
        from timothy_gb300 import autotune as AT

        s = S.Session(col.types, dim=3, max_slots=n + 64, device=local, list_capacity=args.list_capacity)
        s.set_tuning(skin_over_h=args.skin, rmax=args.rmax)
        if args.list_variant:
            s.set_tuning(list_variant=args.list_variant)
        verlet = args.list_capacity > 0

        def add():
            return s.add_colony(col, precision=p, update="dt", dt=wl["dt"], cic=wl["cic"], verlet=verlet)

        cid = add()
        if verlet and not args.no_tune:
            # launch shapes and list skin for this colony; then a fresh copy of it
            res = AT.autotune(s)
            tuned[p] = {"tuning": res["best"], "tune_s": round(res["seconds"], 2)}
            s.remove_colony(cid)
            cid = add()
        return s, cid

    s, cid = new_session(prec)
    s.step(args.warmup)
    s.sync()
    nbc = s.download(cid, ["nbcount"])["nbcount"]
    mean_nb, max_nb = float(nbc.mean()), int(nbc.max())
    rb0 = s.stats(cid)["list_rebuilds"]
    s.profile(True)
    clocks = ClockSampler(local)
    clocks.start()
    dist_barrier(pg)
    l0 = s.launches
    s.timer_start()
    s.step(args.steps)
    ms = s.timer_stop()
    launches = s.launches - l0
    clk = clocks.stop()
    s.sync()
    prof = s.profile_read()
    s.profile(False)
    st_end = s.stats(cid)
    rebuilds = st_end["list_rebuilds"] - rb0
    ms_max = dist_max(pg, ms)
    ms_per_step = ms_max / args.steps
    value = aggregate_value(n, world, args.steps, ms_max)

    peak, peak_kind = measured_peaks()
    # dominant kernel: the list pass (k_plist), one launch per step
    list_ms = prof["list_ms"] if prof["list_ms"] > 0 else prof["pair_ms"]
    achieved = B_CELL * n / (list_ms * 1e-3) / 1e9 if list_ms > 0 else None
    kname = "k_plist32" if prec == "fp32c" else "k_plist<0>"
    traffic = TRAFFIC_PER_CELL.get(kname)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak if achieved else None,
                "traffic": traffic * n / 1e9 if traffic else None, "traffic_unit": "GB per launch",
                "peak_source": peak_kind, "kernel": kname, "kernel_ms": list_ms,
                "phases_ms": {k: prof[k] for k in ("build_ms", "search_ms", "list_ms", "fix_ms", "octree_ms",
                                                   "update_ms", "cic_ms")}}
    detail = {"roofline": dict(roofline),
              "octree_walk": {"walked_cells_last_step": st_end["walked_cells"], "cells": n,
                              "density_fp64_cells_last_step": st_end["density_fp64_cells"]}}
    # the compute side of the list pass (a gather-reduce: no tensor cores):
    # pairs within h per second, from this colony's own neighbour counts, and
    # the algorithmic FP32 flops of those pairs (the reference's expressions,
    # about 83 flops per pair for density and force) against the FP32 FMA
    # rate measured on this device (tm_measure_fp32_peak)
    nb = s.download(cid, ["nbcount"])["nbcount"]
    pairs = float(np.sum(nb.astype(np.int64)))
    if list_ms:
        fp32_peak = S.measure_fp32_peak(local)
        pair_rate = pairs / (list_ms * 1e-3)
        detail["roofline"]["compute"] = {
            "pairs_within_h_per_launch": pairs, "pairs_per_s": pair_rate, "algorithmic_tflops": pair_rate * 83 / 1e12,
            "fp32_peak_tflops": fp32_peak,
            "fp32_peak_source": "measured: FMA chains on every SM (tm_measure_fp32_peak)",
            "frac": pair_rate * 83 / 1e12 / fp32_peak if fp32_peak > 0 else None}
    out_fast = s.download(cid, ["x", "y", "z", "density", "fx", "fy", "fz"]) if prec == "fp32c" else None

    extra = {}
    if not args.no_check and world == 1:
        extra["neighbour_check"] = neighbour_check(s, cid, col, local)

    e2e = None
    if not args.no_e2e:
        ke = max(2, args.e2e_steps)
        ems, erb = e2e_loop(s, cid, col, ke)
        ems = dist_max(pg, ems)
        e2e = {"value": n * world * ke / (ems * 1e-3), "unit": UNIT, "h2d_bytes_per_step": n * 24,
               "d2h_bytes_per_step": n * 73, "steps": ke, "ms_per_step": ems / ke, "rebuilds": erb,
               "api": "tm_colony_upload_async of the positions the previous step sent back (the cells' other "
                      "attributes stay resident) + tm_session_step + tm_colony_download_async of all ten "
                      "outputs, tm_session_sync at the end (wall clock)"}
        ems2, erb2 = e2e_loop(s, cid, col, ke, positions_only=False)
        detail["e2e_all_inputs"] = {"value": n * world * ke / (ems2 * 1e-3), "unit": UNIT,
                                    "h2d_bytes_per_step": n * 44, "d2h_bytes_per_step": n * 73, "steps": ke,
                                    "ms_per_step": ems2 / ke, "rebuilds": erb2,
                                    "api": "as e2e, the upload carrying every input field of the cells"}
    s.close()

    if prec == "fp32c" and not args.no_fp64:
        # plain FP64 path on the same colony and GPU: rate and the error of the
        # compensated path against it after the same number of steps
        s64, c64 = new_session("fp64")
        s64.step(args.warmup)
        s64.sync()
        k64 = args.steps
        rb64 = s64.stats(c64)["list_rebuilds"]
        s64.timer_start()
        s64.step(k64)
        ms64 = s64.timer_stop()
        s64.sync()
        rb64 = s64.stats(c64)["list_rebuilds"] - rb64
        ref = s64.download(c64, ["x", "y", "z", "density", "fx", "fy", "fz"])
        s64.close()
        ms64 = dist_max(pg, ms64)
        v64 = n * world * k64 / (ms64 * 1e-3)
        pos = ref["density"] > 0
        drel = np.abs(out_fast["density"][pos] - ref["density"][pos]) / ref["density"][pos]
        f64 = np.stack([ref["fx"], ref["fy"], ref["fz"]])
        f32 = np.stack([out_fast["fx"], out_fast["fy"], out_fast["fz"]])
        fscale = np.max(np.abs(f64))
        ferr = np.abs(f32 - f64) / fscale
        xerr = np.max([np.max(np.abs(out_fast[k] - ref[k])) for k in ("x", "y", "z")])
        extra["fp64"] = {"value": v64, "ms_per_step": ms64 / k64, "steps": k64, "rebuilds": rb64}
        detail["fp64_tuning"] = tuned.get("fp64")
        extra["fp32c_over_fp64"] = value / v64
        extra["error_vs_fp64"] = {
            "steps": args.warmup + args.steps, "density_max_rel": float(drel.max()),
            "density_rms_rel": float(np.sqrt(np.mean(drel ** 2))), "force_max_rel_to_max": float(ferr.max()),
            "force_rms_rel_to_max": float(np.sqrt(np.mean(ferr ** 2))), "position_max_abs": float(xerr)}

    cpu = None
    if not args.no_cpu and rank == 0 and world == 1:
        cpu = cpu_sample(wl)

    if world == 1 and not args.no_scale1m and args.workload == "precision16m":
        detail["scale1m"] = scale1m_record(local, 100, args)
    if dropin is not None:
        detail["e2e_dropin"] = dropin

    if not args.no_forms and world == 1:
        detail["rows"] = {"grid_to_cell": field_rows(local, peak), "cic_deposit": cic_rows(local, peak),
                          "diffusion": diffusion_rows(local), "cell_cycle": cycle_rows(local)}
        forms = {"batched": batched_form(args, local)}
        forms["serving"] = [serving_form_process(local, float(r), args.serve_seconds)
                            for r in args.serve_rates.split(",") if r]
        detail["forms"] = forms

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+kahan (f64 positions)" if prec == "fp32c" else "f64",
            "data": "synthetic",
            "config": {"workload": args.workload, "kind": kind, "cells": n, "seed": seed, "h": 2.5, "dt": wl["dt"],
                       "cic": wl["cic"], "mean_neighbours": r4(mean_nb), "max_neighbours": max_nb,
                       "l2": "inputs > L2",
                       "parallelism": f"replicas x{world}"},
            "roofline": {k: (r4(v) if not isinstance(v, str) else v) for k, v in roofline.items()
                         if k not in ("phases_ms", "traffic_unit", "peak_source", "kernel")},
            "phases_ms": {k[:-3]: r4(v) for k, v in prof.items() if k.endswith("_ms") and k != "pair_ms"
                          and (k not in ("fix_ms", "cic_ms") or v > 0.05)},
            "rebuilds": rebuilds,
            "cpu_baseline": cpu, "gpu_launches": launches, "clocks": clk}
    line["roofline"]["kernel"] = kname
    if e2e is not None:
        line["e2e"] = {k: r4(v) if not isinstance(v, str) else v for k, v in e2e.items()
                       if k not in ("api", "steps")}
    if cpu is not None:
        line["cpu_baseline"] = {k: r4(v) if not isinstance(v, str) else v for k, v in cpu.items()}
        line["cpu_baseline"]["sample"] = cpu["sample"].split(" cells")[0] + " cells of the workload, 1 step"
    if clk:
        line["clocks"] = {k: r4(v) if isinstance(v, (int, float)) else v for k, v in clk.items()
                          if k in ("sm_mhz", "sm_max_mhz", "reasons")}
    short = {"error_vs_fp64": ("steps", "density_max_rel", "force_max_rel_to_max", "position_max_abs"),
             "neighbour_check": ("cells", "mismatched_cells")}
    for k in ("fp64", "fp32c_over_fp64", "error_vs_fp64", "neighbour_check"):
        if k in extra:
            v = extra[k]
            line[k] = {q: r4(w) for q, w in v.items() if not isinstance(w, str) and q in short.get(k, v)} \
                if isinstance(v, dict) else r4(v)
    if "v" in extra.get("neighbour_check", {}):
        line["neighbour_check"]["v_flips"] = extra["neighbour_check"]["v"]["flips_above_1e-5_of_max"]
    if "scale1m" in detail:
        sc = detail["scale1m"]
        par = sc["parity_after_3_steps"]
        line["scale1m"] = {"ms_per_step": r4(sc["ms_per_step"]), "value": r4(sc["value"]),
                           "cpu_value": r4(sc.get("cpu_baseline", {}).get("value")),
                           "density_err": r4(par["density_max_rel"]), "force_err": r4(par["force_max_rel_to_max"]),
                           "grid_err": r4(par["grid_max_rel_to_max"]),
                           "nb_mismatch": par["neighbour_sets_mismatched_cells"]}
    if "e2e_dropin" in detail:
        line["e2e_dropin"] = {k: r4(v["value"]) if "value" in v else None for k, v in detail["e2e_dropin"].items()}
    if "forms" in detail:
        fb = detail["forms"]["batched"]
        line["forms"] = {"batched_fp32c": r4(fb["fp32c"]["value"]), "batched_fp64": r4(fb["fp64"]["value"]),
                         "serving": [{"rate": r4(f["rate_per_s"]), "served": r4(f["served_cell_updates_per_s"]),
                                      "p50": r4(f["p50_s"]), "p99": r4(f["p99_s"])}
                                     for f in [x for x in detail["forms"]["serving"] if "rate_per_s" in x][:1]]}
    detail["tuning"] = tuned
    if rank == 0:
        full = dict(line)
        full.update(detail)
        full.update(extra)
        full["e2e_full"] = e2e
        if args.detail:
            with open(args.detail, "w") as f:
                json.dump(full, f, indent=1, default=float)
        # the full record first (one line, prefixed so it is not the bench line),
        # then the short bench line last
        print("detail " + json.dumps(full, default=float), flush=True)
        print(json.dumps(line, default=float), flush=True)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
