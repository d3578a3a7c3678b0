"""Autotuner for a session's launch shapes and neighbour-list parameters.

The knobs are those of ``tm_tuning`` (include/timothy_gb300.h):

* ``list_variant``  block size / register budget of the list kernel (every step);
* ``walk_block``    block size of the octree walk (every step);
* ``pair_lshift``   Morton level of the search's candidate ranges (rebuild steps);
* ``skin_over_h``   list skin: longer lists every step against fewer rebuilds.

Each knob is tuned in turn (coordinate descent) on the colonies the session
holds, timing steps with CUDA events on the session's stream.  Kernels that
run every step are ranked by the fastest of a few steps (a step that rebuilds
lists is slower for reasons unrelated to the knob); the search level by the
time of a step in which every colony rebuilds; the skin by a cost model,

    t(skin) = t_list(skin) + rate(skin) * (t_rebuild(skin) - t_list(skin)),

where rate is the fraction of cells rebuilding per step extrapolated from the
displacements the colonies show (``tm_session_list_rate``); the two skins the
model ranks first are then timed over a longer run, rebuilds included.

Tuning advances the colonies: run it on a session whose state may move (the
batch runner re-adds its colonies afterwards).  Results can be cached in a
JSON file keyed by device and workload signature.
"""
from __future__ import annotations

import json
import os
import time

SPACE = {
    "list_variant": [1, 2, 3, 4],
    "walk_block": [64, 128, 256],
    "pair_lshift": [0, 1],
    "skin_over_h": [0.05, 0.1, 0.15, 0.2, 0.3],
}


def _step_times(s, k: int) -> list[float]:
    out = []
    for _ in range(k):
        s.timer_start()
        s.step(1)
        out.append(s.timer_stop())
    return out


def _force_rebuild(s):
    """Rebuild every colony's lists at the next step (re-applying the tuning does it)."""
    t = s.tuning
    skin = t["skin_over_h"]
    s.set_tuning(skin_over_h=skin * 1.000001 if skin < 1.0 else skin * 0.999999)
    s.set_tuning(skin_over_h=skin)


def measure_list_step(s, k: int = 4) -> float:
    _step_times(s, 1)
    return min(_step_times(s, k))


def measure_rebuild_step(s, k: int = 2) -> float:
    times = []
    for _ in range(k):
        _force_rebuild(s)
        times.append(_step_times(s, 1)[0])
    return sorted(times)[len(times) // 2]


def measure_skin(s, skin: float, k: int = 4) -> dict:
    s.set_tuning(skin_over_h=skin)             # forces a rebuild at the next step
    t_rb = _step_times(s, 1)[0]
    t_list = min(_step_times(s, k))
    rate, _ = s.list_rate()
    cost = t_list + rate * max(t_rb - t_list, 0.0)
    return {"skin_over_h": skin, "t_rebuild_ms": t_rb, "t_list_ms": t_list, "rate": rate, "cost_ms": cost}


def autotune(s, space: dict | None = None, k: int = 4, log=None, verify_steps: int = 24) -> dict:
    """Tune ``s`` in place; returns {"best": tuning, "trials": [...], "seconds": t}."""
    space = dict(SPACE, **(space or {}))
    t0 = time.time()
    trials = []
    _step_times(s, 2)                          # first steps build lists and warm caches
    for knob in ("list_variant", "walk_block"):
        best, best_t = None, float("inf")
        for v in space[knob]:
            s.set_tuning(**{knob: v})
            t = measure_list_step(s, k)
            trials.append({"knob": knob, "value": v, "ms": t})
            if log:
                log(f"{knob}={v}: {t:.3f} ms")
            if t < best_t:
                best, best_t = v, t
        s.set_tuning(**{knob: best})
    best, best_t = None, float("inf")
    for v in space["pair_lshift"]:
        s.set_tuning(pair_lshift=v)
        t = measure_rebuild_step(s)
        trials.append({"knob": "pair_lshift", "value": v, "ms": t})
        if log:
            log(f"pair_lshift={v}: {t:.3f} ms (rebuild step)")
        if t < best_t:
            best, best_t = v, t
    s.set_tuning(pair_lshift=best)
    ranked = []
    for v in space["skin_over_h"]:
        r = measure_skin(s, v, k)
        trials.append(dict(r, knob="skin_over_h", value=v, ms=r["cost_ms"]))
        if log:
            log(f"skin_over_h={v}: list {r['t_list_ms']:.3f} ms, rebuild {r['t_rebuild_ms']:.3f} ms, "
                f"rate {r['rate']:.4f} -> {r['cost_ms']:.3f} ms")
        ranked.append((r["cost_ms"], v))
    ranked.sort()
    # The rate is extrapolated from the few steps of a trial; the two skins
    # the model ranks first are then timed over a longer run (mean step time
    # from a fresh rebuild, rebuilds included) and the faster one is kept.
    best, best_t = ranked[0][1], float("inf")
    for _, v in ranked[:2]:
        s.set_tuning(skin_over_h=v)
        t = sum(_step_times(s, verify_steps)) / verify_steps
        trials.append({"knob": "skin_over_h (run)", "value": v, "ms": t})
        if log:
            log(f"skin_over_h={v}: {t:.3f} ms per step over {verify_steps} steps")
        if t < best_t:
            best, best_t = v, t
    s.set_tuning(skin_over_h=best)
    return {"best": s.tuning, "trials": trials, "seconds": time.time() - t0}


def signature(device_name: str, colonies) -> str:
    """Cache key: device, precision mix, cell count and colony count to the nearest power of two."""
    import math

    n = sum(c.n for c in colonies)
    return f"{device_name}|cells~2^{round(math.log2(max(n, 1)))}|colonies~2^{round(math.log2(max(len(colonies), 1)))}"


def load_cached(path: str, key: str) -> dict | None:
    try:
        with open(path) as f:
            return json.load(f).get(key)
    except (OSError, ValueError):
        return None


def store_cached(path: str, key: str, tuning: dict):
    data = {}
    try:
        with open(path) as f:
            data = json.load(f)
    except (OSError, ValueError):
        pass
    data[key] = tuning
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    with open(path, "w") as f:
        json.dump(data, f, indent=1)
