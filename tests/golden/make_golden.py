"""Generate the golden fixtures in this directory from the reference itself.

Runs the reference's own hot-path functions, compiled unmodified from its
sources into oracle/_ref (``make -C oracle ref``), on seeded synthetic
colonies and stores inputs and outputs as .npz files.  Two builds are
recorded: ``strict`` (no -ffast-math, no FMA contraction) and ``fast`` (the
reference's own flags, src/Makefile:21).  The CPU oracle and the GPU path are
checked against these files; neither the tests nor the GPU machine need the
reference checkout.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import bindings as B  # noqa: E402
from timothy_gb300 import colonies as C  # noqa: E402

OUT_KEYS = ("x", "y", "z", "density", "v", "mindist", "fx", "fy", "fz", "removecell")


def quirky_types():
    # two types whose h2/h3/h4 were derived from the default h = 1.5, as the
    # reference leaves them (initialisation.c:79-82 before io.c:222)
    t = C.CellTypes.consistent(h=(2.5, 1.8), size=(1.0, 0.9))
    t.h2 = np.array([1.5 * 1.5, 1.5 * 1.5])
    t.h3 = t.h2 * 1.5
    t.h4 = t.h3 * 1.5
    return t


def hand_colony(pts, dim=3, size=None):
    pts = np.asarray(pts, np.float64).reshape(-1, 3)
    n = len(pts)
    return C.Colony(np.ascontiguousarray(pts[:, 0]), np.ascontiguousarray(pts[:, 1]),
                    np.ascontiguousarray(pts[:, 2]),
                    np.full(n, 0.9) if size is None else np.asarray(size, np.float64),
                    np.full(n, 2100.0, np.float32), np.zeros(n, np.int32), np.arange(n, dtype=np.int32) % 6,
                    C.CellTypes.consistent(), dim, "hand", 0, 0.0)


def cases():
    """(name, colony, steps, update_mode, dt, cic) for every fixture."""
    out = []
    r1 = C.calibrate_radius("uniform", 10_000, 1)
    out.append(("c1_uniform10k_dt1", C.make_colony("uniform", 10_000, 1, r1), 10, 0, 1.0, False))
    out.append(("c1_uniform10k_dt001", C.make_colony("uniform", 10_000, 1, r1), 10, 1, 0.01, False))
    r2 = C.calibrate_radius("clustered", 4000, 2)
    out.append(("clustered4k_cic", C.make_colony("clustered", 4000, 2, r2), 3, 1, 0.01, True))
    r3 = C.calibrate_radius("uniform", 2000, 3, dim=2)
    out.append(("uniform2d_2k_cic", C.make_colony("uniform", 2000, 3, r3, dim=2), 3, 0, 1.0, True))
    t = quirky_types()
    out.append(("twotype3k", C.make_colony("uniform", 3000, 4, C.initial_radius("uniform", 3000), types=t),
                3, 1, 0.05, False))
    # sparse colony: many cells without neighbours within h
    out.append(("sparse600", C.make_colony("uniform", 600, 5, 40.0), 2, 0, 1.0, True))
    # tiny hand-made cases
    out.append(("n0", hand_colony(np.zeros((0, 3))), 1, 0, 1.0, False))
    out.append(("n1", hand_colony([[0.3, -0.2, 0.1]]), 1, 0, 1.0, False))
    out.append(("n2_touching", hand_colony([[0.0, 0.0, 0.0], [1.2, 0.4, -0.3]]), 2, 0, 1.0, False))
    out.append(("n2_apart", hand_colony([[0.0, 0.0, 0.0], [7.0, 0.0, 0.0]]), 1, 0, 1.0, False))
    out.append(("n5_line", hand_colony([[0.0, 0.0, 0.0], [0.7, 0.0, 0.0], [1.5, 0.1, 0.0],
                                        [2.6, 0.0, 0.2], [5.0, 0.0, 0.0]]), 2, 0, 1.0, False))
    return out


def main():
    B.build(ref=True)
    manifest = {}
    for name, col, steps, mode, dt, cic in cases():
        rec = {"dim": col.dim, "steps": steps, "update_mode": mode, "dt": dt, "cic": int(cic), "gfh": 8.0,
               "x": col.x, "y": col.y, "z": col.z, "size": col.size, "young": col.young, "ctype": col.ctype,
               "phase": col.phase, "th": col.types.h, "th2": col.types.h2, "th3": col.types.h3,
               "th4": col.types.h4, "tsize": col.types.size, "trandommove": col.types.randommove}
        for build in ("ref_strict", "ref"):
            tag = "strict" if build == "ref_strict" else "fast"
            r = B.run(col, steps, which=build, update_mode=mode, dt=dt, cic=cic)
            for k in OUT_KEYS:
                rec[f"{tag}_{k}"] = getattr(r, k)
            rec[f"{tag}_octsize"] = r.octsize
            rec[f"{tag}_aff"] = r.aff
            rec[f"{tag}_removecount"] = r.removecount
            if cic:
                nz = np.nonzero(r.grid)
                rec[f"{tag}_grid_shape"] = np.array(r.grid.shape)
                rec[f"{tag}_grid_idx"] = np.stack(nz, axis=1).astype(np.int32)
                rec[f"{tag}_grid_val"] = r.grid[nz]
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **rec)
        manifest[name] = {"n": col.n, "dim": col.dim, "steps": steps, "update_mode": mode, "dt": dt,
                          "cic": bool(cic), "kind": col.kind, "seed": col.seed, "radius": col.radius}
        print(name, col.n, "done")
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
