"""Golden fixtures of the grid -> cell gather (patches_applyenv2cells), the
field gradient (fieldgradient_compute) and the VTK writer (writevtk), from the
reference's own functions
compiled unmodified into oracle/_ref (``make -C oracle ref``).

The fields come from tests/golden/fields.py (deterministic formulas), so only
cells and outputs are stored; the gradient fixtures keep a seeded sample of
nodes (always including the faces) plus per-component sums.

    python tests/golden/make_golden_fields.py          # gather and gradient
    python tests/golden/make_golden_fields.py --vtk    # the VTK writer
    python tests/golden/make_golden_fields.py --cycle  # the cell cycle
    python tests/golden/make_golden_fields.py --chain  # step loop with the whole cell update
    python tests/golden/make_golden_fields.py --diffusion  # the implicit diffusion step
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from fields import field, gradient_field  # noqa: E402
from oracle import bindings as B  # noqa: E402
from timothy_gb300 import colonies as C  # noqa: E402


def sample_nodes(dims, count, seed):
    gx, gy, gz = dims
    rng = np.random.Generator(np.random.PCG64(seed))
    idx = [rng.integers(0, gx, count), rng.integers(0, gy, count), rng.integers(0, gz, count)]
    faces = []
    for a in (0, gx - 1):
        for b in (0, gy - 1):
            for c in (0, gz - 1):
                faces.append((a, b, c))
    for a in range(0, gx, max(1, gx // 16)):
        faces += [(a, 0, gz // 2), (a, gy - 1, gz // 2), (a, gy // 2, 0), (a, gy // 2, gz - 1)]
    f = np.array(faces, np.int64).T
    return tuple(np.concatenate([idx[k], f[k]]) for k in range(3))


def main():
    if not (B.available("ref") and B.available("ref_strict")):
        raise SystemExit("build the reference first: make -C oracle ref")
    env_cases = [
        ("field_env_clustered4k", C.make_colony("clustered", 4000, 2, C.initial_radius("clustered", 4000)), 8.0, 2),
        ("field_env_uniform2d", C.make_colony("uniform", 2000, 3, C.initial_radius("uniform", 2000, dim=2), dim=2),
         8.0, 1),
        ("field_env_coarse", C.make_colony("uniform", 3000, 4, C.initial_radius("uniform", 3000)), 32.0, 3),
    ]
    for name, col, gfh, nf in env_cases:
        dims = B.grid_dims(col.dim, gfh)
        data, grad = field(nf, dims), gradient_field(nf, dims)
        rec = {"x": col.x, "y": col.y, "z": col.z, "phase": col.phase, "dim": col.dim, "gfh": gfh, "nfields": nf}
        for w, tag in (("ref_strict", "strict"), ("ref", "fast")):
            rec[f"{tag}_cellenv"] = B.env2cells(col, data, grad, gfh=gfh, which=w)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **rec)
        print(name, col.n, dims)
    for name, dim, gfh, nf in (("field_grad_gfh32", 3, 32.0, 2), ("field_grad_gfh8", 3, 8.0, 1),
                               ("field_grad_2d_gfh8", 2, 8.0, 1)):
        dims = B.grid_dims(dim, gfh)
        data = field(nf, dims)
        idx = sample_nodes(dims, 20000, 11)
        rec = {"dim": dim, "gfh": gfh, "nfields": nf, "dims": np.array(dims), "ix": idx[0], "iy": idx[1],
               "iz": idx[2]}
        for w, tag in (("ref_strict", "strict"), ("ref", "fast")):
            g = B.fieldgradient(data, dim=dim, gfh=gfh, which=w)
            rec[f"{tag}_sample"] = g[:, idx[0], idx[1], idx[2], :]
            rec[f"{tag}_sums"] = g.reshape(nf, -1, 3).sum(axis=1)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **rec)
        print(name, dims)


def make_vtk():
    """writevtk (io.c:372-516) of a two-type colony with seeded forces."""
    import hashlib
    import tempfile

    col = C.make_colony("clustered", 3000, 5, C.initial_radius("clustered", 3000),
                        types=C.CellTypes.consistent(h=(2.5, 2.5, 2.5), size=(1.0, 1.0, 1.0)))
    rng = np.random.Generator(np.random.PCG64(9))
    f = rng.normal(size=(3, col.n))
    with tempfile.TemporaryDirectory() as d:
        img = B.write_vtk(os.path.join(d, "x.vtk"), col.x, col.y, col.z, col.ctype, *f, which="ref_strict")
    np.savez_compressed(os.path.join(HERE, "field_vtk_clustered3k.npz"), x=col.x, y=col.y, z=col.z, ctype=col.ctype,
                        fx=f[0], fy=f[1], fz=f[2], sha256=np.frombuffer(hashlib.sha256(img).digest(), np.uint8),
                        nbytes=len(img))
    print("field_vtk_clustered3k", len(img))


CYCLE_TYPES = dict(g1=np.array([11.0, 9.0], np.float32), s=np.array([8.0, 7.0], np.float32),
                   g2=np.array([4.0, 3.0], np.float32), m=np.array([1.0, 1.5], np.float32),
                   v=np.array([0.2, 0.1], np.float32), rd=np.array([0.1, 0.3], np.float32),
                   cd=np.array([2.0, 3.0], np.float32), size=np.array([1.0, 0.9]))
CYCLE_CL1 = np.array([0.3, 0.2, 0.25, 0.1], np.float32)     # [type][field]
CYCLE_CL2 = np.array([0.1, 0.05, 0.1, 0.02], np.float32)


def cycle_state(n, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    return dict(phase=rng.integers(0, 6, n), phasetime=rng.uniform(0, 12, n), g1=rng.uniform(8, 12, n),
                s=rng.uniform(6, 9, n), g2=rng.uniform(2, 5, n), m=rng.uniform(0.5, 2, n), age=rng.integers(0, 5, n),
                size=rng.uniform(0.7, 1.0, n), young=rng.uniform(2000, 2200, n), x=rng.normal(size=n),
                y=rng.normal(size=n), z=rng.normal(size=n), density=rng.uniform(0, 4, n),
                ctype=rng.integers(0, 2, n)), rng.uniform(0, 1, 2 * n), (rng.random(n) < 0.05).astype(np.uint8)


def make_cycle():
    """updatecellcycles with mitosis (cells.c:124-205, 370-523), the reference
    drawing from rand() after srand(seed); inputs and outputs of each case."""
    for name, dim, seed in (("field_cycle_3d", 3, 21), ("field_cycle_2d", 2, 22)):
        st, env, rem = cycle_state(3000, seed)
        if dim == 2:
            st["z"] = np.zeros(3000)
        out = B.cellcycle(st, CYCLE_TYPES, dim=dim, nfields=2, envvalue=env, cl1=CYCLE_CL1, cl2=CYCLE_CL2,
                          sps=3600.0, seed=seed, removecell=rem, which="ref_strict")
        rec = {"dim": dim, "seed": seed, "env": env, "rem": rem}
        rec.update({"in_" + k: v for k, v in st.items()})
        rec.update({"out_" + k: np.asarray(v) for k, v in out.items()})
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **rec)
        print(name, len(out["phase"]), out["removecount"])


CHAIN_CYCLE = dict(g1=np.array([3.0], np.float32), s=np.array([2.0], np.float32), g2=np.array([1.0], np.float32),
                   m=np.array([1.0], np.float32), v=np.array([0.2], np.float32), rd=np.array([0.05], np.float32))


def chain_records(kind, n, seed, dim, cap):
    """Records of a colony of n cells for the cell-update chain (room for cap)."""
    col = C.make_colony(kind, n, seed, C.initial_radius(kind, n), dim=dim)
    rng = np.random.Generator(np.random.PCG64(seed + 1))
    rec = np.zeros(cap, B.REF_CELL_DTYPE)
    for k in ("x", "y", "z", "size", "young", "ctype"):
        rec[k][:n] = getattr(col, k)
    rec["phase"][:n] = rng.integers(0, 5, n)
    rec["phasetime"][:n] = rng.uniform(0, 3, n)
    for k, lo, hi in (("g1", 2.5, 3.5), ("s", 1.5, 2.5), ("g2", 0.7, 1.3), ("m", 0.7, 1.3)):
        rec[k][:n] = rng.uniform(lo, hi, n)
    rec["age"][:n] = rng.integers(0, 4, n)
    rec["gid"][:n] = np.arange(n)
    rec["lifetime"][:n] = rng.integers(0, 100, n)
    return col, rec


def make_chain():
    """The reference step loop with its whole cell update (cellsupdate,
    cells.c:525-543: random move, cell cycle with mitosis, removal) for a few
    steps after srand(seed): the records before and after, and the counters."""
    for name, kind, n, dim, seed, steps in (("chain_clustered3d", "clustered", 2000, 3, 31, 4),
                                            ("chain_uniform2d", "uniform", 1500, 2, 32, 4)):
        cap = 4 * n
        col, rec = chain_records(kind, n, seed, dim, cap)
        types = C.CellTypes.consistent(randommove=[0.05])
        # a critical density at the colony's median lets about half the cells grow
        r = B.run(col, 1, which="ref_strict", update_mode=2)
        cyc = dict(CHAIN_CYCLE, cd=np.array([np.median(r.density)], np.float32))
        counts = B.phase_counts(rec["phase"][:n], rec["ctype"][:n], 1)
        out, cnt = B.ref_cellsupdate(rec, n, types, cyc, dim=dim, sps=3600.0, seed=seed, steps=steps,
                                     counts=counts)
        data = {"dim": dim, "seed": seed, "steps": steps, "cap": cap, "n": n, "sps": 3600.0,
                "randommove": types.randommove, "h": types.h, "tsize": types.size, "counts_in": counts,
                "counts_out": cnt}
        data.update({"cy_" + k: v for k, v in cyc.items()})
        data.update({"in_" + k: rec[k][:n].copy() for k in B.REF_CELL_DTYPE.names})
        data.update({"out_" + k: out[k].copy() for k in B.REF_CELL_DTYPE.names})
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **data)
        print(name, n, "->", len(out), "counts", cnt[:7])


DIFFUSION_CASES = {
    # name: dim, gfh, secondsperstep, gfdt, step, dc, bc, mean, lambda
    "field_diffuse_3d_two": (3, 128.0, 16000.0, 4000.0, 1, [4.0, 1.82e-5], [1.0, 0.1575e-6], [0.5, 0.1575e-6],
                             [0.0, 0.001]),
    "field_diffuse_3d_stiff": (3, 64.0, 16000.0, 3000.0, 1, [200.0], [0.2], [1.0], [1e-4]),
    "field_diffuse_2d": (2, 128.0, 16000.0, 16000.0, 1, [2.0], [0.3], [0.7], [0.0]),
    "field_diffuse_3d_step0": (3, 128.0, 16000.0, 16000.0, 0, [2.0], [0.3], [0.7], [0.0]),
}


def make_diffusion():
    """environment_initsystem + environment_compute (environment.c:131-523),
    compiled unmodified on the Hypre stand-in (oracle/shim_hypre), twice per
    case: the solve count, z, the assembled operator's coefficients, the last
    right-hand side and the solution (fields x-major, z fastest)."""
    for name, (dim, gfh, sps, gfdt, step, dc, bc, mean, lam) in DIFFUSION_CASES.items():
        r = B.ref_environment(dim, gfh, sps, gfdt, step, dc, bc, mean, lam, ncalls=2)
        nx, ny, nz = r["gsize"]
        co = r["coef"]
        rec = {"dim": dim, "gfh": gfh, "sps": sps, "gfdt": gfdt, "step": step, "dc": np.array(dc),
               "bc": np.array(bc), "mean": np.array(mean), "lam": np.array(lam), "gsize": np.array(r["gsize"]),
               "iters": r["iters"], "z": r["z"], "tol": r["tol"], "maxiter": r["maxiter"], "nsolves": r["nsolves"],
               # the diagonal and the -x coupling of an interior node (every in-grid coupling is the same)
               "diag": co[:, 1, 1, min(1, nz - 1), 0], "off": co[:, 1, 1, min(1, nz - 1), 1],
               "b": r["b"], "x": r["x"]}
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **rec)
        print(name, r["gsize"], r["iters"], r["z"])


if __name__ == "__main__":
    if "--diffusion" in sys.argv:
        make_diffusion()
    elif "--chain" in sys.argv:
        make_chain()
    elif "--vtk" in sys.argv:
        make_vtk()
    elif "--cycle" in sys.argv:
        make_cycle()
    else:
        main()
