"""Implicit diffusion step (environment_compute, environment.c:131-523) on the
GPU (FP64 residuals, FP32 multigrid-preconditioned corrections): against the reference's own environment.c run on the Hypre stand-in
(tests/golden/field_diffuse_*.npz), against the oracle on other grids and
inputs, and at the full grid of the default resolution (GFH 8, 257^3 nodes)
through the residual of the solution, checked with an independent torch FP64
stencil.

Tolerances: every GPU solve here runs to a relative residual of 1e-14; the
reference run and the oracle solve to 1e-15; solutions are compared within
1e-11 of their largest value (condition numbers up to ~2e3 here)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DIFFUSION = ["field_diffuse_3d_two", "field_diffuse_3d_stiff", "field_diffuse_2d", "field_diffuse_3d_step0"]


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def point_source(gsize, nf, step):
    """environment_pcfunction (environment.c:251-266): 100 at node (5, 5, 5) from step 1 on."""
    src = np.zeros((nf,) + tuple(gsize))
    nx, ny, nz = gsize
    if step != 0 and nx > 5 and ny > 5 and nz > 5:
        src[:, 5, 5, 5] = 100.0
    return src


def stencil_residual(torch, u, b, diag, z):
    """|b - A u| / |b| with A the 7-point operator of the step (torch, FP64)."""
    au = diag * u
    for ax in range(3):
        n = u.shape[ax]
        if n < 2:
            continue
        lo = [slice(None)] * 3
        hi = [slice(None)] * 3
        lo[ax] = slice(0, n - 1)
        hi[ax] = slice(1, n)
        au[tuple(lo)] -= z * u[tuple(hi)]
        au[tuple(hi)] -= z * u[tuple(lo)]
    return float(torch.linalg.vector_norm(b - au) / torch.linalg.vector_norm(b))


@pytest.mark.parametrize("name", DIFFUSION)
def test_diffusion_matches_reference(name):
    torch = _torch()
    from timothy_gb300.session import Diffusion

    rec = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    gs = tuple(int(v) for v in rec["gsize"])
    nf = len(rec["dc"])
    data = torch.from_numpy(np.broadcast_to(rec["mean"][:, None, None, None], (nf,) + gs).copy()).cuda()
    src = torch.from_numpy(point_source(gs, nf, int(rec["step"]))).cuda()
    with Diffusion(gs) as d:
        st = d.step(data, float(rec["gfh"]), rec["dc"], rec["bc"], rec["lam"], float(rec["sps"]),
                    float(rec["gfdt"]), source=src, tol=1e-14)
    torch.cuda.synchronize()
    got = data.cpu().numpy()
    assert st["solves_per_field"] == int(rec["iters"])
    assert st["max_relative_residual"] <= 1e-14
    for f in range(nf):
        assert np.max(np.abs(got[f] - rec["x"][f])) <= 1e-11 * np.max(np.abs(rec["x"][f])), f


@pytest.mark.parametrize("gsize,dc,lam,sps,gfdt", [((33, 33, 33), [40.0], [0.0], 9000.0, 3000.0),
                                                    ((20, 13, 7), [3.0], [0.01], 1000.0, 1000.0),
                                                    ((24, 31, 1), [500.0], [0.0], 1000.0, 1000.0),
                                                    ((9, 9, 9), [1e-3], [0.0], 1000.0, 1000.0)])
def test_diffusion_matches_oracle(oracle_lib, gsize, dc, lam, sps, gfdt):
    """Start from a field and a source of the caller's (not the reference's
    mean and point source), on grids of even, odd and one-layer sizes."""
    torch = _torch()
    from timothy_gb300.session import Diffusion

    rng = np.random.default_rng(11)
    u0 = rng.uniform(0.0, 2.0, (1,) + gsize)
    src = rng.uniform(0.0, 0.5, (1,) + gsize)
    bc, res = [0.4], 16.0
    ref = oracle_lib.diffuse(gsize, res, sps, gfdt, 1, dc, bc, [0.0], lam, u0=u0, source=src)
    data = torch.from_numpy(u0.copy()).cuda()
    with Diffusion(gsize) as d:
        st = d.step(data, res, dc, bc, lam, sps, gfdt, source=torch.from_numpy(src).cuda(), tol=1e-14)
    torch.cuda.synchronize()
    assert st["solves_per_field"] == ref["iters"]
    got = data.cpu().numpy()
    assert np.max(np.abs(got - ref["u"])) <= 1e-11 * np.max(np.abs(ref["u"]))


def test_diffusion_reproducible_and_multigrid():
    """Deterministic reductions: the same inputs give the same bits; a stiff
    operator takes the multigrid preconditioner and converges in few iterations."""
    torch = _torch()
    from timothy_gb300.session import Diffusion

    gs = (65, 65, 65)
    rng = np.random.default_rng(5)
    u0 = rng.uniform(0.0, 1.0, (1,) + gs)
    outs = []
    for _ in range(2):
        data = torch.from_numpy(u0.copy()).cuda()
        with Diffusion(gs) as d:
            st = d.step(data, 8.0, [2000.0], [0.1], [0.0], 1000.0, 1000.0, tol=1e-12)
        torch.cuda.synchronize()
        outs.append(data.cpu().numpy())
    assert np.array_equal(outs[0], outs[1])
    assert st["multigrid_fields"] == 1 and st["levels"] == 6
    assert st["max_iterations"] <= 60 and st["refinements"] <= 6
    assert st["max_relative_residual"] <= 1e-12


def test_diffusion_full_grid_residual():
    """The default grid (GFH 8: 257^3 nodes, two fields): every solve reaches
    the reference's tolerance, checked by an independent stencil in torch."""
    torch = _torch()
    from oracle import bindings
    from timothy_gb300.session import Diffusion

    gs = bindings.grid_dims(3, 8.0)
    assert gs == (257, 257, 257)
    g = torch.Generator(device="cuda").manual_seed(3)
    u0 = torch.rand((2,) + gs, generator=g, device="cuda", dtype=torch.float64)
    src = torch.rand((2,) + gs, generator=g, device="cuda", dtype=torch.float64) * 0.01
    dc, bc, lam, gfh, gfdt = [1.82e-5 * 1e6, 2.0], [0.1575e-6, 1.0], [0.0, 1e-4], 8.0, 2000.0
    data = u0.clone()
    with Diffusion(gs) as d:
        st = d.step(data, gfh, dc, bc, lam, 2000.0, gfdt, source=src, tol=1e-12)
    torch.cuda.synchronize()
    assert st["solves_per_field"] == 1 and st["max_relative_residual"] <= 1e-12
    for f in range(2):
        z = bindings.diffusion_z(dc[f], gfdt, gfh)
        diag = 1 + 6.0 * z + lam[f] * gfdt
        b = u0[f].clone() + src[f]
        zb = z * bc[f]
        for ax in range(3):
            for end in (0, gs[ax] - 1):
                sl = [slice(None)] * 3
                sl[ax] = end
                b[tuple(sl)] += zb
        assert stencil_residual(torch, data[f], b, diag, z) <= 2e-12


def test_environment_dropins_match_reference():
    """environment_allocate / init / initsystem / compute through the
    reference-signature drop-ins: data keeps the initial values (as the
    reference leaves it), the step's solution matches the reference's run;
    with write-back the solution lands in data.  The drop-in solves to the
    reference's 1e-12 (condition number ~13 here: 1e-10 of the largest value)."""
    _torch()
    from timothy_gb300.refabi import EnvironmentRun

    rec = np.load(os.path.join(GOLDEN, "field_diffuse_3d_two.npz"))
    fields = [{"dc": float(rec["dc"][f]), "bc": float(rec["bc"][f]), "mean": float(rec["mean"][f]),
               "lam": float(rec["lam"][f])} for f in range(len(rec["dc"]))]
    with EnvironmentRun(int(rec["dim"]), float(rec["gfh"]), fields, secondsperstep=float(rec["sps"]),
                        gfdt=float(rec["gfdt"]), step=int(rec["step"])) as run:
        assert run.gsize == tuple(int(v) for v in rec["gsize"])
        run.compute()
        for f in range(len(fields)):
            assert np.all(run.data(f) == fields[f]["mean"])
            sol = run.solution(f)
            assert np.max(np.abs(sol - rec["x"][f])) <= 1e-10 * np.max(np.abs(rec["x"][f])), f
        run.compute(writeback=True)
        for f in range(len(fields)):
            assert np.array_equal(run.data(f), run.solution(f))


def test_one_shot_and_two_fields(oracle_lib):
    """tm_field_diffuse (a solver made for the call) on two fields at once,
    against the oracle field by field."""
    torch = _torch()
    import ctypes as C

    from timothy_gb300 import session as S

    gs = (21, 18, 12)
    rng = np.random.default_rng(2)
    u0 = rng.uniform(0.0, 1.0, (2,) + gs)
    src = rng.uniform(0.0, 0.2, (2,) + gs)
    # field 0: z = 0.625 (plain CG); field 1: z = 3750 (multigrid)
    dc, bc, lam, res, sps, gfdt = [0.01, 60.0], [0.3, 0.0], [0.0, 0.002], 4.0, 3000.0, 1000.0
    ref = oracle_lib.diffuse(gs, res, sps, gfdt, 1, dc, bc, [0.0, 0.0], lam, u0=u0, source=src)
    data = torch.from_numpy(u0.copy()).cuda()
    st = S.DiffusionStats()
    arr = [np.ascontiguousarray(v, np.float64) for v in (dc, bc, lam)]
    gsz = np.array(gs, np.int64)
    lib = S.load_library()
    rc = lib.tm_field_diffuse(data.data_ptr(), gsz.ctypes.data, res, 2, *[a.ctypes.data for a in arr], sps, gfdt,
                              torch.from_numpy(src).cuda().data_ptr(), 1e-14, C.byref(st), None)
    assert rc == 0
    torch.cuda.synchronize()
    assert st.solves_per_field == ref["iters"] == 3 and st.multigrid_fields == 1
    got = data.cpu().numpy()
    for f in range(2):
        assert np.max(np.abs(got[f] - ref["u"][f])) <= 1e-11 * np.max(np.abs(ref["u"][f])), f


def test_environment_dropins_2d():
    """The drop-ins on a one-layer (2-D) grid: the reference's fixture (the
    point source lies off the grid there: no z node 5)."""
    _torch()
    from timothy_gb300.refabi import EnvironmentRun

    rec = np.load(os.path.join(GOLDEN, "field_diffuse_2d.npz"))
    fields = [{"dc": float(rec["dc"][0]), "bc": float(rec["bc"][0]), "mean": float(rec["mean"][0]),
               "lam": float(rec["lam"][0])}]
    with EnvironmentRun(2, float(rec["gfh"]), fields, secondsperstep=float(rec["sps"]), gfdt=float(rec["gfdt"]),
                        step=int(rec["step"])) as run:
        assert run.gsize == tuple(int(v) for v in rec["gsize"])
        run.compute(writeback=True)
        sol = run.data(0)
        assert np.max(np.abs(sol - rec["x"][0])) <= 1e-10 * np.max(np.abs(rec["x"][0]))
