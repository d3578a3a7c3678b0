"""Grid -> cell gather (patches_applyenv2cells) and field gradient
(fieldgradient_compute) on the GPU against the oracle, bit for bit: both are
FP64 with the reference's roundings and summation order."""
import os
import sys

import numpy as np
import pytest

from timothy_gb300 import colonies as C

pytestmark = pytest.mark.gpu
sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
from fields import field, gradient_field  # noqa: E402


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def lower_of(dim):
    return (-1024.0, -1024.0, -1024.0 if dim == 3 else 0.0)


@pytest.mark.parametrize("dim,gfh,nf", [(3, 8.0, 1), (3, 32.0, 2), (2, 8.0, 1), (3, 10.0, 1)])
def test_field_gradient_matches_oracle(oracle_lib, dim, gfh, nf):
    torch = _torch()
    from timothy_gb300 import session as S

    dims = oracle_lib.grid_dims(dim, gfh)
    data = field(nf, dims)
    ref = oracle_lib.fieldgradient(data, dim=dim, gfh=gfh, which="oracle")
    d = torch.from_numpy(data).cuda()
    g = torch.zeros(data.shape + (3,), dtype=torch.float64, device="cuda")
    S.field_gradient_device(d, dims, gfh, nf, g)
    torch.cuda.synchronize()
    assert np.array_equal(g.cpu().numpy(), ref)


@pytest.mark.parametrize("kind,n,dim,gfh,nf", [("clustered", 4000, 3, 8.0, 2), ("uniform", 2000, 2, 8.0, 1),
                                                ("uniform", 3000, 3, 32.0, 3), ("clustered", 5000, 3, 10.0, 1)])
def test_env2cells_matches_oracle(oracle_lib, kind, n, dim, gfh, nf):
    torch = _torch()
    from timothy_gb300 import session as S

    col = C.make_colony(kind, n, 61, C.initial_radius(kind, n, dim=dim), dim=dim)
    dims = oracle_lib.grid_dims(dim, gfh)
    data, grad = field(nf, dims), gradient_field(nf, dims)
    ref = oracle_lib.env2cells(col, data, grad, gfh=gfh, which="oracle")
    xs = [torch.from_numpy(np.ascontiguousarray(getattr(col, k))).cuda() for k in ("x", "y", "z")]
    out = torch.zeros((nf, n, 4), dtype=torch.float64, device="cuda")
    S.env2cells_device(*xs, n, dim, lower_of(dim), gfh, dims, nf, torch.from_numpy(data).cuda(),
                       torch.from_numpy(grad).cuda(), out)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), ref)


def test_colony_env2cells_after_steps(oracle_lib):
    """The session gathers for its resident (Morton-ordered) cells in caller order."""
    torch = _torch()
    from timothy_gb300 import session as S

    col = C.make_colony("clustered", 20000, 62, C.initial_radius("clustered", 20000))
    gfh, nf = 8.0, 2
    dims = oracle_lib.grid_dims(3, gfh)
    data, grad = field(nf, dims), gradient_field(nf, dims)
    with S.Session(col.types, max_slots=col.n + 64, list_capacity=384) as s:
        cid = s.add_colony(col, precision="fp64", update="dt", dt=0.01, verlet=True)
        s.step(3)
        s.sync()
        pos = s.download(cid, ["x", "y", "z"])
        got = s.env2cells(cid, lower_of(3), gfh, dims, nf, torch.from_numpy(data).cuda(),
                          torch.from_numpy(grad).cuda())
    moved = C.Colony(pos["x"], pos["y"], pos["z"], col.size, col.young, col.ctype, col.phase, col.types)
    assert np.array_equal(got, oracle_lib.env2cells(moved, data, grad, gfh=gfh, which="oracle"))


def test_dropin_env2cells_and_fieldgradient(oracle_lib):
    """The reference-signature drop-ins inside the reference step order."""
    from timothy_gb300.refabi import DropinRun

    col = C.make_colony("clustered", 3000, 63, C.initial_radius("clustered", 3000))
    gfh, nf = 8.0, 2
    dims = oracle_lib.grid_dims(3, gfh)
    data, grad = field(nf, dims), gradient_field(nf, dims)
    # the drop-ins page-lock the run's cells until shutdown: leave none behind
    with DropinRun(col, cic=True, gfh=gfh, nfields=nf) as run:
        run.step(update=False, env=(data, grad))
        assert np.array_equal(run.cellenv, oracle_lib.env2cells(col, data, grad, gfh=gfh, which="oracle"))
        run.step(update=True, env=(data, grad))        # again, with the position update after it
        assert np.array_equal(run.cellenv, oracle_lib.env2cells(col, data, grad, gfh=gfh, which="oracle"))
        g = run.fieldgradient(data)
    assert np.array_equal(g, oracle_lib.fieldgradient(data, dim=3, gfh=gfh, which="oracle"))


def test_colony_vtk_matches_oracle(oracle_lib, tmp_path):
    """The reference's VTK file of a resident colony, assembled on the device."""
    from timothy_gb300 import session as S

    types = C.CellTypes.consistent(h=(2.5, 2.5), size=(1.0, 1.0))
    col = C.make_colony("clustered", 6000, 64, C.initial_radius("clustered", 6000), types=types)
    with S.Session(types, max_slots=col.n + 64, list_capacity=384) as s:
        cid = s.add_colony(col, precision="fp64", update="dt", dt=0.01, verlet=True)
        s.step(3)
        s.sync()
        out = s.download(cid, ["x", "y", "z", "fx", "fy", "fz"])
        s.write_vtk(cid, str(tmp_path / "gpu.vtk"))
    ref = oracle_lib.write_vtk(str(tmp_path / "cpu.vtk"), out["x"], out["y"], out["z"], col.ctype, out["fx"],
                               out["fy"], out["fz"], which="oracle")
    assert (tmp_path / "gpu.vtk").read_bytes() == ref
