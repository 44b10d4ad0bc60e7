"""GPU boundary conditions through the C ABI: constrainVelocity
(GridFractionalBoundaryConditionSolver3, src/jet/
grid_fractional_boundary_condition_solver3.cpp:26-233) and extrapolateToRegion
(include/jet/detail/array_utils-inl.h:172-244) must match the reference bit
for bit — against its golden outputs, and against the oracle port on larger
random scenes."""
import numpy as np
import pytest

import jetgpu
import oracle
from conftest import golden

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

KMAX = float(np.finfo(np.float64).max)


@pytest.fixture(scope="module")
def solver():
    s = jetgpu.FdmMgpcgSolver3(200, 4, 2, 2, 10, 2, 1e-6, 1.0, True)
    yield s
    s.close()


def gpu_constrain(solver, res, h, org, u, v, w, sdf, col, closed, depth,
                  blocked=False):
    """Host-pointer path through the Python mirror class."""
    vel = jetgpu.FaceCenteredGrid3(res, h, org, u.copy(), v.copy(), w.copy())
    cls = (jetgpu.GridBlockedBoundaryConditionSolver3 if blocked
           else jetgpu.GridFractionalBoundaryConditionSolver3)
    bc = cls(solver)
    sdf_f = (jetgpu.CellCenteredScalarGrid3(res, h, org, sdf)
             if isinstance(sdf, np.ndarray) else jetgpu.ConstantScalarField3(sdf))
    bc.updateCollider(sdf_f, None if col is None else jetgpu.Collider.make(
        col["lin"], col["ang"], col["centre"], col["friction"]))
    bc.setClosedDomainBoundaryFlag(closed)
    bc.constrainVelocity(vel, depth)
    return vel.u, vel.v, vel.w


def test_constrain_velocity_matches_reference(solver):
    g = golden("boundary_20x16x12.npz")
    res = tuple(int(x) for x in g["res"])
    h, org = tuple(g["h"]), tuple(g["origin"])
    m = g["moving"]
    centre = tuple(g["centre"])
    cases = [("a", g["sdf"], dict(lin=m[:3], ang=m[3:6], centre=centre,
                                  friction=float(m[6])), 63, 5),
             ("b", g["sdf"], dict(lin=(0, 0, 0), ang=(0, 0, 0), centre=centre,
                                  friction=0.0), 41, 3),
             ("c", KMAX, None, 63, 5)]
    for tag, sdf, col, closed, depth in cases:
        out = gpu_constrain(solver, res, h, org, g["u"], g["v"], g["w"], sdf,
                            col, closed, depth)
        for a, k in enumerate("uvw"):
            assert np.array_equal(out[a], g[f"{tag}_{k}"]), (tag, k)


def test_constrain_velocity_blocked_matches_reference(solver):
    """GridBlockedBoundaryConditionSolver3::constrainVelocity
    (grid_blocked_boundary_condition_solver3.cpp:23-67)."""
    g = golden("boundary_20x16x12.npz")
    gb = golden("boundary_blocked_20x16x12.npz")
    res = tuple(int(x) for x in g["res"])
    h, org = tuple(g["h"]), tuple(g["origin"])
    m = g["moving"]
    centre = tuple(g["centre"])
    cases = [("a", dict(lin=m[:3], ang=m[3:6], centre=centre,
                        friction=float(m[6])), 63, 5),
             ("b", dict(lin=(0, 0, 0), ang=(0, 0, 0), centre=centre,
                        friction=0.0), 41, 3)]
    for tag, col, closed, depth in cases:
        out = gpu_constrain(solver, res, h, org, g["u"], g["v"], g["w"],
                            g["sdf"], col, closed, depth, blocked=True)
        for a, k in enumerate("uvw"):
            assert np.array_equal(out[a], gb[f"{tag}_{k}"]), (tag, k)


def test_extrapolate_matches_reference(solver):
    g = golden("boundary_20x16x12.npz")
    dev = torch.device("cuda", 0)
    data = torch.from_numpy(g["ext_in"].copy()).to(dev)
    valid = torch.from_numpy(g["ext_valid"].astype(np.uint8)).to(dev)
    jetgpu.extrapolate_to_region_device(solver, data, valid, 4)
    torch.cuda.synchronize()
    assert np.array_equal(data.cpu().numpy(), g["ext_out"])
    # The caller's validity is left as it was.
    assert np.array_equal(valid.cpu().numpy(), g["ext_valid"].astype(np.uint8))


@pytest.mark.parametrize("blocked", [False, True])
@pytest.mark.parametrize("res,closed,fr,depth", [((64, 64, 64), 63, 0.25, 5),
                                                 ((72, 40, 56), 22, 0.0, 3)])
def test_constrain_velocity_device_matches_port(solver, res, closed, fr, depth,
                                                blocked):
    """The device-pointer entry on larger random scenes, against the oracle
    port (itself pinned to the reference)."""
    nx, ny, nz = res
    hh = 1.0 / max(res)
    h, org = (hh, hh, hh), (0.0, 0.0, 0.0)
    rng = np.random.default_rng(3)
    k, j, i = np.indices((nz, ny, nx))
    c = (0.6 * nx * hh, 0.35 * ny * hh, 0.5 * nz * hh)
    sdf = np.sqrt(((i + .5) * hh - c[0]) ** 2 + ((j + .5) * hh - c[1]) ** 2 +
                  ((k + .5) * hh - c[2]) ** 2) - 0.2
    u = rng.uniform(-1, 1, (nz, ny, nx + 1))
    v = rng.uniform(-1, 1, (nz, ny + 1, nx))
    w = rng.uniform(-1, 1, (nz + 1, ny, nx))
    col = dict(lin=(0.1, 0.2, -0.3), ang=(-0.6, 0.2, 0.9), centre=c, friction=fr)
    ref = oracle.port().constrain_velocity(res, h, org, u, v, w, sdf, col,
                                           closed, depth, blocked=blocked)
    dev = torch.device("cuda", 0)
    tu, tv, tw = (torch.from_numpy(a.copy()).to(dev) for a in (u, v, w))
    tsdf = torch.from_numpy(sdf).to(dev)
    grid = jetgpu.Grid()
    grid.res[:] = res
    grid.spacing[:] = h
    grid.origin[:] = org
    f = jetgpu.ScalarField()
    f.kind = 1
    f.data = tsdf.data_ptr()
    f.res[:] = res
    f.origin[:] = (0.5 * hh,) * 3
    f.spacing[:] = h
    jetgpu.constrain_velocity_device(
        solver, grid, tu, tv, tw, f,
        jetgpu.Collider.make(col["lin"], col["ang"], col["centre"], fr),
        closed, depth, blocked=blocked)
    torch.cuda.synchronize()
    for a, t in enumerate((tu, tv, tw)):
        assert np.array_equal(t.cpu().numpy(), ref[a]), "uvw"[a]


def test_bad_inputs_rejected(solver):
    L = jetgpu.library()
    g = jetgpu.Grid()
    g.res[:] = (0, 4, 4)
    g.spacing[:] = (1, 1, 1)
    f = jetgpu.ScalarField()
    f.kind = 0
    a = np.zeros(8)
    assert L.jetgpu_constrain_velocity(solver.context(), g, a.ctypes.data,
                                       a.ctypes.data, a.ctypes.data, f, None,
                                       63, 5) == 3
    f.kind = 7
    g.res[:] = (4, 4, 4)
    assert L.jetgpu_constrain_velocity(solver.context(), g, a.ctypes.data,
                                       a.ctypes.data, a.ctypes.data, f, None,
                                       63, 5) == 3
    res = (jetgpu.C.c_int * 3)(4, 0, 4)
    assert L.jetgpu_extrapolate_to_region_device(solver.context(), res,
                                                 a.ctypes.data, a.ctypes.data,
                                                 1) == 3
