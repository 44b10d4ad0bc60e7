"""GPU particle motion through the C ABI: PicSolver3::moveParticles
(src/jet/pic_solver3.cpp:206-282) with Collider3::resolveCollision
(src/jet/collider3.cpp:19-73) against a transformed sphere must match the
reference bit for bit — its golden outputs, and the oracle port on a larger
random case through the device-pointer entry."""
import numpy as np
import pytest

import jetgpu
import oracle
from conftest import golden

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def solver():
    s = jetgpu.FdmMgpcgSolver3(200, 4, 2, 2, 10, 2, 1e-6, 1.0, True)
    yield s
    s.close()


def test_move_particles_matches_reference(solver):
    g = golden("particles_20x12x16.npz")
    res = tuple(int(x) for x in g["res"])
    grid = jetgpu.FaceCenteredGrid3(res, tuple(g["h"]), tuple(g["origin"]),
                                    g["u"].copy(), g["v"].copy(), g["w"].copy())
    col = jetgpu.Collider.make((0.3, -0.2, 0.1), (0.5, -1.0, 0.7), g["centre"],
                               0.5)
    sph = jetgpu.Sphere.make(0.2, (0.01, -0.02, 0.0), False, g["orient"],
                             g["inv_orient"])
    flipped = jetgpu.Sphere.make(0.3, (0.01, -0.02, 0.0), True, g["orient"],
                                 g["inv_orient"])
    for tag, dt, cfl, closed, c, s in (("a", 0.01, 3.0, 45, col, sph),
                                       ("b", 0.02, 2.0, 63, col, flipped),
                                       ("c", 0.01, 5.0, 63, None, None)):
        pos, vel = g["pos"].copy(), g["vel"].copy()
        jetgpu.move_particles(solver, grid, pos, vel, dt, cfl, closed, c, s)
        assert np.array_equal(pos, g[f"{tag}_pos"]), tag
        assert np.array_equal(vel, g[f"{tag}_vel"]), tag


def test_move_particles_device_matches_port(solver):
    """200,000 particles on a 64^3 grid (config-3-like sphere obstacle)."""
    n = 64
    h = 1.0 / n
    rng = np.random.default_rng(8)
    grids = [rng.uniform(-1, 1, (n, n, n + 1)), rng.uniform(-1, 1, (n, n + 1, n)),
             rng.uniform(-1, 1, (n + 1, n, n))]
    pos = rng.uniform(-0.02, 1.02, (200_000, 3))
    vel = rng.uniform(-1, 1, (200_000, 3))
    centre = (0.6, 0.2, 0.5)
    colp = dict(lin=(0, 0, 0), ang=(0, 0, 0), centre=centre, friction=0.0)
    sphp = dict(center=(0, 0, 0), radius=0.15, normal_flipped=0)
    ref = oracle.port().move_particles((n, n, n), (h, h, h), (0, 0, 0), pos,
                                       vel, grids, 1.0 / 60, 5.0, 63, colp, sphp)
    dev = torch.device("cuda", 0)
    tp, tv = (torch.from_numpy(a.copy()).to(dev) for a in (pos, vel))
    tu, tvv, tw = (torch.from_numpy(a).to(dev) for a in grids)
    g = jetgpu.Grid()
    g.res[:] = (n, n, n)
    g.spacing[:] = (h, h, h)
    g.origin[:] = (0, 0, 0)
    jetgpu.move_particles_device(solver, g, tp, tv, tu, tvv, tw, 1.0 / 60, 5.0,
                                 63, jetgpu.Collider.make(centre=centre),
                                 jetgpu.Sphere.make(0.15))
    torch.cuda.synchronize()
    assert np.array_equal(tp.cpu().numpy(), ref[0])
    assert np.array_equal(tv.cpu().numpy(), ref[1])


def test_move_particles_rejects_bad_inputs(solver):
    grid = jetgpu.FaceCenteredGrid3((4, 4, 4), (0.25,) * 3)
    pos = np.zeros((3, 3))
    vel = np.zeros((3, 3))
    with pytest.raises(jetgpu.JetGpuError):
        jetgpu.move_particles(solver, grid, pos, vel, float("nan"))
    with pytest.raises(jetgpu.JetGpuError):
        jetgpu.move_particles(solver, grid, pos, vel, 0.01, 5.0, 63,
                              jetgpu.Collider.make(), jetgpu.Sphere.make(-1.0))


def test_particle_sdf_matches_reference(solver):
    g = golden("particle_sdf_20x12x16.npz")
    res = tuple(int(x) for x in g["res"])
    h, org = tuple(g["h"]), tuple(g["origin"])
    grid = jetgpu.FaceCenteredGrid3(res, h, org)
    col = jetgpu.CellCenteredScalarGrid3(res, h, org, g["collider_sdf"])
    a = jetgpu.build_signed_distance_field(solver, grid, g["pos"], col, 2.5)
    assert np.array_equal(a, g["a"])
    b = jetgpu.build_signed_distance_field(solver, grid, g["pos"], None, 5.0)
    assert np.array_equal(b, g["b"])


@pytest.mark.parametrize("n", [64, 96])
def test_particle_sdf_device_matches_port(solver, n):
    """Dam-break particles at 8 per cell (the FLIP scenes' seeding) plus
    particles on grid lines and outside the box, with a sphere collider."""
    h = 1.0 / n
    rng = np.random.default_rng(n)
    m = n // 4
    cells = np.stack(np.meshgrid(np.arange(m), np.arange(3 * m),
                                 np.arange(n), indexing="ij"), -1).reshape(-1, 3)
    pos = ((np.repeat(cells, 8, 0) + rng.uniform(size=(cells.shape[0] * 8, 3)))
           * h)
    pos = np.concatenate([pos, rng.integers(0, n, (5000, 3)) * h,
                          rng.uniform(-0.05, 1.05, (5000, 3))])
    k, j, i = np.indices((n, n, n))
    col = np.sqrt(((i + .5) * h - .6) ** 2 + ((j + .5) * h - .2) ** 2 +
                  ((k + .5) * h - .5) ** 2) - 0.15
    ref = oracle.port().build_particle_sdf((n, n, n), (h, h, h), (0, 0, 0), pos,
                                           col, 5.0)
    dev = torch.device("cuda", 0)
    tp = torch.from_numpy(np.ascontiguousarray(pos)).to(dev)
    tcol = torch.from_numpy(col).to(dev)
    out = torch.empty((n, n, n), dtype=torch.float64, device=dev)
    grid = jetgpu.Grid()
    grid.res[:] = (n, n, n)
    grid.spacing[:] = (h, h, h)
    grid.origin[:] = (0, 0, 0)
    f = jetgpu.ScalarField()
    f.kind = 1
    f.data = tcol.data_ptr()
    f.res[:] = (n, n, n)
    f.origin[:] = (0.5 * h,) * 3
    f.spacing[:] = (h, h, h)
    jetgpu.build_signed_distance_field_device(solver, grid, tp, f, out, 5.0)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), ref)
