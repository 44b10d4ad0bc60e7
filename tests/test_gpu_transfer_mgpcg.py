"""GPU FLIP/PIC transfers and the standalone MGPCG linear solver against the
reference's golden outputs, through the C ABI."""
import numpy as np
import pytest

import jetgpu
from conftest import golden
from make_systems import poisson_system

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def solver():
    s = jetgpu.FdmMgpcgSolver3(200, 4, 2, 2, 10, 2, 1e-6, 1.0, True)
    yield s
    s.close()


def test_p2g_matches_reference(solver):
    """The default P2G sums each face's contributions in particle order, as
    the reference's serial loop does: grids, markers and FLIP snapshots
    equal the reference's bit for bit."""
    g = golden("transfer_16.npz")
    n, h = 16, 1.0 / 16
    grid = jetgpu.FaceCenteredGrid3((n, n, n), (h, h, h))
    marks, snaps = jetgpu.transfer_from_particles_to_grids(solver, grid,
                                                           g["pos"], g["vel"])
    for a, k in enumerate("uvw"):
        assert np.array_equal(getattr(grid, k), g[k]), k
        assert np.array_equal(marks[a], g["m" + k].astype(np.uint8))
        assert np.array_equal(snaps[a], g["s" + k]), k


def test_p2g_atomic_scatter_matches_reference():
    """orderedP2G=False: FP64 atomics reorder the reference's serial sums,
    so the grids agree to rounding only."""
    s = jetgpu.FdmMgpcgSolver3(200, 4, 2, 2, 10, 2, 1e-6, 1.0, True,
                               orderedP2G=False)
    g = golden("transfer_16.npz")
    n, h = 16, 1.0 / 16
    grid = jetgpu.FaceCenteredGrid3((n, n, n), (h, h, h))
    marks, snaps = jetgpu.transfer_from_particles_to_grids(s, grid, g["pos"],
                                                           g["vel"])
    for a, k in enumerate("uvw"):
        assert np.allclose(getattr(grid, k), g[k], rtol=1e-12, atol=1e-13)
        assert np.array_equal(marks[a], g["m" + k].astype(np.uint8))
        assert np.allclose(snaps[a], g["s" + k], rtol=2e-7, atol=1e-30)
    s.close()


def test_p2g_ordered_is_deterministic_and_exact_at_size():
    """64^3 dam break particles (393,216, jittered): the ordered P2G gives
    the same bits on every call and equals the reference restatement's
    serial sums bit for bit."""
    import oracle
    from jetgpu import scenes
    n = 64
    h = 1.0 / n
    pos, vel = scenes.dam_break_particles(n, (0.25, 0.75, 1.0), seed=0)
    rng = np.random.default_rng(3)
    vel = rng.uniform(-1, 1, pos.shape)
    s = jetgpu.FdmMgpcgSolver3(200, 4, 2, 2, 10, 2, 1e-6, 1.0, True)
    out = []
    for _ in range(2):
        grid = jetgpu.FaceCenteredGrid3((n, n, n), (h, h, h))
        jetgpu.transfer_from_particles_to_grids(s, grid, pos, vel)
        out.append((grid.u.copy(), grid.v.copy(), grid.w.copy()))
    s.close()
    for a in range(3):
        assert np.array_equal(out[0][a], out[1][a])
    port = oracle.port()
    grids, marks, snaps = port.p2g((n, n, n), (h, h, h), (0, 0, 0), pos, vel)
    for a in range(3):
        assert np.array_equal(out[0][a], grids[a]), a


def test_g2p_flip_and_pic_match_reference(solver):
    g = golden("transfer_16.npz")
    n, h = 16, 1.0 / 16
    grid = jetgpu.FaceCenteredGrid3((n, n, n), (h, h, h), (0, 0, 0),
                                    g["new_u"].copy(), g["new_v"].copy(),
                                    g["new_w"].copy())
    snaps = [g["su"].copy(), g["sv"].copy(), g["sw"].copy()]
    vel = g["vel"].copy()
    jetgpu.flip_transfer_from_grids_to_particles(solver, grid, g["pos"], vel,
                                                 snaps)
    # Same snapshot bits in, same float arithmetic: exact.
    assert np.array_equal(vel, g["vel_flip"])
    for a, k in enumerate("uvw"):
        assert np.array_equal(snaps[a], g["d" + k])
    snaps = [g["su"].copy(), g["sv"].copy(), g["sw"].copy()]
    vel = g["vel"].copy()
    jetgpu.flip_transfer_from_grids_to_particles(solver, grid, g["pos"], vel,
                                                 snaps, picBlendingFactor=0.25)
    assert np.allclose(vel, g["vel_blend"], rtol=0, atol=1e-14)
    vel = g["vel"].copy()
    jetgpu.pic_transfer_from_grids_to_particles(solver, grid, g["pos"], vel)
    assert np.array_equal(vel, g["vel_pic"])


def test_mgpcg_poisson_system(solver):
    """fdm_mgpcg_solver3_tests.cpp:13-60 on the GPU: converges; the solution
    matches the reference's tight solve up to the constant null space."""
    g = golden("mgpcg_poisson_32.npz")
    A, b = poisson_system()
    for l in range(4):
        assert np.array_equal(A[l], g[f"A{l}"]) and np.array_equal(b[l], g[f"b{l}"])
    system = jetgpu.FdmMgLinearSystem3(A=A, b=b, x=[np.zeros(a.shape[:3]) for a in A])
    assert solver.solve(system)
    assert solver.lastResidual() <= 1e-6
    x = system.x[0]
    ref = g["x_tight"]
    d = (x - x.mean()) - (ref - ref.mean())
    assert np.linalg.norm(d) / np.linalg.norm(ref - ref.mean()) < 1e-5
