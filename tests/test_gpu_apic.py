"""GPU APIC (ApicSolver3, src/jet/apic_solver3.cpp) through the C ABI: the
gather (velocities and affine matrices) bit-exact with the reference's
golden outputs, the scatter within FP64 rounding of the reference's serial
sums, and 3 frames of the 24^3 dam break as a whole device-resident APIC step
(tolerances as for FLIP in test_gpu_flip.py: every stage but the pressure
solve is exact)."""
import numpy as np
import pytest

import jetgpu
from conftest import golden
from jetgpu import scenes

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def solver():
    s = jetgpu.FdmMgpcgSolver3(200, 4, 2, 2, 10, 2, 1e-6, 1.0, True)
    yield s
    s.close()


def _grid(res, h, org):
    g = jetgpu.Grid()
    g.res[:] = res
    g.spacing[:] = h
    g.origin[:] = org
    return g


def test_apic_transfers_match_reference(solver):
    g = golden("apic_20x12x16.npz")
    res = tuple(int(x) for x in g["res"])
    h, org = tuple(g["h"]), tuple(g["origin"])
    dev = torch.device("cuda", 0)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    grid = _grid(res, h, org)
    pos, vel, aff = T(g["pos"]), T(g["vel"]), T(g["affine"])
    uvw = [torch.empty(g[k].shape, dtype=torch.float64, device=dev) for k in "uvw"]
    mk = [torch.empty(g[k].shape, dtype=torch.uint8, device=dev) for k in "uvw"]
    jetgpu.apic_transfer_from_particles_to_grids_device(solver, grid, pos, vel,
                                                        aff, *uvw, *mk)
    stream = torch.cuda.ExternalStream(solver.stream(), device=dev)
    stream.synchronize()
    for a, k in enumerate("uvw"):
        assert np.allclose(uvw[a].cpu().numpy(), g[k], rtol=1e-12, atol=1e-13)
        assert np.array_equal(mk[a].cpu().numpy(), g["m" + k].astype(np.uint8))
    gg = [T(g[k]) for k in ("gu", "gv", "gw")]
    vout = torch.empty_like(vel)
    aout = torch.empty_like(aff)
    jetgpu.apic_transfer_from_grids_to_particles_device(solver, grid, pos, vout,
                                                        aout, *gg)
    stream.synchronize()
    assert np.array_equal(vout.cpu().numpy(), g["g2p_vel"])
    assert np.array_equal(aout.cpu().numpy(), g["g2p_affine"])


def test_apic_dam_break_three_frames_matches_reference():
    g = golden("apic_20x12x16.npz")
    n = 24
    ps = jetgpu.FdmMgpcgSolver3(200, 5, 2, 2, 10, 2, 1e-6, 1.0, True)
    sim = jetgpu.FlipSolver3((n, n, n), 1.0 / n, (0, 0, 0), pressureSolver=ps,
                             transfer="apic")
    pos, _ = scenes.dam_break_particles(n, (0.25, 0.75, 1.0), seed=0)
    sim.setParticles(pos)
    for _ in range(3):
        sim.update(1.0 / 60)
    assert np.abs(sim.positions() - g["dam_pos"]).max() < 2e-8
    assert np.abs(sim.velocities() - g["dam_vel"]).max() < 2e-6
    ps.close()
