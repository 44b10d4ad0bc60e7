"""A whole FLIP / PIC step resident on the GPU (jetgpu_flip_substep_device
driven by the reference's adaptive sub-stepping) against the reference's
FlipSolver3 / PicSolver3 (src/jet/flip_solver3.cpp, src/jet/pic_solver3.cpp):
3 frames of the 64^3 dam break's geometry at 24^3, 20,736 particles.

The reference's run solved every pressure system to an absolute
sqrt(r.M^-1 r) of 1e-10 (golden fixture); the GPU solves each to a relative
true residual of 1e-6. Every other stage is bit-exact with the reference, so
the particles differ only through the pressure solves' residuals: the
positions after 3 frames must agree to 2e-8 (h = 1/24 ~ 4.2e-2; measured
6.3e-9; a run of the reference itself at tolerance 1e-6 lands 1.2e-9 away)
and the velocities to 2e-6 (measured 3.7e-7)."""
import numpy as np
import pytest

import jetgpu
from conftest import golden
from jetgpu import scenes

pytestmark = pytest.mark.gpu
pytest.importorskip("torch")

POS_TOL = 2e-8
VEL_TOL = 2e-6


@pytest.mark.parametrize("flip", [True, False])
def test_dam_break_three_frames_matches_reference(flip):
    g = golden("flip_dam_break_24.npz")
    n = 24
    h = 1.0 / n
    ps = jetgpu.FdmMgpcgSolver3(200, 5, 2, 2, 10, 2, 1e-6, 1.0, True)
    sim = jetgpu.FlipSolver3((n, n, n), h, (0, 0, 0), pressureSolver=ps,
                             flip=flip)
    # The reference's seeding (std::mt19937(0), cell order k, j, i).
    pos, _ = scenes.dam_break_particles(n, (0.25, 0.75, 1.0), seed=0)
    sim.setParticles(pos)
    for _ in range(3):
        sim.update(1.0 / 60)
    tag = "flip" if flip else "pic"
    pos, vel = sim.positions(), sim.velocities()
    assert sim.subSteps >= 3
    assert np.abs(pos - g[f"{tag}_pos"]).max() < POS_TOL
    assert np.abs(vel - g[f"{tag}_vel"]).max() < VEL_TOL
    ps.close()


def test_dam_break_with_sphere_collider_matches_reference():
    """The 24^3 dam break with a static sphere collider cutting into the
    water column (some particles start inside it): collisions, the collider
    classification shared by a sub-step's boundary passes, its cached
    normals and the extrapolation fronts next to the collider, against
    FlipSolver3 with GridFluidSolver3::setCollider (flip_sphere_24.npz)."""
    g = golden("flip_sphere_24.npz")
    n = 24
    h = 1.0 / n
    ps = jetgpu.FdmMgpcgSolver3(200, 5, 2, 2, 10, 2, 1e-6, 1.0, True)
    sim = jetgpu.FlipSolver3((n, n, n), h, (0, 0, 0), pressureSolver=ps)
    pos, _ = scenes.dam_break_particles(n, (0.25, 0.75, 1.0), seed=0)
    sim.setParticles(pos)
    centre = tuple(float(x) for x in g["centre"])
    sim.setCollider(g["sdf"],
                    jetgpu.Collider.make(centre=centre,
                                         friction=float(g["friction"])),
                    jetgpu.Sphere.make(float(g["radius"])))
    for _ in range(3):
        sim.update(1.0 / 60)
    pos, vel = sim.positions(), sim.velocities()
    assert sim.subSteps >= 3
    assert np.abs(pos - g["flip_pos"]).max() < POS_TOL
    assert np.abs(vel - g["flip_vel"]).max() < VEL_TOL
    ps.close()


# The 64^3 dam break for 60 frames: bounds on the GPU run's deviation from the
# reference's (golden fixture flip_dam_break_64.npz). The reference itself,
# run again with its solver at a tolerance of 1e-6 instead of 1e-10, lands
# 3.6e-8 / 3.2e-8 / 2.2e-6 / 6.6e-2 (pressure relative L2 after frames 1,
# 10, 30, 60) and 0.053 RMS / 0.81 maximum (final positions of every 16th
# particle; h = 1/64) away from it: before the splash the solves agree to
# their tolerance, after it the flow is chaotic and only the statistics of
# the particle cloud are comparable.
DAM64_P_REL = {1: 1e-5, 10: 1e-5, 30: 1e-3, 60: 0.3}
DAM64_POS_RMS = 0.2
DAM64_CLOUD = 0.01  # |mean| and |std| of all final positions, per axis


def test_dam_break_64_sixty_frames_vs_reference():
    """The 64^3 FlipSolver3 dam break (393,216 particles,
    closed box, gravity) for 60 frames of 1/60 s, resident on the GPU, against
    the reference's own run (tests/golden/flip_dam_break_64.npz, pressure
    solved to an absolute 1e-10). The GPU solves every system to a relative
    true residual of 1e-6; every other stage is bit-exact. Compared: the
    pressure after frames 1, 10, 30 and 60 (relative L2) and the final
    positions of every 16th particle (RMS and maximum distance). After the
    splash the flow is chaotic, so the later bounds follow the reference's
    own spread: the reference run again at a tolerance of 1e-6 differs from
    the fixture by the amounts quoted beside the bounds."""
    g = golden("flip_dam_break_64.npz")
    n = 64
    h = 1.0 / n
    ps = jetgpu.FdmMgpcgSolver3(200, 5, 2, 2, 5, 2, 1e-6, 1.2, True)
    sim = jetgpu.FlipSolver3((n, n, n), h, (0, 0, 0), pressureSolver=ps)
    pos, _ = scenes.dam_break_particles(n, (0.25, 0.75, 1.0), seed=0)
    sim.setParticles(pos)
    frames = [int(f) for f in g["frames"]]
    rel = {}
    for f in range(1, 61):
        sim.update(1.0 / 60)
        if f in frames:
            p = sim.pressure()
            want = g["pressure"][frames.index(f)].astype(np.float64)
            rel[f] = float(np.linalg.norm(p - want) / np.linalg.norm(want))
    stride = int(g["stride"])
    allpos = sim.positions()
    got = allpos[::stride]
    d = np.linalg.norm(got - g["pos"], axis=1)
    rms, dmax = float(np.sqrt(np.mean(d * d))), float(d.max())
    dmean = np.abs(allpos.mean(axis=0) - g["pos_mean"]).max()
    dstd = np.abs(allpos.std(axis=0) - g["pos_std"]).max()
    print({"pressure_rel_l2": rel, "pos_rms": rms, "pos_max": dmax,
           "cloud_mean": float(dmean), "cloud_std": float(dstd),
           "substeps": sim.subSteps})
    ps.close()
    assert allpos.shape[0] == int(g["count"])
    for f, bound in DAM64_P_REL.items():
        assert rel[f] < bound, (f, rel[f])
    assert rms < DAM64_POS_RMS, rms
    assert dmean < DAM64_CLOUD and dstd < DAM64_CLOUD, (dmean, dstd)
