"""Generates the golden fixtures in tests/golden/ from the Jet reference.

Run in a checkout where the reference sources exist (the harness is compiled
from them by oracle/Makefile.ref):

    python tests/golden/make_golden.py

Every fixture holds inputs and the reference's outputs for one small case:

* kat_free_surface_3.npz — the reference's own known-answer case
  (src/tests/unit_tests/grid_fractional_single_phase_pressure_solver3_tests.cpp:17-74),
  solved with FdmMgpcgSolver3 installed.
* sphere_union_16.npz — 16^3 sphere-union liquid, solid sphere, random face
  velocities (seed 1): weights, fluid SDF and matrix of every level, rhs,
  pressure and projected velocity.
* noncubic_12x8x16.npz — a non-cubic anisotropic grid with a moving solid.
* mgpcg_poisson_32.npz — the 4-level Poisson system of
  src/tests/unit_tests/fdm_mgpcg_solver3_tests.cpp:13-60 and its solution.
* transfer_16.npz — P2G (grids, markers, FLIP snapshot) and G2P (FLIP, FLIP
  with PIC blending, PIC) for 3,000 particles on a 16^3 grid.
* boundary_20x16x12.npz — GridFractionalBoundaryConditionSolver3::
  constrainVelocity on an anisotropic 20x16x12 grid with the reference's own
  sphere-collider SDF: a moving, rotating collider with friction and all
  walls closed; the same inputs with three walls closed, no friction and a
  shallower extrapolation; and no collider at all. Plus extrapolateToRegion
  of a random field from 15% valid cells.
* particles_20x12x16.npz — PicSolver3::moveParticles of 3,000 particles
  (some starting outside the box) through a random face velocity: with a
  rotated, moving sphere collider (friction 0.5, three walls closed,
  maxCfl 3), with a normal-flipped sphere (all walls closed), and with no
  collider (maxCfl 5); plus the Transform3 matrices the reference builds.
* particle_sdf_20x12x16.npz — PicSolver3::buildSignedDistanceField with
  extrapolation into the collider for 3,000 particles on an anisotropic
  grid, with the reference's sphere-collider SDF (maxCfl 2.5) and with no
  collider (maxCfl 5).
* flip_dam_break_24.npz — FlipSolver3 and PicSolver3 (the reference's
  whole step: transfers, SDF, boundary conditions, gravity, pressure with
  FdmMgpcgSolver3 at tolerance 1e-10, advection) for 3 frames of 1/60 s on
  the 64^3 dam break's geometry at 24^3 (water box [0,.25]x[0,.75]x[0,1],
  8 particles per cell from seed 0, closed walls, gravity (0,-9.8,0)).
* flip_sphere_24.npz — FlipSolver3 for 3 frames of the 24^3 dam break (as
  flip_dam_break_24.npz) with a static sphere collider (radius 0.12 at
  (0.3, 0.15, 0.5), friction 0.2) that cuts into the water column: the
  reference's collider SDF on the grid and the final particles.
* flip_dam_break_64.npz — FlipSolver3 on the full-size dam break: 64^3,
  60 frames of the same dam break (393,216 particles), pressure
  to an absolute 1e-10; the pressure after frames 1, 10, 30 and 60
  (float32), every 16th particle's final position and velocity, and the
  mean / standard deviation of all final positions.
* apic_20x12x16.npz — ApicSolver3's transfers for 2,000 particles (some
  outside the box) on an anisotropic grid: P2G with random affine matrices,
  G2P from a random grid; and ApicSolver3 for 3 frames of the 24^3 dam break
  (as flip_dam_break_24.npz).
* rng_streams.npz — the first doubles of std::mt19937(seed) +
  std::uniform_real_distribution<double>(0,1) for seeds 0, 1, 2, produced by
  a C++ program compiled here.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "fluid-engine-dev_gb300"))
sys.path.insert(0, os.path.join(REPO, "tests"))

import oracle  # noqa: E402
from jetgpu import scenes  # noqa: E402
from make_systems import poisson_system  # noqa: E402

KMAX = float(np.finfo(np.float64).max)


def save(name, **arrays):
    np.savez_compressed(os.path.join(HERE, name), **arrays)
    print("wrote", name)


def pressure_case(ref, res, h, fields, params):
    out = ref.pressure_solve(res, h, (0, 0, 0), fields["u"], fields["v"],
                             fields["w"], fields["boundary_sdf"],
                             fields["fluid_sdf"], params,
                             solid=fields.get("solid", (None, None, None)))
    arrays = dict(out_u=out["u"], out_v=out["v"], out_w=out["w"], p=out["p"],
                  iters=np.array(out["iters"]), resid=np.array(out["resid"]))
    for l in range(ref.level_count()):
        for what in ("fluid", "uw", "vw", "ww", "A"):
            arrays[f"L{l}_{what}"] = ref.level(l, what, res)
    arrays["L0_b"] = ref.level(0, "b", res)
    arrays["levels"] = np.array(ref.level_count())
    return arrays


def params_array(p: oracle.MgParams):
    return np.array([p.max_cg_iter, p.max_levels, p.restrict_iter,
                     p.correct_iter, p.coarsest_iter, p.final_iter,
                     p.tolerance, p.sor, float(p.red_black)])


def kat_free_surface(ref):
    n = 3
    u = np.zeros((n, n, n + 1))
    v = np.zeros((n, n + 1, n))
    w = np.zeros((n + 1, n, n))
    v[:, 1:3, :] = 1.0
    ys = np.arange(n) + 0.5
    fluid = np.broadcast_to((ys - 2.0)[None, :, None], (n, n, n)).copy()
    p = oracle.MgParams(100, 5, 5, 5, 20, 20, 1e-12, 1.5, True)
    f = dict(u=u, v=v, w=w, boundary_sdf=KMAX, fluid_sdf=fluid)
    a = pressure_case(ref, (n, n, n), (1.0, 1.0, 1.0), f, p)
    save("kat_free_surface_3.npz", u=u, v=v, w=w, fluid_sdf=fluid,
         params=params_array(p), **a)


def sphere_union(ref):
    n = 16
    h = 1.0 / n
    sc = scenes.sphere_union_scene(n, seed=1)
    p = oracle.MgParams(200, 4, 5, 5, 20, 20, 1e-10, 1.5, True)
    a = pressure_case(ref, (n, n, n), (h, h, h), sc, p)
    save("sphere_union_16.npz", u=sc["u"], v=sc["v"], w=sc["w"],
         fluid_sdf=sc["fluid_sdf"], boundary_sdf=sc["boundary_sdf"],
         params=params_array(p), **a)


def noncubic(ref):
    res = (12, 8, 16)
    h = (1.0 / 12, 0.8 / 8, 1.5 / 16)
    nx, ny, nz = res
    rng = np.random.default_rng(7)
    cz, cy, cx = [(np.arange(m) + 0.5) * hh for m, hh in zip((nz, ny, nx),
                                                              (h[2], h[1], h[0]))]
    Z, Y, X = np.meshgrid(cz, cy, cx, indexing="ij")
    fluid = np.minimum(Y - 0.55, np.sqrt((X - .6) ** 2 + (Y - .6) ** 2 +
                                         (Z - .7) ** 2) - 0.25)
    solid = np.sqrt((X - 0.4) ** 2 + (Y - 0.3) ** 2 + (Z - 0.8) ** 2) - 0.2
    u = rng.uniform(-1, 1, (nz, ny, nx + 1))
    v = rng.uniform(-1, 1, (nz, ny + 1, nx))
    w = rng.uniform(-1, 1, (nz + 1, ny, nx))
    su = rng.uniform(-0.5, 0.5, u.shape)
    sv = rng.uniform(-0.5, 0.5, v.shape)
    sw = rng.uniform(-0.5, 0.5, w.shape)
    p = oracle.MgParams(200, 3, 5, 5, 20, 20, 1e-10, 1.5, True)
    f = dict(u=u, v=v, w=w, boundary_sdf=solid, fluid_sdf=fluid,
             solid=(su, sv, sw))
    a = pressure_case(ref, res, h, f, p)
    save("noncubic_12x8x16.npz", u=u, v=v, w=w, fluid_sdf=fluid,
         boundary_sdf=solid, solid_u=su, solid_v=sv, solid_w=sw,
         spacing=np.array(h), params=params_array(p), **a)


def blocked_case(ref, res, h, fields, params):
    out = ref.blocked_pressure_solve(res, h, (0, 0, 0), fields["u"],
                                     fields["v"], fields["w"],
                                     fields["boundary_sdf"],
                                     fields["fluid_sdf"], params)
    arrays = dict(out_u=out["u"], out_v=out["v"], out_w=out["w"], p=out["p"],
                  iters=np.array(out["iters"]), resid=np.array(out["resid"]))
    levels = 0
    while True:
        try:
            arrays[f"L{levels}_markers"] = ref.blocked_level(levels, "markers",
                                                             res)
        except ValueError:
            break
        arrays[f"L{levels}_A"] = ref.blocked_level(levels, "A", res)
        levels += 1
    arrays["L0_b"] = ref.blocked_level(0, "b", res)
    arrays["levels"] = np.array(levels)
    return arrays


def blocked(ref):
    """GridSinglePhasePressureSolver3 with MGPCG: a sphere-union scene on a
    cubic power-of-two grid and a non-cubic grid with non-power-of-two
    spacing (true divisions in the divergence)."""
    n = 16
    h = 1.0 / n
    sc = scenes.sphere_union_scene(n, seed=4)
    p = oracle.MgParams(200, 4, 5, 5, 20, 20, 1e-10, 1.5, True)
    a = blocked_case(ref, (n, n, n), (h, h, h), sc, p)
    save("blocked_sphere_union_16.npz", u=sc["u"], v=sc["v"], w=sc["w"],
         fluid_sdf=sc["fluid_sdf"], boundary_sdf=sc["boundary_sdf"],
         params=params_array(p), **a)
    res = (12, 8, 16)
    hh = (1.0 / 12, 0.8 / 8, 1.5 / 16)
    nx, ny, nz = res
    rng = np.random.default_rng(9)
    cz, cy, cx = [(np.arange(m) + 0.5) * d for m, d in zip((nz, ny, nx),
                                                           (hh[2], hh[1], hh[0]))]
    Z, Y, X = np.meshgrid(cz, cy, cx, indexing="ij")
    fluid = np.minimum(Y - 0.5, np.sqrt((X - .6) ** 2 + (Y - .6) ** 2 +
                                        (Z - .7) ** 2) - 0.25)
    solid = np.sqrt((X - 0.4) ** 2 + (Y - 0.3) ** 2 + (Z - 0.8) ** 2) - 0.2
    u = rng.uniform(-1, 1, (nz, ny, nx + 1))
    v = rng.uniform(-1, 1, (nz, ny + 1, nx))
    w = rng.uniform(-1, 1, (nz + 1, ny, nx))
    p = oracle.MgParams(200, 3, 5, 5, 20, 20, 1e-10, 1.5, True)
    f = dict(u=u, v=v, w=w, boundary_sdf=solid, fluid_sdf=fluid)
    a = blocked_case(ref, res, hh, f, p)
    save("blocked_noncubic_12x8x16.npz", u=u, v=v, w=w, fluid_sdf=fluid,
         boundary_sdf=solid, spacing=np.array(hh), params=params_array(p), **a)


def mgpcg_poisson(ref):
    A, b = poisson_system()
    p = oracle.MgParams(50, 4, 5, 5, 10, 10, 1e-4, 1.5, False)
    r = ref.mgpcg_system(A, b, p)
    pt = oracle.MgParams(500, 4, 5, 5, 10, 10, 1e-11, 1.5, True)
    rt = ref.mgpcg_system(A, b, pt)
    out = {f"A{l}": a for l, a in enumerate(A)}
    out.update({f"b{l}": x for l, x in enumerate(b)})
    save("mgpcg_poisson_32.npz", x=r["x"], ok=np.array(r["ok"]),
         iters=np.array(r["iters"]), resid=np.array(r["resid"]),
         x_tight=rt["x"], params=params_array(p), params_tight=params_array(pt),
         **out)


def transfers(ref):
    n = 16
    h = 1.0 / n
    rng = np.random.default_rng(3)
    pos = rng.uniform(0.0, 1.0, (3000, 3))
    pos[:8] = [[0, 0, 0], [1, 1, 1], [0.5, 0.5, 0.5], [1e-12, 0.3, 0.99999],
               [1.02, -0.01, 0.5], [0.03125, 0.5, 0.5], [0.0625, 0.5, 1.0],
               [0.999, 0.001, 0.25]]
    vel = rng.uniform(-1.0, 1.0, (3000, 3))
    grids, marks, snaps = ref.p2g((n, n, n), (h, h, h), (0, 0, 0), pos, vel)
    new = [g + rng.uniform(-0.2, 0.2, g.shape) for g in grids]
    vflip, dflip = ref.g2p_flip((n, n, n), (h, h, h), (0, 0, 0), pos, vel, new,
                                snaps, 0.0)
    vblend, _ = ref.g2p_flip((n, n, n), (h, h, h), (0, 0, 0), pos, vel, new,
                             snaps, 0.25)
    vpic = ref.g2p_pic((n, n, n), (h, h, h), (0, 0, 0), pos, vel, new)
    save("transfer_16.npz", pos=pos, vel=vel, u=grids[0], v=grids[1],
         w=grids[2], mu=marks[0], mv=marks[1], mw=marks[2], su=snaps[0],
         sv=snaps[1], sw=snaps[2], new_u=new[0], new_v=new[1], new_w=new[2],
         vel_flip=vflip, du=dflip[0], dv=dflip[1], dw=dflip[2],
         vel_blend=vblend, vel_pic=vpic)


RNG_CPP = r"""
#include <cstdio>
#include <random>
int main() {
  for (unsigned seed = 0; seed < 3; ++seed) {
    std::mt19937 g(seed);
    std::uniform_real_distribution<double> d(0.0, 1.0);
    for (int i = 0; i < 64; ++i) std::printf("%.17g\n", d(g));
  }
}
"""


def boundary(ref):
    res = (20, 16, 12)
    nx, ny, nz = res
    h = (0.05, 0.0625, 0.08)
    org = (0.1, -0.2, 0.05)
    rng = np.random.default_rng(7)
    centre = (org[0] + 0.55 * nx * h[0], org[1] + 0.4 * ny * h[1],
              org[2] + 0.5 * nz * h[2])
    sdf = ref.sphere_collider_sdf(res, h, org, centre, 0.3)
    u = rng.uniform(-1, 1, (nz, ny, nx + 1))
    v = rng.uniform(-1, 1, (nz, ny + 1, nx))
    w = rng.uniform(-1, 1, (nz + 1, ny, nx))
    moving = dict(lin=(0.3, -0.2, 0.1), ang=(0.5, -1.0, 0.7), centre=centre,
                  friction=0.4)
    still = dict(lin=(0, 0, 0), ang=(0, 0, 0), centre=centre, friction=0.0)
    a = ref.constrain_velocity(res, h, org, u, v, w, sdf, moving, 63, 5)
    b = ref.constrain_velocity(res, h, org, u, v, w, sdf, still, 1 + 8 + 32, 3)
    c = ref.constrain_velocity(res, h, org, u, v, w, KMAX, None, 63, 5)
    data = rng.standard_normal((nz, ny, nx))
    valid = (rng.uniform(size=data.shape) < 0.15).astype(np.int8)
    ext = ref.extrapolate(data, valid, 4)
    save("boundary_20x16x12.npz", res=np.array(res), h=np.array(h),
         origin=np.array(org), centre=np.array(centre), sdf=sdf, u=u, v=v, w=w,
         moving=np.array(moving["lin"] + moving["ang"] + (moving["friction"],)),
         a_u=a[0], a_v=a[1], a_w=a[2], b_u=b[0], b_v=b[1], b_w=b[2],
         c_u=c[0], c_v=c[1], c_w=c[2], ext_in=data, ext_valid=valid,
         ext_out=ext)


def boundary_blocked(ref):
    """GridBlockedBoundaryConditionSolver3::constrainVelocity on the scene of
    boundary(): the fractional constraint plus the no-flux pass on the faces
    of collider cells."""
    g = np.load(os.path.join(HERE, "boundary_20x16x12.npz"))
    res = tuple(int(x) for x in g["res"])
    h, org = tuple(g["h"]), tuple(g["origin"])
    m = g["moving"]
    centre = tuple(g["centre"])
    moving = dict(lin=tuple(m[:3]), ang=tuple(m[3:6]), centre=centre,
                  friction=float(m[6]))
    still = dict(lin=(0, 0, 0), ang=(0, 0, 0), centre=centre, friction=0.0)
    a = ref.constrain_velocity(res, h, org, g["u"], g["v"], g["w"], g["sdf"],
                               moving, 63, 5, blocked=True)
    b = ref.constrain_velocity(res, h, org, g["u"], g["v"], g["w"], g["sdf"],
                               still, 1 + 8 + 32, 3, blocked=True)
    save("boundary_blocked_20x16x12.npz", a_u=a[0], a_v=a[1], a_w=a[2],
         b_u=b[0], b_v=b[1], b_w=b[2])


def particles(ref):
    res = (20, 12, 16)
    nx, ny, nz = res
    h = 1.0 / 20
    sp, org = (h, h, h), (0.05, 0.0, -0.1)
    rng = np.random.default_rng(13)
    grids = [rng.uniform(-2, 2, (nz, ny, nx + 1)),
             rng.uniform(-2, 2, (nz, ny + 1, nx)),
             rng.uniform(-2, 2, (nz + 1, ny, nx))]
    lo = np.array(org)
    hi = lo + h * np.array(res)
    pos = lo + (hi - lo) * rng.uniform(-0.05, 1.05, (3000, 3))
    vel = rng.uniform(-1, 1, (3000, 3))
    q = np.array([0.9, 0.1, -0.3, 0.2])
    q /= np.linalg.norm(q)
    o, i = ref.quaternion_matrices(q)
    centre = tuple(lo + (hi - lo) * np.array([0.5, 0.4, 0.55]))
    col = dict(lin=(0.3, -0.2, 0.1), ang=(0.5, -1.0, 0.7), centre=centre,
               friction=0.5)
    sph = dict(center=(0.01, -0.02, 0.0), radius=0.2, normal_flipped=0,
               orient=o, inv_orient=i, quat=q)
    a = ref.move_particles(res, sp, org, pos, vel, grids, 0.01, 3.0, 45, col,
                           sph)
    sphf = dict(sph, normal_flipped=1, radius=0.3)
    b = ref.move_particles(res, sp, org, pos, vel, grids, 0.02, 2.0, 63, col,
                           sphf)
    c = ref.move_particles(res, sp, org, pos, vel, grids, 0.01, 5.0, 63)
    save("particles_20x12x16.npz", res=np.array(res), h=np.array(sp),
         origin=np.array(org), u=grids[0], v=grids[1], w=grids[2], pos=pos,
         vel=vel, quat=q, orient=o, inv_orient=i, centre=np.array(centre),
         a_pos=a[0], a_vel=a[1], b_pos=b[0], b_vel=b[1], c_pos=c[0],
         c_vel=c[1])


def particle_sdf(ref):
    res = (20, 12, 16)
    h = (0.05, 0.0625, 0.055)
    org = (0.1, 0.0, -0.05)
    rng = np.random.default_rng(17)
    lo = np.array(org)
    hi = lo + np.array(h) * np.array(res)
    pos = lo + (hi - lo) * rng.uniform(-0.1, 1.1, (3000, 3))
    col = ref.sphere_collider_sdf(res, h, org, tuple(lo + (hi - lo) * 0.5),
                                  0.25)
    a = ref.build_particle_sdf(res, h, org, pos, col, 2.5)
    b = ref.build_particle_sdf(res, h, org, pos, KMAX, 5.0)
    save("particle_sdf_20x12x16.npz", res=np.array(res), h=np.array(h),
         origin=np.array(org), pos=pos, collider_sdf=col, a=a, b=b)


def flip_dam_break(ref):
    n = 24
    h = 1.0 / n
    pos, vel = scenes.dam_break_particles(n, (0.25, 0.75, 1.0), seed=0)
    p = oracle.MgParams(100, 5, 5, 5, 20, 20, 1e-10, 1.5, True)
    fp, fv = ref.flip_run((n, n, n), (h, h, h), (0, 0, 0), pos, vel, 3,
                          params=p)
    pp, pv = ref.flip_run((n, n, n), (h, h, h), (0, 0, 0), pos, vel, 3,
                          flip=False, params=p)
    save("flip_dam_break_24.npz", flip_pos=fp, flip_vel=fv, pic_pos=pp,
         pic_vel=pv)


def flip_sphere(ref):
    n = 24
    h = 1.0 / n
    pos, vel = scenes.dam_break_particles(n, (0.25, 0.75, 1.0), seed=0)
    p = oracle.MgParams(100, 5, 5, 5, 20, 20, 1e-10, 1.5, True)
    centre, radius, friction = (0.3, 0.15, 0.5), 0.12, 0.2
    sdf = ref.sphere_collider_sdf((n, n, n), (h, h, h), (0, 0, 0), centre,
                                  radius)
    fp, fv = ref.flip_run_sphere((n, n, n), (h, h, h), (0, 0, 0), pos, vel, 3,
                                 centre, radius, friction, params=p)
    save("flip_sphere_24.npz", sdf=sdf, centre=np.array(centre),
         radius=np.array(radius), friction=np.array(friction), flip_pos=fp,
         flip_vel=fv)


# Frames after which the 64^3 dam break's pressure is kept, and the particle
# stride of the kept final positions (the whole set is 393,216 particles).
DAM64_FRAMES = (1, 10, 30, 60)
DAM64_STRIDE = 16


def dam64_pressure(pr):
    """The kept pressure fields in float32, with the values of air cells
    (|p| below 1e-9 of the frame's maximum: what the solve leaves in the
    identity rows) set to zero so that the fixture compresses."""
    out = pr.astype(np.float32)
    for f in range(out.shape[0]):
        small = np.abs(pr[f]) < 1e-9 * np.abs(pr[f]).max()
        out[f][small] = 0.0
    return out


def flip_dam_break_64(ref):
    """The full-size dam break: FlipSolver3, 64^3 over the unit
    cube, the water box [0,.25]x[0,.75]x[0,1] at 8 particles per cell from
    seed 0, gravity (0,-9.8,0), closed walls, maxCfl 5, 60 frames of 1/60 s,
    the pressure solved with FdmMgpcgSolver3 to an absolute 1e-10. Kept: the
    pressure after frames DAM64_FRAMES (float32), every DAM64_STRIDE-th
    particle's final position and velocity, and the mean and standard
    deviation of all final positions."""
    n = 64
    h = 1.0 / n
    pos, vel = scenes.dam_break_particles(n, (0.25, 0.75, 1.0), seed=0)
    p = oracle.MgParams(100, 5, 5, 5, 20, 20, 1e-10, 1.5, True)
    fp, fv, pr = ref.flip_run_record((n, n, n), (h, h, h), (0, 0, 0), pos,
                                     vel, 60, DAM64_FRAMES, params=p)
    save("flip_dam_break_64.npz", frames=np.array(DAM64_FRAMES),
         pressure=dam64_pressure(pr), stride=np.array(DAM64_STRIDE),
         pos=fp[::DAM64_STRIDE], vel=fv[::DAM64_STRIDE],
         pos_mean=fp.mean(axis=0), pos_std=fp.std(axis=0),
         count=np.array(fp.shape[0]))


def apic(ref):
    res = (20, 12, 16)
    nx, ny, nz = res
    h = (0.05, 0.07, 0.06)
    org = (0.1, -0.2, 0.05)
    rng = np.random.default_rng(29)
    lo = np.array(org)
    hi = lo + np.array(h) * np.array(res)
    pos = lo + (hi - lo) * rng.uniform(-0.05, 1.05, (2000, 3))
    vel = rng.uniform(-1, 1, (2000, 3))
    aff = rng.uniform(-2, 2, (2000, 9))
    grids, marks = ref.apic_p2g(res, h, org, pos, vel, aff)
    g2 = [rng.uniform(-1, 1, (nz, ny, nx + 1)), rng.uniform(-1, 1, (nz, ny + 1, nx)),
          rng.uniform(-1, 1, (nz + 1, ny, nx))]
    gv, ga = ref.apic_g2p(res, h, org, pos, g2)
    n = 24
    d0, dv0 = scenes.dam_break_particles(n, (0.25, 0.75, 1.0), seed=0)
    p = oracle.MgParams(100, 5, 5, 5, 20, 20, 1e-10, 1.5, True)
    ap, av = ref.flip_run((n, n, n), (1 / n,) * 3, (0, 0, 0), d0, dv0, 3,
                          flip=2, params=p)
    save("apic_20x12x16.npz", res=np.array(res), h=np.array(h),
         origin=np.array(org), pos=pos, vel=vel, affine=aff, u=grids[0],
         v=grids[1], w=grids[2], mu=marks[0], mv=marks[1], mw=marks[2],
         gu=g2[0], gv=g2[1], gw=g2[2], g2p_vel=gv, g2p_affine=ga,
         dam_pos=ap, dam_vel=av)


def rng_streams():
    with tempfile.TemporaryDirectory() as td:
        src = os.path.join(td, "rng.cpp")
        exe = os.path.join(td, "rng")
        with open(src, "w") as f:
            f.write(RNG_CPP)
        subprocess.run(["g++", "-O2", src, "-o", exe], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True)
    vals = np.array([float(x) for x in out.stdout.split()]).reshape(3, 64)
    save("rng_streams.npz", seed0=vals[0], seed1=vals[1], seed2=vals[2])


def main():
    ref = oracle.reference()
    if ref is None:
        raise SystemExit("the reference harness is required (reference sources "
                         "not found)")
    ref.set_threads(0)
    if len(sys.argv) > 1:  # named cases only
        for name in sys.argv[1:]:
            globals()[name](ref)
        return
    kat_free_surface(ref)
    sphere_union(ref)
    noncubic(ref)
    mgpcg_poisson(ref)
    blocked(ref)
    transfers(ref)
    boundary(ref)
    boundary_blocked(ref)
    particles(ref)
    particle_sdf(ref)
    flip_dam_break(ref)
    flip_dam_break_64(ref)
    apic(ref)
    rng_streams()


if __name__ == "__main__":
    main()
