"""Pins the oracle port to the reference (CPU only).

The port (oracle/port/jet_port.cpp) must reproduce the reference's outputs bit
for bit: against the committed golden fixtures everywhere, and against the
reference compiled from its own sources where those sources exist.
"""
import numpy as np
import pytest

import oracle
from conftest import golden
from jetgpu import scenes

KMAX = float(np.finfo(np.float64).max)


def params_from(arr):
    a = list(arr)
    return oracle.MgParams(int(a[0]), int(a[1]), int(a[2]), int(a[3]),
                           int(a[4]), int(a[5]), float(a[6]), float(a[7]),
                           bool(a[8]))


def check_pressure_case(o, g, res, h, bsdf, fsdf, solid=(None, None, None)):
    out = o.pressure_solve(res, h, (0, 0, 0), g["u"], g["v"], g["w"], bsdf,
                           fsdf, params_from(g["params"]), solid=solid)
    assert out["iters"] == int(g["iters"])
    for k in ("u", "v", "w"):
        assert np.array_equal(out[k], g["out_" + k]), k
    assert np.array_equal(out["p"], g["p"])
    assert o.level_count() == int(g["levels"])
    for l in range(int(g["levels"])):
        for what in ("fluid", "uw", "vw", "ww", "A"):
            assert np.array_equal(o.level(l, what, res), g[f"L{l}_{what}"]), \
                (l, what)
    assert np.array_equal(o.level(0, "b", res), g["L0_b"])


def test_known_answer_free_surface(port):
    """grid_fractional_single_phase_pressure_solver3_tests.cpp:17-74."""
    g = golden("kat_free_surface_3.npz")
    check_pressure_case(port, g, (3, 3, 3), (1.0, 1.0, 1.0), KMAX,
                        g["fluid_sdf"])
    p = g["p"]
    for j in range(2):
        assert np.allclose(p[:, j, :], 1.5 - j, atol=1e-6)
    for k in ("out_u", "out_v", "out_w"):
        assert np.abs(g[k]).max() < 1e-6


def test_sphere_union_bit_exact(port):
    g = golden("sphere_union_16.npz")
    h = 1.0 / 16
    check_pressure_case(port, g, (16, 16, 16), (h, h, h), g["boundary_sdf"],
                        g["fluid_sdf"])


def test_noncubic_moving_solid_bit_exact(port):
    g = golden("noncubic_12x8x16.npz")
    check_pressure_case(port, g, (12, 8, 16), tuple(g["spacing"]),
                        g["boundary_sdf"], g["fluid_sdf"],
                        solid=(g["solid_u"], g["solid_v"], g["solid_w"]))


def test_mgpcg_poisson(port):
    """fdm_mgpcg_solver3_tests.cpp:13-60: converges (returns true)."""
    g = golden("mgpcg_poisson_32.npz")
    A = [g[f"A{l}"] for l in range(4)]
    b = [g[f"b{l}"] for l in range(4)]
    r = port.mgpcg_system(A, b, params_from(g["params"]))
    assert r["ok"] and bool(g["ok"])
    assert r["iters"] == int(g["iters"])
    assert np.array_equal(r["x"], g["x"])
    rt = port.mgpcg_system(A, b, params_from(g["params_tight"]))
    assert np.array_equal(rt["x"], g["x_tight"])


def test_transfers_bit_exact(port):
    g = golden("transfer_16.npz")
    n, h = 16, 1.0 / 16
    grids, marks, snaps = port.p2g((n, n, n), (h, h, h), (0, 0, 0), g["pos"],
                                   g["vel"])
    for a, k in enumerate("uvw"):
        assert np.array_equal(grids[a], g[k])
        assert np.array_equal(marks[a], g["m" + k])
        assert np.array_equal(snaps[a], g["s" + k])
    new = [g["new_u"], g["new_v"], g["new_w"]]
    v, d = port.g2p_flip((n, n, n), (h, h, h), (0, 0, 0), g["pos"], g["vel"],
                         new, snaps, 0.0)
    assert np.array_equal(v, g["vel_flip"])
    for a, k in enumerate("uvw"):
        assert np.array_equal(d[a], g["d" + k])
    v, _ = port.g2p_flip((n, n, n), (h, h, h), (0, 0, 0), g["pos"], g["vel"],
                         new, snaps, 0.25)
    assert np.array_equal(v, g["vel_blend"])
    v = port.g2p_pic((n, n, n), (h, h, h), (0, 0, 0), g["pos"], g["vel"], new)
    assert np.array_equal(v, g["vel_pic"])


def test_red_black_relax_decreases_residual(port):
    """fdm_gauss_seidel_solver3_tests.cpp:66-85 on the test-helper system."""
    from make_systems import helper_system
    A, b = helper_system(32)
    x = np.zeros_like(b)
    r0 = np.linalg.norm(port.residual(A, x, b))
    for it in range(40):
        x = port.relax(A, b, x, 1.0, True, 1)
        r = np.linalg.norm(port.residual(A, x, b))
        if it > 0:
            assert r < r0
        r0 = r


def test_restrict_correct_transpose(port):
    """Restriction is 1/8 of the prolongation's transpose (boundaries too),
    which the GPU's symmetric V-cycle relies on."""
    rng = np.random.default_rng(0)
    f = rng.standard_normal((8, 8, 8))
    c = rng.standard_normal((4, 4, 4))
    Rf = port.mg_restrict(f)
    Pc = port.mg_correct(c, np.zeros((8, 8, 8)))
    assert abs(np.sum(Rf * c) - np.sum(f * Pc) / 8.0) < 1e-12


def test_rng_streams_match_cpp():
    g = golden("rng_streams.npz")
    for s in range(3):
        ours = scenes.Mt19937Uniform(s).canonical(64)
        assert np.array_equal(ours, g[f"seed{s}"])


def test_dam_break_particle_counts():
    pos, vel = scenes.dam_break_particles(64, (0.25, 0.75, 1.0), seed=0)
    assert pos.shape == (393216, 3)
    assert pos.min() >= 0 and pos[:, 0].max() < 0.25 + 1e-12
    # 256^3 box [0,.3]x[0,.8]x[0,1]: cells whose centre is inside.
    c = (np.arange(256) + 0.5) / 256
    counts = [int(np.count_nonzero(c < b)) for b in (0.3, 0.8, 1.0)]
    assert counts == [77, 205, 256]


def test_port_matches_reference_random(port, reference):
    """Fresh random scenes through both libraries (needs the reference)."""
    rng = np.random.default_rng(11)
    for n, levels in ((20, 3), (24, 4)):
        h = 1.0 / n
        X, Y, Z = scenes.cell_centres(n)
        fl = np.minimum(Y - rng.uniform(0.3, 0.7),
                        np.sqrt((X - .5) ** 2 + (Y - .5) ** 2 + (Z - .5) ** 2) - .2)
        bs = np.sqrt((X - .3) ** 2 + (Y - .2) ** 2 + (Z - .6) ** 2) - .18
        u = rng.uniform(-1, 1, (n, n, n + 1))
        v = rng.uniform(-1, 1, (n, n + 1, n))
        w = rng.uniform(-1, 1, (n + 1, n, n))
        p = oracle.MgParams(100, levels, 3, 3, 10, 10, 1e-9, 1.5, True)
        a = port.pressure_solve((n, n, n), (h, h, h), (0, 0, 0), u, v, w, bs,
                                fl, p)
        b = reference.pressure_solve((n, n, n), (h, h, h), (0, 0, 0), u, v, w,
                                     bs, fl, p)
        for k in ("u", "v", "w", "p"):
            assert np.array_equal(a[k], b[k]), k
        assert a["iters"] == b["iters"]


def _boundary_golden():
    g = golden("boundary_20x16x12.npz")
    res = tuple(int(x) for x in g["res"])
    m = g["moving"]
    moving = dict(lin=tuple(m[:3]), ang=tuple(m[3:6]), centre=tuple(g["centre"]),
                  friction=float(m[6]))
    still = dict(lin=(0, 0, 0), ang=(0, 0, 0), centre=tuple(g["centre"]),
                 friction=0.0)
    cases = [("a", g["sdf"], moving, 63, 5), ("b", g["sdf"], still, 41, 3),
             ("c", KMAX, None, 63, 5)]
    return g, res, tuple(g["h"]), tuple(g["origin"]), cases


def test_constrain_velocity_bit_exact(port):
    """GridFractionalBoundaryConditionSolver3::constrainVelocity
    (grid_fractional_boundary_condition_solver3.cpp:26-233): moving rotating
    collider with friction, partly closed walls, no collider."""
    g, res, h, org, cases = _boundary_golden()
    for tag, sdf, col, closed, depth in cases:
        out = port.constrain_velocity(res, h, org, g["u"], g["v"], g["w"], sdf,
                                      col, closed, depth)
        for a, k in enumerate("uvw"):
            assert np.array_equal(out[a], g[f"{tag}_{k}"]), (tag, k)


def test_constrain_velocity_blocked_bit_exact(port):
    """GridBlockedBoundaryConditionSolver3::constrainVelocity
    (grid_blocked_boundary_condition_solver3.cpp:23-67) on the same scenes."""
    g, res, h, org, cases = _boundary_golden()
    gb = golden("boundary_blocked_20x16x12.npz")
    for tag, sdf, col, closed, depth in cases[:2]:
        out = port.constrain_velocity(res, h, org, g["u"], g["v"], g["w"], sdf,
                                      col, closed, depth, blocked=True)
        for a, k in enumerate("uvw"):
            assert np.array_equal(out[a], gb[f"{tag}_{k}"]), (tag, k)


def test_extrapolate_to_region_bit_exact(port):
    """extrapolateToRegion (include/jet/detail/array_utils-inl.h:172-244)."""
    g = golden("boundary_20x16x12.npz")
    out = port.extrapolate(g["ext_in"], g["ext_valid"], 4)
    assert np.array_equal(out, g["ext_out"])


def test_port_boundary_matches_reference_random(port, reference):
    """Fresh random collider scenes through both libraries (needs the
    reference)."""
    rng = np.random.default_rng(23)
    for res, closed, fr in (((16, 16, 16), 63, 0.0), ((24, 16, 20), 45, 0.3),
                            ((12, 20, 8), 0, 0.9)):
        nx, ny, nz = res
        h = 1.0 / max(res)
        sp, org = (h, h, h), (0.1, -0.05, 0.0)
        centre = (org[0] + 0.55 * nx * h, org[1] + 0.45 * ny * h,
                  org[2] + 0.5 * nz * h)
        sdf = reference.sphere_collider_sdf(res, sp, org, centre,
                                            0.3 * min(res) * h)
        u = rng.uniform(-1, 1, (nz, ny, nx + 1))
        v = rng.uniform(-1, 1, (nz, ny + 1, nx))
        w = rng.uniform(-1, 1, (nz + 1, ny, nx))
        col = dict(lin=(0.2, -0.1, 0.05), ang=(0.3, 0.7, -0.4), centre=centre,
                   friction=fr)
        a = reference.constrain_velocity(res, sp, org, u, v, w, sdf, col,
                                         closed, 5)
        b = port.constrain_velocity(res, sp, org, u, v, w, sdf, col, closed, 5)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)
        a = reference.constrain_velocity(res, sp, org, u, v, w, sdf, col,
                                         closed, 5, blocked=True)
        b = port.constrain_velocity(res, sp, org, u, v, w, sdf, col, closed, 5,
                                    blocked=True)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)
        d = rng.standard_normal((nz, ny, nx))
        m = (rng.uniform(size=d.shape) < 0.2).astype(np.int8)
        assert np.array_equal(reference.extrapolate(d, m, 4),
                              port.extrapolate(d, m, 4))


def _particle_cases(g):
    col = dict(lin=(0.3, -0.2, 0.1), ang=(0.5, -1.0, 0.7),
               centre=tuple(g["centre"]), friction=0.5)
    sph = dict(center=(0.01, -0.02, 0.0), radius=0.2, normal_flipped=0,
               orient=g["orient"], inv_orient=g["inv_orient"], quat=g["quat"])
    return [("a", 0.01, 3.0, 45, col, sph),
            ("b", 0.02, 2.0, 63, col, dict(sph, normal_flipped=1, radius=0.3)),
            ("c", 0.01, 5.0, 63, None, None)]


def test_move_particles_bit_exact(port):
    """PicSolver3::moveParticles (pic_solver3.cpp:206-282) with
    Collider3::resolveCollision (collider3.cpp:19-73) against a rotated,
    moving sphere; a normal-flipped sphere; no collider."""
    g = golden("particles_20x12x16.npz")
    res = tuple(int(x) for x in g["res"])
    for tag, dt, cfl, closed, col, sph in _particle_cases(g):
        pos, vel = port.move_particles(res, tuple(g["h"]), tuple(g["origin"]),
                                       g["pos"], g["vel"],
                                       (g["u"], g["v"], g["w"]), dt, cfl,
                                       closed, col, sph)
        assert np.array_equal(pos, g[f"{tag}_pos"]), tag
        assert np.array_equal(vel, g[f"{tag}_vel"]), tag


def test_port_move_particles_matches_reference_random(port, reference):
    rng = np.random.default_rng(31)
    for res, closed, quat, flip in (((16, 16, 16), 63, (1, 0, 0, 0), 0),
                                    ((12, 20, 8), 18, (0.6, 0.3, 0.5, -0.4), 1)):
        nx, ny, nz = res
        h = 1.0 / max(res)
        sp, org = (h, h, h), (0.0, 0.1, 0.0)
        grids = [rng.uniform(-2, 2, (nz, ny, nx + 1)),
                 rng.uniform(-2, 2, (nz, ny + 1, nx)),
                 rng.uniform(-2, 2, (nz + 1, ny, nx))]
        lo = np.array(org)
        hi = lo + h * np.array(res)
        pos = lo + (hi - lo) * rng.uniform(-0.05, 1.05, (2000, 3))
        vel = rng.uniform(-1, 1, (2000, 3))
        q = np.array(quat, float) / np.linalg.norm(quat)
        o, i = reference.quaternion_matrices(q)
        centre = tuple(lo + (hi - lo) * 0.5)
        col = dict(lin=(0.1, 0.2, -0.1), ang=(0.3, 0.1, -0.7), centre=centre,
                   friction=0.3)
        sph = dict(center=(0, 0, 0), radius=0.25, normal_flipped=flip,
                   orient=o, inv_orient=i, quat=q)
        a = reference.move_particles(res, sp, org, pos, vel, grids, 0.015, 4.0,
                                     closed, col, sph)
        b = port.move_particles(res, sp, org, pos, vel, grids, 0.015, 4.0,
                                closed, col, sph)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_particle_sdf_bit_exact(port):
    """PicSolver3::buildSignedDistanceField (pic_solver3.cpp:296-317) and
    extrapolateIntoCollider (grid_fluid_solver3.cpp:423-438)."""
    g = golden("particle_sdf_20x12x16.npz")
    res = tuple(int(x) for x in g["res"])
    h, org = tuple(g["h"]), tuple(g["origin"])
    a = port.build_particle_sdf(res, h, org, g["pos"], g["collider_sdf"], 2.5)
    assert np.array_equal(a, g["a"])
    b = port.build_particle_sdf(res, h, org, g["pos"], KMAX, 5.0)
    assert np.array_equal(b, g["b"])


def test_port_particle_sdf_matches_reference_random(port, reference):
    rng = np.random.default_rng(41)
    for res, h in (((16, 16, 16), (1 / 16,) * 3), ((24, 10, 14), (0.04, 0.07, 0.05))):
        lo = np.zeros(3)
        hi = np.array(h) * np.array(res)
        pos = hi * rng.uniform(-0.1, 1.1, (4000, 3))
        pos[::5] = hi * rng.integers(0, 8, (800, 3)) / 8.0  # on grid lines
        col = reference.sphere_collider_sdf(res, h, (0, 0, 0), tuple(hi * 0.4),
                                            0.2)
        a = reference.build_particle_sdf(res, h, (0, 0, 0), pos, col, 3.0)
        b = port.build_particle_sdf(res, h, (0, 0, 0), pos, col, 3.0)
        assert np.array_equal(a, b)


def test_apic_transfers_bit_exact(port):
    """ApicSolver3::transferFromParticlesToGrids / transferFromGridsToParticles
    (apic_solver3.cpp:26-228)."""
    g = golden("apic_20x12x16.npz")
    res = tuple(int(x) for x in g["res"])
    h, org = tuple(g["h"]), tuple(g["origin"])
    grids, marks = port.apic_p2g(res, h, org, g["pos"], g["vel"], g["affine"])
    for a, k in enumerate("uvw"):
        assert np.array_equal(grids[a], g[k]), k
        assert np.array_equal(marks[a], g["m" + k]), k
    vel, aff = port.apic_g2p(res, h, org, g["pos"], (g["gu"], g["gv"], g["gw"]))
    assert np.array_equal(vel, g["g2p_vel"])
    assert np.array_equal(aff, g["g2p_affine"])


def test_port_apic_matches_reference_random(port, reference):
    rng = np.random.default_rng(37)
    res, h, org = (16, 12, 20), (1 / 16, 1 / 16, 1 / 16), (0.0, 0.1, 0.0)
    nx, ny, nz = res
    lo = np.array(org)
    hi = lo + np.array(h) * np.array(res)
    pos = lo + (hi - lo) * rng.uniform(-0.05, 1.05, (2500, 3))
    vel = rng.uniform(-1, 1, (2500, 3))
    aff = rng.uniform(-3, 3, (2500, 9))
    a, b = (o.apic_p2g(res, h, org, pos, vel, aff) for o in (reference, port))
    for x, y in zip(a[0] + a[1], b[0] + b[1]):
        assert np.array_equal(x, y)
    grids = [rng.uniform(-1, 1, (nz, ny, nx + 1)),
             rng.uniform(-1, 1, (nz, ny + 1, nx)),
             rng.uniform(-1, 1, (nz + 1, ny, nx))]
    a, b = (o.apic_g2p(res, h, org, pos, grids) for o in (reference, port))
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


# ---------------------------------------------------------------------------
# Blocked pressure solver (GridSinglePhasePressureSolver3 + FdmMgpcgSolver3)


def check_blocked_case(o, g, res, h):
    out = o.blocked_pressure_solve(res, h, (0, 0, 0), g["u"], g["v"], g["w"],
                                   g["boundary_sdf"], g["fluid_sdf"],
                                   params_from(g["params"]))
    assert out["iters"] == int(g["iters"])
    for k in ("u", "v", "w"):
        assert np.array_equal(out[k], g["out_" + k]), k
    assert np.array_equal(out["p"], g["p"])
    for l in range(int(g["levels"])):
        assert np.array_equal(o.blocked_level(l, "markers", res),
                              g[f"L{l}_markers"]), l
        assert np.array_equal(o.blocked_level(l, "A", res), g[f"L{l}_A"]), l
    assert np.array_equal(o.blocked_level(0, "b", res), g["L0_b"])


def test_blocked_sphere_union_bit_exact(port):
    g = golden("blocked_sphere_union_16.npz")
    check_blocked_case(port, g, (16, 16, 16), (1.0 / 16,) * 3)


def test_blocked_noncubic_bit_exact(port):
    g = golden("blocked_noncubic_12x8x16.npz")
    check_blocked_case(port, g, (12, 8, 16), tuple(g["spacing"]))


def blocked_kat_case(kind):
    """The scenes of grid_single_phase_pressure_solver3_tests.cpp: a 3^3
    box with v = 1 on the interior y faces, alone (SolveSinglePhase, :14-67),
    with a wall in the right-most column (…WithBoundary, :69-130), with air
    in the top row (SolveFreeSurface, :132-189) or both
    (SolveFreeSurfaceWithBoundary, :250-311)."""
    n = 3
    u = np.zeros((n, n, n + 1))
    v = np.zeros((n, n + 1, n))
    w = np.zeros((n + 1, n, n))
    v[:, 1:3, :] = 1.0
    c = np.arange(n) + 0.5
    bs, fs = KMAX, -KMAX
    if "boundary" in kind:
        bs = np.broadcast_to((2.0 - c)[None, None, :], (n, n, n)).copy()
    if "free_surface" in kind:
        fs = np.broadcast_to((c - 2.0)[None, :, None], (n, n, n)).copy()
    return u, v, w, bs, fs


def check_blocked_kat(kind, out_u, out_v, out_w, p):
    """The reference tests' expectations, with their 1e-6 tolerance."""
    assert np.abs(out_u).max() < 1e-6
    assert np.abs(out_w).max() < 1e-6
    exp_v = np.zeros_like(out_v)
    cols = slice(0, 3)
    if "boundary" in kind:
        exp_v[:, 1:3, 2] = 1.0  # the wall column keeps its velocity
        cols = slice(0, 2)
    assert np.abs(out_v - exp_v).max() < 1e-6
    if "free_surface" in kind:
        for j in range(2):
            assert np.abs(p[:, j, cols] - (2.0 - j)).max() < 1e-6
    else:
        assert np.abs(p[:, 1:, cols] - p[:, :-1, cols] + 1.0).max() < 1e-6


BLOCKED_KATS = ["plain", "boundary", "free_surface", "free_surface_boundary"]


@pytest.mark.parametrize("kind", BLOCKED_KATS)
def test_blocked_known_answers(port, kind):
    u, v, w, bs, fs = blocked_kat_case(kind)
    prm = oracle.MgParams(100, 5, 5, 5, 20, 20, 1e-12, 1.5, True)
    out = port.blocked_pressure_solve((3, 3, 3), (1.0,) * 3, (0, 0, 0), u, v,
                                      w, bs, fs, prm)
    check_blocked_kat(kind, out["u"], out["v"], out["w"], out["p"])


def test_port_blocked_matches_reference_random(port, reference):
    """Fresh random scenes through both libraries (needs the reference)."""
    rng = np.random.default_rng(23)
    for n, levels in ((20, 3), (24, 4)):
        h = 1.0 / n
        X, Y, Z = scenes.cell_centres(n)
        fl = np.minimum(Y - rng.uniform(0.3, 0.7),
                        np.sqrt((X - .5) ** 2 + (Y - .5) ** 2 + (Z - .5) ** 2) - .2)
        bs = np.sqrt((X - .3) ** 2 + (Y - .2) ** 2 + (Z - .6) ** 2) - .18
        u = rng.uniform(-1, 1, (n, n, n + 1))
        v = rng.uniform(-1, 1, (n, n + 1, n))
        w = rng.uniform(-1, 1, (n + 1, n, n))
        p = oracle.MgParams(100, levels, 3, 3, 10, 10, 1e-9, 1.5, True)
        a = port.blocked_pressure_solve((n, n, n), (h, h, h), (0, 0, 0), u, v,
                                        w, bs, fl, p)
        b = reference.blocked_pressure_solve((n, n, n), (h, h, h), (0, 0, 0),
                                             u, v, w, bs, fl, p)
        for k in ("u", "v", "w", "p"):
            assert np.array_equal(a[k], b[k]), k
        assert a["iters"] == b["iters"]
