"""GPU pressure projection against the reference (golden fixtures) and the
oracle port, through the C ABI.

Bars: cell classification, face weights (every level) and the FP64 matrix and
rhs are bit-exact; FP32 coarse rows equal the FP32 rounding of the reference's
rows; pressure within 1e-5 relative L2 of the tightly-solved reference and
true relative residual <= the 1e-6 tolerance.
"""
import numpy as np
import pytest

import jetgpu
import oracle
from conftest import golden
from jetgpu import scenes

pytestmark = pytest.mark.gpu

KMAX = jetgpu.kMaxD
TOL = 1e-6          # relative true residual the solver must reach
P_REL_L2 = 1e-5     # pressure vs FP64 reference


def grid_field(data, res, h):
    return jetgpu.CellCenteredScalarGrid3(res, h, (0, 0, 0), data)


def solve(res, h, u, v, w, bsdf, fsdf, precision="fp32", levels=5, solid=None,
          **kw):
    solver = jetgpu.FdmMgpcgSolver3(200, levels, 2, 2, 10, 2, TOL, 1.0, True,
                                    precision=precision, **kw)
    ps = jetgpu.GridFractionalSinglePhasePressureSolver3(solver)
    vel = jetgpu.FaceCenteredGrid3(res, h, (0, 0, 0), u.copy(), v.copy(),
                                   w.copy())
    out = vel.clone()
    b = bsdf if np.isscalar(bsdf) else grid_field(bsdf, res, h)
    f = fsdf if np.isscalar(fsdf) else grid_field(fsdf, res, h)
    st = ps.solve(vel, 1.0 / 60.0, out, b, solid, f)
    return ps, out, st


def rel_l2(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def check_levels(ps, g, res):
    for l in range(int(g["levels"])):
        for what in ("fluid", "uw", "vw", "ww"):
            got = ps.level(l, what)
            assert np.array_equal(got, g[f"L{l}_{what}"].reshape(-1)), (l, what)
        A = ps.level(l, "A")
        ref = g[f"L{l}_A"].reshape(-1)
        if l == 0:
            assert np.array_equal(A, ref), "level-0 FP64 matrix"
        else:
            assert np.array_equal(A, ref.astype(np.float32).astype(np.float64)), l
    assert np.array_equal(ps.level(0, "b"), g["L0_b"].reshape(-1))


@pytest.mark.parametrize("precision", ["fp32", "fp64", "mixed"])
def test_sphere_union_16(precision):
    g = golden("sphere_union_16.npz")
    n, h = 16, (1 / 16,) * 3
    ps, out, st = solve((n,) * 3, h, g["u"], g["v"], g["w"], g["boundary_sdf"],
                        g["fluid_sdf"], precision, levels=int(g["params"][1]))
    assert st == 0
    check_levels(ps, g, (n,) * 3)
    assert ps.last_stats.relative_residual <= TOL
    assert rel_l2(ps.pressure(), g["p"]) < P_REL_L2
    for k in "uvw":
        assert np.abs(getattr(out, k) - g["out_" + k]).max() < 1e-4


def test_noncubic_moving_solid():
    g = golden("noncubic_12x8x16.npz")
    res, h = (12, 8, 16), tuple(g["spacing"])
    ps, out, st = solve(res, h, g["u"], g["v"], g["w"], g["boundary_sdf"],
                        g["fluid_sdf"], levels=int(g["params"][1]),
                        solid=(g["solid_u"], g["solid_v"], g["solid_w"]))
    assert st == 0
    check_levels(ps, g, res)
    assert rel_l2(ps.pressure(), g["p"]) < P_REL_L2


def test_known_answer_free_surface():
    """grid_fractional_single_phase_pressure_solver3_tests.cpp:17-74."""
    g = golden("kat_free_surface_3.npz")
    ps, out, st = solve((3, 3, 3), (1.0, 1.0, 1.0), g["u"], g["v"], g["w"],
                        KMAX, g["fluid_sdf"])
    assert st == 0
    check_levels(ps, g, (3, 3, 3))
    p = ps.pressure()
    for j in range(2):
        assert np.allclose(p[:, j, :], 1.5 - j, atol=1e-6)
    for k in "uvw":
        assert np.abs(getattr(out, k)).max() < 1e-6


@pytest.mark.parametrize("n,precision", [(32, "fp32"), (64, "fp32"),
                                         (64, "mixed")])
def test_sphere_union_vs_port(port, n, precision):
    h = (1.0 / n,) * 3
    sc = scenes.sphere_union_scene(n, seed=1)
    ref = port.pressure_solve((n,) * 3, h, (0, 0, 0), sc["u"], sc["v"], sc["w"],
                              sc["boundary_sdf"], sc["fluid_sdf"],
                              oracle.MgParams(400, 5, 3, 3, 20, 20, 1e-13, 1.5,
                                              True))
    ps, out, st = solve((n,) * 3, h, sc["u"], sc["v"], sc["w"],
                        sc["boundary_sdf"], sc["fluid_sdf"], precision)
    assert st == 0
    for what in ("fluid", "uw", "vw", "ww"):
        assert np.array_equal(ps.level(0, what),
                              port.level(0, what, (n,) * 3).reshape(-1))
    assert np.array_equal(ps.level(0, "A"), port.level(0, "A", (n,) * 3).reshape(-1))
    assert ps.last_stats.relative_residual <= TOL
    assert rel_l2(ps.pressure(), ref["p"]) < P_REL_L2


@pytest.mark.parametrize("precision", ["fp32", "mixed"])
def test_flip_substep_64_vs_port(port, precision):
    n = 64
    h = (1.0 / n,) * 3
    sc = scenes.flip_first_substep(n, box_hi=(0.25, 0.75, 1.0))
    ref = port.pressure_solve((n,) * 3, h, (0, 0, 0), sc["u"], sc["v"], sc["w"],
                              sc["boundary_sdf"], sc["fluid_sdf"],
                              oracle.MgParams(400, 5, 3, 3, 20, 20, 1e-13, 1.5,
                                              True))
    ps, out, st = solve((n,) * 3, h, sc["u"], sc["v"], sc["w"],
                        sc["boundary_sdf"], sc["fluid_sdf"], precision)
    assert st == 0
    assert ps.last_stats.relative_residual <= TOL
    assert rel_l2(ps.pressure(), ref["p"]) < P_REL_L2
    for k in "uvw":
        assert np.abs(getattr(out, k) - ref[k]).max() < 1e-4


def test_deterministic():
    n = 32
    h = (1.0 / n,) * 3
    sc = scenes.sphere_union_scene(n, seed=1)
    a = solve((n,) * 3, h, sc["u"], sc["v"], sc["w"], sc["boundary_sdf"],
              sc["fluid_sdf"])
    b = solve((n,) * 3, h, sc["u"], sc["v"], sc["w"], sc["boundary_sdf"],
              sc["fluid_sdf"])
    assert np.array_equal(a[0].pressure(), b[0].pressure())
    for k in "uvw":
        assert np.array_equal(getattr(a[1], k), getattr(b[1], k))


def test_no_fluid_leaves_velocity():
    n = 16
    h = (1.0 / n,) * 3
    rng = np.random.default_rng(0)
    u = rng.uniform(-1, 1, (n, n, n + 1))
    v = rng.uniform(-1, 1, (n, n + 1, n))
    w = rng.uniform(-1, 1, (n + 1, n, n))
    ps, out, st = solve((n,) * 3, h, u, v, w, KMAX, 1.0)
    assert st == 0
    assert np.array_equal(ps.pressure(), np.zeros((n, n, n)))
    assert np.array_equal(out.u, u) and np.array_equal(out.v, v)


def test_bad_inputs_rejected():
    solver = jetgpu.FdmMgpcgSolver3()
    ps = jetgpu.GridFractionalSinglePhasePressureSolver3(solver)
    vel = jetgpu.FaceCenteredGrid3((8, 8, 8), (0.0, 0.1, 0.1))
    with pytest.raises(jetgpu.JetGpuError) as e:
        ps.solve(vel, 0.1, vel.clone())
    assert e.value.status == 3


def test_all_fluid_closed_box_smoke_system(port):
    """GridSmokeSolver3's projection (fluidSdf = -kMaxD everywhere,
    grid_fluid_solver3.cpp:313-315): a singular pure-Neumann system in a
    closed box. The pressure is defined up to a constant; with the mean
    removed it must match the reference algorithm (the oracle port solved to
    1e-12) within 1e-5 relative L2, and the true residual must reach 1e-6."""
    n = 48
    h = 1.0 / n
    k, j, i = np.indices((n, n + 1, n))
    x, y, z = (i + .5) * h, j * h, (k + .5) * h
    v = np.where((x - .5) ** 2 + (y - .25) ** 2 + (z - .5) ** 2 < 0.15 ** 2,
                 1.0, 0.0)
    v[:, 0, :] = 0
    v[:, -1, :] = 0
    u = np.zeros((n, n, n + 1))
    w = np.zeros((n + 1, n, n))
    for prec in ("fp32", "mixed", "fp64"):
        s = jetgpu.FdmMgpcgSolver3(200, 5, 2, 2, 10, 2, 1e-6, 1.0, True,
                                   precision=prec)
        ps = jetgpu.GridFractionalSinglePhasePressureSolver3(s)
        vel = jetgpu.FaceCenteredGrid3((n, n, n), (h, h, h), (0, 0, 0), u, v, w)
        st = ps.solve(vel, 1 / 60, vel.clone(), jetgpu.ConstantScalarField3(KMAX),
                      None, jetgpu.ConstantScalarField3(-KMAX))
        assert st == 0, prec
        assert ps.last_stats.relative_residual <= 1e-6, prec
        ref = port.pressure_solve((n, n, n), (h, h, h), (0, 0, 0), u, v, w, KMAX,
                                  -KMAX, oracle.MgParams(300, 5, 5, 5, 20, 20,
                                                         1e-12, 1.5, True))
        p = ps.pressure().reshape(-1)
        q = ref["p"].reshape(-1)
        p, q = p - p.mean(), q - q.mean()
        assert np.linalg.norm(p - q) / np.linalg.norm(q) < 1e-5, prec
        s.close()


def test_constant_fields_build_bit_exact(port):
    """Constant boundary and fluid SDFs (ConstantScalarField3, as
    GridSmokeSolver3 without colliders passes them) on a power-of-two cubic
    grid: the fluid SDF and face weights of every level (filled, not
    sampled), and the level-0 FP64 rows (the interior unit-weight cells'
    centre from the exact shortcut) and rhs equal the reference's bit for
    bit."""
    n = 32
    h = 1.0 / n
    rng = np.random.default_rng(5)
    u = rng.uniform(-1, 1, (n, n, n + 1))
    v = rng.uniform(-1, 1, (n, n + 1, n))
    w = rng.uniform(-1, 1, (n + 1, n, n))
    s = jetgpu.FdmMgpcgSolver3(200, 4, 2, 2, 10, 2, 1e-6, 1.0, True)
    ps = jetgpu.GridFractionalSinglePhasePressureSolver3(s)
    vel = jetgpu.FaceCenteredGrid3((n, n, n), (h, h, h), (0, 0, 0), u, v, w)
    ps.solve(vel, 1 / 60, vel.clone(), jetgpu.ConstantScalarField3(KMAX),
             None, jetgpu.ConstantScalarField3(-KMAX))
    port.pressure_solve((n, n, n), (h, h, h), (0, 0, 0), u, v, w, KMAX, -KMAX,
                        oracle.MgParams(1, 4, 1, 1, 1, 1, 1e-6, 1.5, True))
    for l in range(ps.last_stats.levels):
        for what in ("fluid", "uw", "vw", "ww"):
            assert np.array_equal(ps.level(l, what),
                                  port.level(l, what, (n,) * 3).reshape(-1)), (l, what)
    assert np.array_equal(ps.level(0, "A"), port.level(0, "A", (n,) * 3).reshape(-1))
    assert np.array_equal(ps.level(0, "b"), port.level(0, "b", (n,) * 3).reshape(-1))
    s.close()


def test_gradient_paths_agree():
    """The vectorised gradient (16-byte aligned faces) and the per-cell one
    (output faces at an 8-byte offset) give the same bits."""
    import torch
    n = 64
    h = (1.0 / n,) * 3
    sc = scenes.sphere_union_scene(n, seed=3)
    dev = torch.device("cuda", 0)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    u, v, w = T(sc["u"]), T(sc["v"]), T(sc["w"])
    bs, fs = T(sc["boundary_sdf"]), T(sc["fluid_sdf"])
    g = jetgpu.Grid()
    g.res[:] = (n,) * 3
    g.spacing[:] = h
    g.origin[:] = (0, 0, 0)

    def dfield(t):
        f = jetgpu.ScalarField()
        f.kind = 1
        f.data = t.data_ptr()
        f.res[:] = (n,) * 3
        f.origin[:] = tuple(x / 2 for x in h)
        f.spacing[:] = h
        return f

    B, F = dfield(bs), dfield(fs)
    outs = []
    for shift in (0, 1):
        o = [torch.zeros(a.numel() + 1, dtype=torch.float64, device=dev)
             [shift:shift + a.numel()].view(a.shape) for a in (u, v, w)]
        solver = jetgpu.FdmMgpcgSolver3(200, 5, 2, 2, 10, 2, TOL, 1.0, True)
        torch.cuda.synchronize()
        st = jetgpu.solve_pressure_device(solver, g, u, v, w, B, F, *o)
        assert st == 0
        outs.append([a.cpu().numpy() for a in o])
        solver.close()
    for a, b in zip(*outs):
        assert np.array_equal(a, b)


def rigid_face_velocities(n, h, linear, angular, centre):
    """RigidBodyCollider3::velocityAt (src/jet/rigid_body_collider3.cpp:
    25-28) at every u/v/w face position (origin 0; face data origins
    (0, h/2, h/2), (h/2, 0, h/2), (h/2, h/2, 0)), component a on axis-a
    faces, in double arithmetic."""
    out = []
    for a, shape in enumerate([(n, n, n + 1), (n, n + 1, n), (n + 1, n, n)]):
        k, j, i = np.indices(shape, dtype=np.float64)
        o = [0.5 * h] * 3
        o[a] = 0.0
        p = (o[0] + h * i, o[1] + h * j, o[2] + h * k)
        r = [p[d] - centre[d] for d in range(3)]
        w = angular
        cr = (w[1] * r[2] - r[1] * w[2], w[2] * r[0] - r[2] * w[0],
              w[0] * r[1] - r[0] * w[1])
        out.append(linear[a] + cr[a])
    return out


def test_moving_rigid_collider_on_device(port):
    """jetgpu_solve_pressure_collider evaluates the collider's velocityAt on
    the GPU: the same bits as passing the host-sampled face velocities to
    jetgpu_solve_pressure, and the reference's answer for them."""
    n = 32
    h = 1.0 / n
    sc = scenes.sphere_union_scene(n, seed=2)
    lin, ang, ctr = (0.3, -0.2, 0.1), (0.5, 1.0, -0.7), (0.5, 0.3, 0.5)
    solid = rigid_face_velocities(n, h, lin, ang, ctr)
    ps_a, out_a, st = solve((n,) * 3, (h,) * 3, sc["u"], sc["v"], sc["w"],
                            sc["boundary_sdf"], sc["fluid_sdf"],
                            solid=tuple(solid))
    assert st == 0
    col = jetgpu.Collider.make(linear=lin, angular=ang, centre=ctr)
    ps_b, out_b, st = solve((n,) * 3, (h,) * 3, sc["u"], sc["v"], sc["w"],
                            sc["boundary_sdf"], sc["fluid_sdf"], solid=col)
    assert st == 0
    assert np.array_equal(ps_a.level(0, "b"), ps_b.level(0, "b"))
    assert np.array_equal(ps_a.pressure(), ps_b.pressure())
    for k in "uvw":
        assert np.array_equal(getattr(out_a, k), getattr(out_b, k))
    ref = port.pressure_solve((n,) * 3, (h,) * 3, (0, 0, 0), sc["u"], sc["v"],
                              sc["w"], sc["boundary_sdf"], sc["fluid_sdf"],
                              oracle.MgParams(400, 5, 3, 3, 20, 20, 1e-13, 1.5,
                                              True), solid=tuple(solid))
    assert np.array_equal(ps_b.level(0, "b"), port.level(0, "b", (n,) * 3).reshape(-1))
    assert rel_l2(ps_b.pressure(), ref["p"]) < P_REL_L2
    # A resting collider is a static one.
    still = jetgpu.Collider.make(centre=ctr)
    ps_c, out_c, st = solve((n,) * 3, (h,) * 3, sc["u"], sc["v"], sc["w"],
                            sc["boundary_sdf"], sc["fluid_sdf"], solid=still)
    ps_d, out_d, st2 = solve((n,) * 3, (h,) * 3, sc["u"], sc["v"], sc["w"],
                             sc["boundary_sdf"], sc["fluid_sdf"])
    assert st == 0 and st2 == 0
    assert np.array_equal(ps_c.pressure(), ps_d.pressure())


@pytest.mark.parametrize("precision", ["fp32", "mixed"])
def test_device_loop_matches_host_loop(precision):
    """The FP32 PCG runs as one CUDA graph whose while node ends the loop on
    the device; with the live profile on, the same kernels are launched one
    by one from a host loop that reads the residual after every iteration.
    Both must give the same iterations and the same bits (the V-cycle tail
    of the small levels runs in one CTA on both paths)."""
    n = 64
    h = (1.0 / n,) * 3
    sc = scenes.flip_first_substep(n, box_hi=(0.3, 0.8, 1.0),
                                   sphere=((0.6, 0.2, 0.5), 0.15))
    res = []
    for profile in (False, True):
        s = jetgpu.FdmMgpcgSolver3(200, 6, 2, 2, 5, 2, TOL, 1.2, True,
                                   precision=precision)
        s.profile(profile)
        ps = jetgpu.GridFractionalSinglePhasePressureSolver3(s)
        vel = jetgpu.FaceCenteredGrid3((n,) * 3, h, (0, 0, 0), sc["u"].copy(),
                                       sc["v"].copy(), sc["w"].copy())
        out = vel.clone()
        for _ in range(2):  # the second solve replays the captured graphs
            st = ps.solve(vel, 1 / 60, out, grid_field(sc["boundary_sdf"], (n,) * 3, h),
                          None, grid_field(sc["fluid_sdf"], (n,) * 3, h))
        assert st == 0
        res.append((ps.last_stats.iterations, ps.pressure().copy()))
        s.close()
    assert res[0][0] == res[1][0]
    assert np.array_equal(res[0][1], res[1][1])


@pytest.mark.parametrize("case", ["flip", "wide_fluid", "sphere_union",
                                  "noncubic_solid", "moving_collider",
                                  "no_fluid", "all_fluid"])
def test_fluid_box_io_matches_full_io(case):
    """fluid_box_io moves only the velocity faces around the fluid cells;
    with the output holding the input's values (a clone, as
    GridFluidSolver3::computePressure passes), pressure and output are the
    full-transfer solve's bits, and fewer bytes cross the host link."""
    solid = None
    if case == "flip":
        n = 48
        res, h = (n,) * 3, (1.0 / n,) * 3
        sc = scenes.flip_first_substep(n, box_hi=(0.3, 0.6, 0.8))
        args = (sc["u"], sc["v"], sc["w"], sc["boundary_sdf"], sc["fluid_sdf"])
    elif case == "wide_fluid":  # the box spans x: whole rows each way
        n = 64
        res, h = (n,) * 3, (1.0 / n,) * 3
        sc = scenes.flip_first_substep(n, box_hi=(1.0, 0.5, 0.7))
        args = (sc["u"], sc["v"], sc["w"], sc["boundary_sdf"], sc["fluid_sdf"])
    elif case in ("sphere_union", "moving_collider"):
        n = 32
        res, h = (n,) * 3, (1.0 / n,) * 3
        sc = scenes.sphere_union_scene(n, seed=3)
        args = (sc["u"], sc["v"], sc["w"], sc["boundary_sdf"], sc["fluid_sdf"])
        if case == "moving_collider":  # face velocities made on the device
            solid = jetgpu.Collider.make((0.2, -0.1, 0.05), (0.3, 0.0, -0.4),
                                         (0.5, 0.5, 0.5), 0.0)
    elif case == "noncubic_solid":
        g = golden("noncubic_12x8x16.npz")
        res, h = (12, 8, 16), tuple(g["spacing"])
        args = (g["u"], g["v"], g["w"], g["boundary_sdf"], g["fluid_sdf"])
        solid = (g["solid_u"], g["solid_v"], g["solid_w"])
    else:
        n = 16
        res, h = (n,) * 3, (1.0 / n,) * 3
        rng = np.random.default_rng(5)
        args = (rng.uniform(-1, 1, (n, n, n + 1)),
                rng.uniform(-1, 1, (n, n + 1, n)),
                rng.uniform(-1, 1, (n + 1, n, n)), KMAX,
                1.0 if case == "no_fluid" else -1.0)
    full = solve(res, h, *args, solid=solid)
    box = solve(res, h, *args, solid=solid, fluidBoxIo=True)
    # (The all-fluid closed box with random velocities is a singular
    # system that stops at the iteration cap: both report it alike.)
    assert full[2] == box[2]
    assert np.array_equal(full[0].pressure(), box[0].pressure())
    for k in "uvw":
        assert np.array_equal(getattr(full[1], k), getattr(box[1], k)), k
    fs, bs = full[0].last_stats, box[0].last_stats
    if case in ("flip", "wide_fluid", "sphere_union", "moving_collider",
                "no_fluid"):
        assert bs.h2d_bytes < fs.h2d_bytes and bs.d2h_bytes < fs.d2h_bytes
    else:  # fluid cells span the grid: the box is every face
        assert bs.h2d_bytes == fs.h2d_bytes and bs.d2h_bytes == fs.d2h_bytes
