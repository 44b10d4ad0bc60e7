"""GPU blocked pressure solver (GridSinglePhasePressureSolver3 with MGPCG)
against the reference (golden fixtures) and the oracle port, through the C
ABI.

Bars: cell markers of every level, the level-0 FP64 matrix and rhs are
bit-exact; FP32 coarse rows equal the FP32 rounding of the reference's rows;
pressure within 1e-5 relative L2 of the tightly-solved reference and true
relative residual <= the 1e-6 tolerance; the reference's own known-answer
scenes meet its 1e-6 expectations.
"""
import numpy as np
import pytest
import torch

import jetgpu
import oracle
from conftest import golden
from jetgpu import scenes
from test_oracle import BLOCKED_KATS, blocked_kat_case, check_blocked_kat

pytestmark = pytest.mark.gpu

KMAX = jetgpu.kMaxD
TOL = 1e-6
P_REL_L2 = 1e-5


def field(data, res, h):
    if np.isscalar(data):
        return data
    return jetgpu.CellCenteredScalarGrid3(res, h, (0, 0, 0), data)


def solve(res, h, u, v, w, bsdf, fsdf, precision="fp32", levels=5, tol=TOL):
    solver = jetgpu.FdmMgpcgSolver3(200, levels, 2, 2, 10, 2, tol, 1.0, True,
                                    precision=precision)
    ps = jetgpu.GridSinglePhasePressureSolver3(solver)
    vel = jetgpu.FaceCenteredGrid3(res, h, (0, 0, 0), u.copy(), v.copy(),
                                   w.copy())
    out = vel.clone()
    st = ps.solve(vel, 1.0 / 60.0, out, field(bsdf, res, h), None,
                  field(fsdf, res, h))
    return ps, out, st


def rel_l2(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def check_levels(ps, g):
    for l in range(int(g["levels"])):
        fluid = ps.level(l, "fluid") < 0
        assert np.array_equal(fluid, g[f"L{l}_markers"].reshape(-1) == 0), l
        A = ps.level(l, "A")
        ref = g[f"L{l}_A"].reshape(-1)
        if l == 0:
            assert np.array_equal(A, ref), "level-0 FP64 matrix"
        else:
            assert np.array_equal(A, ref.astype(np.float32).astype(np.float64)), l
    assert np.array_equal(ps.level(0, "b"), g["L0_b"].reshape(-1))


@pytest.mark.parametrize("precision", ["fp32", "fp64", "mixed"])
def test_blocked_sphere_union_16(precision):
    g = golden("blocked_sphere_union_16.npz")
    n, h = 16, (1 / 16,) * 3
    ps, out, st = solve((n,) * 3, h, g["u"], g["v"], g["w"], g["boundary_sdf"],
                        g["fluid_sdf"], precision, levels=int(g["params"][1]))
    assert st == 0
    check_levels(ps, g)
    assert ps.last_stats.relative_residual <= TOL
    assert rel_l2(ps.pressure(), g["p"]) < P_REL_L2
    for k in "uvw":
        assert np.abs(getattr(out, k) - g["out_" + k]).max() < 1e-4


def test_blocked_noncubic():
    g = golden("blocked_noncubic_12x8x16.npz")
    res, h = (12, 8, 16), tuple(g["spacing"])
    ps, out, st = solve(res, h, g["u"], g["v"], g["w"], g["boundary_sdf"],
                        g["fluid_sdf"], levels=int(g["params"][1]))
    assert st == 0
    check_levels(ps, g)
    assert rel_l2(ps.pressure(), g["p"]) < P_REL_L2
    for k in "uvw":
        assert np.abs(getattr(out, k) - g["out_" + k]).max() < 1e-4


@pytest.mark.parametrize("kind", BLOCKED_KATS)
def test_blocked_known_answers(kind):
    u, v, w, bs, fs = blocked_kat_case(kind)
    ps, out, st = solve((3, 3, 3), (1.0,) * 3, u, v, w, bs, fs, "fp64",
                        tol=1e-10)
    check_blocked_kat(kind, out.u, out.v, out.w, ps.pressure())


@pytest.mark.parametrize("n,precision", [(64, "fp32"), (64, "mixed")])
def test_blocked_vs_port(n, precision):
    sc = scenes.sphere_union_scene(n, seed=5)
    h = (1.0 / n,) * 3
    ps, out, st = solve((n,) * 3, h, sc["u"], sc["v"], sc["w"],
                        sc["boundary_sdf"], sc["fluid_sdf"], precision)
    assert st == 0
    assert ps.last_stats.relative_residual <= TOL
    ref = oracle.port().blocked_pressure_solve(
        (n,) * 3, h, (0, 0, 0), sc["u"], sc["v"], sc["w"], sc["boundary_sdf"],
        sc["fluid_sdf"], oracle.MgParams(300, 5, 5, 5, 20, 20, 1e-12, 1.5,
                                         True))
    assert rel_l2(ps.pressure(), ref["p"]) < P_REL_L2
    for k in "uvw":
        assert np.abs(getattr(out, k) - ref[k]).max() < 1e-3


def test_blocked_device_matches_host():
    """The device-pointer entry gives the host entry's result bit for bit."""
    n = 48
    sc = scenes.sphere_union_scene(n, seed=6)
    h = (1.0 / n,) * 3
    ps, out, st = solve((n,) * 3, h, sc["u"], sc["v"], sc["w"],
                        sc["boundary_sdf"], sc["fluid_sdf"])
    solver = ps.linearSystemSolver
    dev = torch.device("cuda", 0)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    du, dv, dw = T(sc["u"]), T(sc["v"]), T(sc["w"])
    ou, ov, ow = du.clone(), dv.clone(), dw.clone()
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
    p = torch.zeros((n, n, n), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    st2 = jetgpu.solve_pressure_blocked_device(solver, g, du, dv, dw, B, F, ou,
                                               ov, ow, p)
    assert st2 == st == 0
    assert np.array_equal(p.cpu().numpy(), ps.pressure())
    for a, b in ((ou, out.u), (ov, out.v), (ow, out.w)):
        assert np.array_equal(a.cpu().numpy(), b)
