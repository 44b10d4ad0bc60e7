"""Accuracy at the sizes the headline metric is quoted on (GPU, C ABI).

Two workloads:

* the standalone 128^3 solve (16 liquid spheres, solid sphere r = .15 at
  (.5,.3,.5), i.i.d. U[-1,1] face velocities, seed 1) in FP32, FP64 and the
  mixed BF16 V-cycle, against the reference algorithm (the oracle port)
  solved as far as its own MGPCG goes (relative true residual ~1e-8);
* the 256^3 FLIP dam-break sub-step with the static sphere (the bench
  workload). The reference's MGPCG breaks down there before 1e-6, so the FP64
  answer it is held to is the GPU's FP64 mode solved to a relative residual
  below 1e-12, whose residual is recomputed on the CPU with the reference's
  FdmBlas3::residual (src/jet/fdm_linear_system3.cpp:98-116) over the
  reference's own level-0 rows, which the port builds and the GPU's must
  equal bit for bit.

Reported and bounded per precision: the relative L2 of pressure, and the
maximum of FaceCenteredGrid3::divergenceAtCellCenter
(src/jet/face_centered_grid3.cpp:137-151) over fluid cells after
projection, next to the same maximum of the FP64 answer and their largest
cell-wise difference. (With fractional face weights the plain divergence of
a projected field is not zero at cells next to a solid: the system enforces
the weighted divergence; so the check is the divergence's agreement with the
FP64 answer.)
"""
import numpy as np
import pytest

import jetgpu
import oracle
from jetgpu import scenes

pytestmark = pytest.mark.gpu

TOL = 1e-6         # relative true residual every variant reaches
P_REL_L2 = 1e-5    # pressure vs the FP64 answer
DIV_REL = 1e-4     # max |div - div_FP64| over fluid cells, relative to the
                   # input velocity's max |div| there


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def solve(n, sc, precision, tol, levels, iters=300):
    h = (1.0 / n,) * 3
    s = jetgpu.FdmMgpcgSolver3(iters, levels, 2, 2, 5, 2, tol, 1.2, True,
                               precision=precision, maxRefinements=20)
    ps = jetgpu.GridFractionalSinglePhasePressureSolver3(s)
    vel = jetgpu.FaceCenteredGrid3((n,) * 3, h, (0, 0, 0), sc["u"].copy(),
                                   sc["v"].copy(), sc["w"].copy())
    out = vel.clone()
    g = lambda d: jetgpu.CellCenteredScalarGrid3((n,) * 3, h, (0, 0, 0), d)
    st = ps.solve(vel, 1 / 60, out, g(sc["boundary_sdf"]), None,
                  g(sc["fluid_sdf"]))
    return ps, out, st


def divergence(o, n):
    return oracle.divergence_at_cell_center(o.u, o.v, o.w, (1.0 / n,) * 3)


def port_residual(port, A, x, b):
    r = port.residual(A, x, b)
    return float(np.linalg.norm(r) / np.linalg.norm(b))


class Fp64Answer:
    """The GPU's FP64 solve to < 1e-12, rechecked on the CPU."""

    def __init__(self, port, n, sc, levels):
        ps, out, st = solve(n, sc, "fp64", 1e-12, levels)
        assert st == 0
        self.p = ps.pressure().copy()
        self.A = ps.level(0, "A").reshape(n, n, n, 4)
        self.b = ps.level(0, "b").reshape(n, n, n)
        self.fluid = ps.level(0, "fluid").reshape(n, n, n) < 0
        self.div = divergence(out, n)
        self.rel_res = port_residual(port, self.A, self.p, self.b)
        vin = jetgpu.FaceCenteredGrid3((n,) * 3, (1.0 / n,) * 3, (0, 0, 0),
                                       sc["u"], sc["v"], sc["w"])
        self.div_in = float(np.abs(divergence(vin, n)[self.fluid]).max())
        ps.linearSystemSolver.close()


def check_variant(n, sc, precision, levels, ans, ref_p=None):
    ps, out, st = solve(n, sc, precision, TOL, levels)
    assert st == 0
    stats = ps.last_stats
    assert stats.relative_residual <= TOL
    p = ps.pressure()
    d = divergence(out, n)
    rep = dict(precision=precision, iterations=stats.iterations,
               relative_residual=stats.relative_residual,
               p_rel_l2=rel_l2(p, ans.p),
               max_div=float(np.abs(d[ans.fluid]).max()),
               max_div_fp64=float(np.abs(ans.div[ans.fluid]).max()),
               max_div_diff=float(np.abs(d - ans.div)[ans.fluid].max()))
    if ref_p is not None:
        rep["p_rel_l2_reference"] = rel_l2(p, ref_p)
    print(rep)
    assert rep["p_rel_l2"] < P_REL_L2, rep
    if ref_p is not None:
        assert rep["p_rel_l2_reference"] < P_REL_L2, rep
    assert rep["max_div_diff"] <= DIV_REL * ans.div_in, rep
    return ps


# ---- 128^3 standalone solve (sphere union, seed 1) ---------------------

N2 = 128
LEVELS2 = 5


@pytest.fixture(scope="module")
def config2(port):
    sc = scenes.sphere_union_scene(N2, seed=1)
    h = (1.0 / N2,) * 3
    ref = port.pressure_solve((N2,) * 3, h, (0, 0, 0), sc["u"], sc["v"],
                              sc["w"], sc["boundary_sdf"], sc["fluid_sdf"],
                              oracle.MgParams(400, LEVELS2, 3, 3, 20, 20,
                                              1e-13, 1.5, True))
    levels = []
    for l in range(port.level_count()):
        levels.append({w: port.level(l, w, (N2,) * 3)
                       for w in ("fluid", "uw", "vw", "ww", "A")})
    b0 = port.level(0, "b", (N2,) * 3)
    ref_rel = port_residual(port, levels[0]["A"], ref["p"], b0)
    ans = Fp64Answer(port, N2, sc, LEVELS2)
    return dict(sc=sc, ref=ref, levels=levels, b0=b0, ref_rel=ref_rel,
                ans=ans)


def test_config2_fp64_answer_pinned(config2):
    ans = config2["ans"]
    # The GPU's FP64 answer has a true residual far below the tolerance,
    # measured by the reference's residual on the reference's rows.
    assert ans.rel_res < 1e-11, ans.rel_res
    assert np.array_equal(ans.A.reshape(-1),
                          config2["levels"][0]["A"].reshape(-1))
    # The reference's own MGPCG gets to ~1e-8 here; the two answers agree
    # to well inside the 1e-5 bar.
    assert config2["ref_rel"] < 1e-7, config2["ref_rel"]
    assert rel_l2(ans.p, config2["ref"]["p"]) < 1e-6


@pytest.mark.parametrize("precision", ["fp32", "fp64", "mixed"])
def test_config2_sphere_union_128(config2, precision):
    ps = check_variant(N2, config2["sc"], precision, LEVELS2, config2["ans"],
                       config2["ref"]["p"])
    # Cell classification and face weights of every level, and the level-0
    # FP64 rows and rhs, bit for bit; coarse rows are the FP32 rounding of
    # the reference's.
    for l, ref in enumerate(config2["levels"]):
        for what in ("fluid", "uw", "vw", "ww"):
            assert np.array_equal(ps.level(l, what), ref[what].reshape(-1)), \
                (l, what)
        A = ps.level(l, "A")
        want = ref["A"].reshape(-1)
        if l == 0:
            assert np.array_equal(A, want)
        else:
            assert np.array_equal(A, want.astype(np.float32).astype(np.float64)), l
    assert np.array_equal(ps.level(0, "b"), config2["b0"].reshape(-1))
    ps.linearSystemSolver.close()


# ---- 256^3 headline sub-step ------------------------------------------

N3 = 256
LEVELS3 = 6


@pytest.fixture(scope="module")
def headline(port):
    sc = scenes.flip_first_substep(N3, box_hi=(0.3, 0.8, 1.0),
                                   sphere=((0.6, 0.2, 0.5), 0.15))
    # The reference's weights and system (one MGPCG iteration: only the
    # level-0 rows and rhs are used).
    port.pressure_solve((N3,) * 3, (1.0 / N3,) * 3, (0, 0, 0), sc["u"],
                        sc["v"], sc["w"], sc["boundary_sdf"], sc["fluid_sdf"],
                        oracle.MgParams(1, 5, 1, 1, 1, 1, 1e-6, 1.5, True))
    A0 = port.level(0, "A", (N3,) * 3)
    b0 = port.level(0, "b", (N3,) * 3)
    ans = Fp64Answer(port, N3, sc, LEVELS3)
    return dict(sc=sc, A0=A0, b0=b0, ans=ans)


def test_headline_rows_and_fp64_answer(headline):
    ans = headline["ans"]
    assert np.array_equal(ans.A.reshape(-1), headline["A0"].reshape(-1))
    assert np.array_equal(ans.b.reshape(-1), headline["b0"].reshape(-1))
    assert ans.rel_res < 1e-11, ans.rel_res


@pytest.mark.parametrize("precision", ["fp32", "mixed"])
def test_headline_256(headline, precision):
    ps = check_variant(N3, headline["sc"], precision, LEVELS3,
                       headline["ans"])
    ps.linearSystemSolver.close()
